"""Gradient refinement between HIO / RAAR epochs (no reference counterpart).

``FarFieldLoss`` is a ``torch.autograd.Function`` over the engine's
hand-written loss and adjoint kernels (``spe_loss_grad``): the forward pass
returns the per-individual loss of the masked far field and, up to a size
bound, keeps the adjoint's column-transformed gradient, so that the backward
pass is one row pass (FFT, support, upstream scale); above the bound the
backward pass recomputes the transform and the whole adjoint.  Bulk
arithmetic is FP32;
the per-individual loss sums are FP64.

``refine`` runs Adam on individuals that stay in the engine's population
slots: the optimiser works on a tensor that aliases the engine's device
memory, so refinement and iteration share the data without copies.  By
default each step is fused on the device (``spe_adam_step``: loss, adjoint,
and the Adam update inside the adjoint's last pass); the autograd path
(``fused=False``) runs the same arithmetic through torch.optim.Adam.
"""
from __future__ import annotations

import torch

from . import _lib

LOSSES = {"amplitude": _lib.SPE_LOSS_AMPLITUDE, "poisson": _lib.SPE_LOSS_POISSON}


class _DeviceArray:
    """``__cuda_array_interface__`` of engine memory, for torch.as_tensor."""

    def __init__(self, ptr, shape, typestr, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2, "strides": None}
        self.owner = owner  # keeps the engine alive while the tensor lives


def population_tensors(engine, first, count, device):
    """(density, support) torch tensors aliasing population slots
    [first, first+count) of `engine`: complex64 and int32, (count, n, n).
    They stay valid until the engine's capacity grows."""
    n = engine.n
    d, s = engine.population_arrays(first, count)
    dens = torch.as_tensor(_DeviceArray(d, (count, n, n, 2), "<f4", engine), device=device)
    supp = torch.as_tensor(_DeviceArray(s, (count, n, n), "<i4", engine), device=device)
    return torch.view_as_complex(dens), supp


_LEGACY_DEFAULT_STREAM = 1  # cudaStreamLegacy


def _bind_stream(engine, device):
    """Runs the engine on torch's current stream.  torch's default stream is
    the legacy default stream (handle 0), which the engine would read as
    "its own stream"; it is passed as cudaStreamLegacy instead."""
    h = torch.cuda.current_stream(device).cuda_stream
    engine.set_stream(h if h else _LEGACY_DEFAULT_STREAM)


# gradients up to this size are computed with the loss in the forward pass
# and kept for the backward; larger ones are recomputed there
STORE_GRADIENT_BYTES = 4 << 30


class FarFieldLoss(torch.autograd.Function):
    """loss[k] = sum over known pixels of the far-field loss of
    support[k] * density[k] (see ``spe_loss_grad``).  Gradient with respect
    to `density` only (complex autograd convention).

    With a gradient of at most STORE_GRADIENT_BYTES (or recompute=False) the
    forward pass computes the loss and the adjoint up to its column pass in
    one set of passes (``spe_loss_grad_cols``) and keeps that half-transformed
    gradient; the backward pass is the adjoint's last row pass with the
    upstream scale fused in, in place (``spe_grad_rows``).  Above that size
    (or with recompute=True) nothing is kept: the backward pass recomputes the
    transform and the whole adjoint (``spe_loss_grad``).  Both run the same
    kernels on the same values, so the gradients are bit-identical."""

    @staticmethod
    def forward(ctx, density, support, engine, loss="amplitude", eps=0.0, recompute=None):
        if density.dtype != torch.complex64 or not density.is_cuda:
            raise TypeError("density must be a complex64 CUDA tensor")
        density = density.contiguous()
        support = support.to(torch.int32).contiguous()
        count = density.shape[0]
        _bind_stream(engine, density.device)
        out = torch.empty(count, dtype=torch.float64, device=density.device)
        if recompute is None:
            recompute = density.numel() * density.element_size() > STORE_GRADIENT_BYTES
        ctx.half = None
        if recompute or not ctx.needs_input_grad[0]:
            engine.loss_grad(density.data_ptr(), support.data_ptr(), count, LOSSES[loss], eps, out.data_ptr(), 0, 0)
        else:
            half = torch.empty_like(density)
            engine.loss_grad_cols(density.data_ptr(), support.data_ptr(), count, half.data_ptr(), LOSSES[loss], eps,
                                  out.data_ptr())
            ctx.half = half
        ctx.save_for_backward(density, support)
        ctx.engine, ctx.loss, ctx.eps = engine, loss, eps
        return out

    @staticmethod
    def backward(ctx, grad_out):
        density, support = ctx.saved_tensors
        count = density.shape[0]
        scale = grad_out.to(torch.float32).contiguous()
        _bind_stream(ctx.engine, density.device)
        if ctx.half is not None:
            grad, ctx.half = ctx.half, None
            ctx.engine.grad_rows(grad.data_ptr(), support.data_ptr(), count, grad.data_ptr(), scale.data_ptr())
            return grad, None, None, None, None, None
        grad = torch.empty_like(density)
        ctx.engine.loss_grad(density.data_ptr(), support.data_ptr(), count, LOSSES[ctx.loss], ctx.eps, 0,
                             grad.data_ptr(), scale.data_ptr())
        return grad, None, None, None, None, None


def farfield_loss(density, support, engine, loss="amplitude", eps=0.0, recompute=None):
    return FarFieldLoss.apply(density, support, engine, loss, eps, recompute)


def refine(engine, first, count, steps=50, lr=1e-3, loss="poisson", eps=1e-6, device=None, fused=True,
           betas=(0.9, 0.999), adam_eps=1e-8):
    """Adam on individuals [first, first+count) of `engine`'s population, in
    place: `steps` steps on the summed per-individual loss.  Returns the
    per-step loss sums (on the host at the end).

    fused=True runs each step as three passes on the device (loss, adjoint,
    and the Adam update applied by the adjoint's last pass: spe_adam_step);
    fused=False runs FarFieldLoss through torch autograd and
    torch.optim.Adam -- the same arithmetic, the gradient going through
    memory and the optimiser's own kernels."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    dens, supp = population_tensors(engine, first, count, device)
    history = []
    if fused:
        _bind_stream(engine, device)
        m = torch.zeros_like(dens)
        v = torch.zeros_like(dens)
        losses = torch.empty((steps, count), dtype=torch.float64, device=device)
        for t in range(steps):
            engine.adam_step(dens.data_ptr(), supp.data_ptr(), m.data_ptr(), v.data_ptr(), count, LOSSES[loss], eps,
                             lr, betas[0], betas[1], adam_eps, t + 1, losses[t].data_ptr())
        torch.cuda.synchronize(device)
        return losses.sum(dim=1).tolist()
    param = torch.nn.Parameter(dens)  # shares the engine's memory
    opt = torch.optim.Adam([param], lr=lr, betas=betas, eps=adam_eps)
    for _ in range(steps):
        opt.zero_grad(set_to_none=True)
        total = FarFieldLoss.apply(param, supp, engine, loss, eps).sum()
        total.backward()
        opt.step()
        history.append(total.detach())
    torch.cuda.synchronize(device)
    return [float(h) for h in history]
