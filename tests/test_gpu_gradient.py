"""Gradient refinement: the hand-written far-field loss and adjoint kernels
(spe_loss_grad) behind torch.autograd.Function, against the FP64 oracle,
FP64 finite differences and torch autograd through torch.fft (FP64).

Tolerances (FP32 kernels against FP64): loss 2e-5 relative, gradient 2e-5
relative in norm and 1e-4 of the largest component pointwise; directional
derivatives 1e-4 relative to FP64 central differences."""
import numpy as np
import pytest
import torch

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic
from s_spi_spring_gb300.refine import FarFieldLoss, population_tensors, refine

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda", 0)


def setup(n, P, seed=0):
    I, obj, supp = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.3, photons=1e8,
                                             stop_radius=max(2, n // 64))
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, P, n * 0.32, seed=seed + 1)
    eng = _lib.Engine(n, 0)
    eng.set_amplitudes(A)
    return eng, A, dens, S


def kernel_loss_grad(eng, dens, S, loss, eps, weights=None):
    d = torch.tensor(dens, device=DEV, requires_grad=True)
    s = torch.tensor(S, device=DEV)
    L = FarFieldLoss.apply(d, s, eng, loss, eps)
    w = torch.ones_like(L) if weights is None else torch.tensor(weights, device=DEV, dtype=torch.float64)
    (L * w).sum().backward()
    return L.detach().cpu().numpy(), d.grad.cpu().numpy()


@pytest.mark.parametrize("n", [64, 128, 512, 1024, 1054])
@pytest.mark.parametrize("loss,eps", [("amplitude", 0.0), ("poisson", 1e-3)])
def test_loss_and_gradient_match_fp64_oracle(n, loss, eps):
    P = 3
    eng, A, dens, S = setup(n, P, seed=n)
    weights = np.array([1.0, 0.5, 2.0])
    L, G = kernel_loss_grad(eng, dens, S, loss, eps, weights)
    for k in range(P):
        Lo, Go = o.farfield_loss_grad(dens[k], S[k], A, loss, eps)
        Go = Go * weights[k]
        rl = abs(L[k] - Lo) / abs(Lo)
        rg = np.linalg.norm(G[k] - Go) / np.linalg.norm(Go)
        pw = np.abs(G[k] - Go).max() / np.abs(Go).max()
        print(f"n={n} {loss} item {k}: loss rel {rl:.2e}, grad rel {rg:.2e}, pointwise {pw:.2e}")
        assert rl <= 2e-5 and rg <= 2e-5 and pw <= 1e-4
        assert np.all(G[k][S[k] == 0] == 0)


@pytest.mark.parametrize("loss,eps", [("amplitude", 0.0), ("poisson", 1e-3)])
def test_directional_derivatives_match_fp64_finite_differences(loss, eps):
    n = 64
    eng, A, dens, S = setup(n, 1, seed=9)
    _, G = kernel_loss_grad(eng, dens, S, loss, eps)
    rng = np.random.default_rng(1)
    for _ in range(3):
        dvec = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * (S[0] > 0)
        h = 1e-5
        Lp, _ = o.farfield_loss_grad(dens[0] + h * dvec, S[0], A, loss, eps)
        Lm, _ = o.farfield_loss_grad(dens[0] - h * dvec, S[0], A, loss, eps)
        fd = (Lp - Lm) / (2 * h)
        an = float(np.real(np.vdot(G[0], dvec)))
        assert abs(fd - an) <= 1e-4 * abs(fd)


def test_gradient_matches_torch_autograd_reference():
    n = 64
    eng, A, dens, S = setup(n, 2, seed=4)
    L, G = kernel_loss_grad(eng, dens, S, "poisson", 1e-3)
    r = torch.tensor(dens.astype(np.complex128), requires_grad=True)
    Sm = torch.tensor((S > 0).astype(np.float64))
    At = torch.tensor(A.astype(np.float64))
    F = torch.fft.ifft2(r * Sm) * (n * n)
    m2 = F.abs() ** 2
    known = (At >= 0).expand_as(m2)
    Lt = torch.where(known, m2 - At ** 2 * torch.log(m2 + 1e-3), torch.zeros_like(m2)).sum(dim=(1, 2))
    Lt.sum().backward()
    assert np.allclose(L, Lt.detach().numpy(), rtol=2e-5)
    ref = r.grad.numpy()
    assert np.linalg.norm(G - ref) <= 2e-5 * np.linalg.norm(ref)


def test_refine_in_place_on_population_slots():
    n, P = 128, 4
    eng, A, dens, S = setup(n, P, seed=2)
    eng.upload(0, dens, S)
    eng.hio(0, P, 20, 0.9, 0.0)
    before, _ = eng.download(0, P)
    m0 = eng.evaluate(0, P)
    hist = refine(eng, 0, P, steps=30, lr=2e-4, loss="poisson", eps=1e-6)
    after, _ = eng.download(0, P)
    assert hist[-1] < hist[0]
    assert np.array_equal(after[S == 0], before[S == 0])  # outside the support nothing moves
    assert not np.array_equal(after, before)
    m1 = eng.evaluate(0, P)
    assert all(np.isfinite(m["error"]) for m in m1)
    # the aliasing tensors see the engine's memory
    d, s = population_tensors(eng, 1, 2, DEV)
    assert np.array_equal(d.cpu().numpy(), after[1:3]) and np.array_equal(s.cpu().numpy(), S[1:3])
    print("refine: loss", hist[0], "->", hist[-1], "R-factor", [round(m["error_fourier"], 4) for m in m0], "->",
          [round(m["error_fourier"], 4) for m in m1])


@pytest.mark.parametrize("n", [100, 128, 256, 512, 1024])
@pytest.mark.parametrize("loss", ["amplitude", "poisson"])
def test_fused_adam_matches_autograd_adam(n, loss):
    """The fused refinement step (loss, adjoint and Adam update on the
    device) against FarFieldLoss + torch.optim.Adam: the same loss history
    and densities within FP32 rounding, at compiled sides (staged loss row
    passes from 256) and at a side without a compiled plan (100)."""
    P = 3
    eng_a, A, dens, S = setup(n, P, seed=12)
    eng_b, _, _, _ = setup(n, P, seed=12)
    for e in (eng_a, eng_b):
        e.upload(0, dens, S)
    ha = refine(eng_a, 0, P, steps=12, lr=5e-4, loss=loss, eps=1e-6, fused=True)
    hb = refine(eng_b, 0, P, steps=12, lr=5e-4, loss=loss, eps=1e-6, fused=False)
    assert np.allclose(ha, hb, rtol=1e-5), (ha, hb)
    da, _ = eng_a.download(0, P)
    db, _ = eng_b.download(0, P)
    assert np.linalg.norm(da - db) <= 1e-4 * np.linalg.norm(db)
    assert np.array_equal(da[S == 0], dens[S == 0])
    assert ha[-1] < ha[0]


@pytest.mark.parametrize("n", [100, 128, 512, 2048])
@pytest.mark.parametrize("loss,eps", [("amplitude", 0.0), ("poisson", 1e-3)])
def test_stored_and_recomputed_gradients_are_bit_identical(n, loss, eps):
    """FarFieldLoss keeps the adjoint's column-transformed gradient from the
    forward pass and finishes it in place in the backward pass
    (spe_loss_grad_cols, spe_grad_rows; small sizes), or recomputes the whole
    adjoint there (spe_loss_grad; large sizes): the same bits either way,
    with unit and non-unit upstream gradients, on a side without a compiled
    plan (100), the generic row pass (128, 2048) and the staged row pass
    (512)."""
    P = 3
    eng, A, dens, S = setup(n, P, seed=21)
    s = torch.tensor(S, device=DEV)
    for weights in (None, np.array([1.0, 0.5, 2.0])):
        out = []
        for recompute in (False, True):
            d = torch.tensor(dens, device=DEV, requires_grad=True)
            L = FarFieldLoss.apply(d, s, eng, loss, eps, recompute)
            w = torch.ones_like(L) if weights is None else torch.tensor(weights, device=DEV, dtype=torch.float64)
            (L * w).sum().backward()
            out.append((L.detach().cpu().numpy(), d.grad.cpu().numpy()))
        assert np.array_equal(out[0][0], out[1][0])
        assert np.array_equal(out[0][1].view(np.uint32), out[1][1].view(np.uint32))


def test_split_gradient_out_of_place_and_argument_checks():
    """spe_grad_rows into a separate buffer gives the in-place result and
    spe_loss_grad's; the entry points refuse a null buffer and a buffer that
    is the density."""
    n, P = 256, 2
    eng, A, dens, S = setup(n, P, seed=5)
    d = torch.tensor(dens, device=DEV)
    s = torch.tensor(S, device=DEV)
    scale = torch.tensor([0.75, 3.0], device=DEV)
    half = torch.empty_like(d)
    loss = torch.empty(P, dtype=torch.float64, device=DEV)
    eng.set_stream(torch.cuda.current_stream(DEV).cuda_stream or 1)
    eng.loss_grad_cols(d.data_ptr(), s.data_ptr(), P, half.data_ptr(), 1, 1e-3, loss.data_ptr())
    out = torch.empty_like(d)
    eng.grad_rows(half.data_ptr(), s.data_ptr(), P, out.data_ptr(), scale.data_ptr())
    eng.grad_rows(half.data_ptr(), s.data_ptr(), P, half.data_ptr(), scale.data_ptr())
    full = torch.empty_like(d)
    loss2 = torch.empty(P, dtype=torch.float64, device=DEV)
    eng.loss_grad(d.data_ptr(), s.data_ptr(), P, 1, 1e-3, loss2.data_ptr(), full.data_ptr(), scale.data_ptr())
    torch.cuda.synchronize(DEV)
    assert torch.equal(loss, loss2)
    assert torch.equal(torch.view_as_real(out).view(torch.int32), torch.view_as_real(full).view(torch.int32))
    assert torch.equal(torch.view_as_real(half).view(torch.int32), torch.view_as_real(full).view(torch.int32))
    with pytest.raises(RuntimeError):
        eng.loss_grad_cols(d.data_ptr(), s.data_ptr(), P, 0, 1, 1e-3, 0)
    with pytest.raises(RuntimeError):
        eng.loss_grad_cols(d.data_ptr(), s.data_ptr(), P, d.data_ptr(), 1, 1e-3, 0)
    with pytest.raises(RuntimeError):
        eng.grad_rows(half.data_ptr(), s.data_ptr(), P, 0)
    eng.close()


def test_misaligned_device_arrays_are_refused():
    """The compiled sides stage caller arrays with 16-byte copies: arrays
    that do not start on a 16-byte boundary (here a view one complex64
    element in) are refused on the host before any launch, and the engine
    stays usable; a side without a compiled plan takes them."""
    n, P = 256, 2
    eng, A, dens, S = setup(n, P, seed=6)
    eng.set_stream(torch.cuda.current_stream(DEV).cuda_stream or 1)
    d = torch.tensor(dens, device=DEV)
    s = torch.tensor(S, device=DEV)
    raw = torch.zeros(P * n * n + 1, dtype=torch.complex64, device=DEV)
    odd = raw[1:]  # 8 bytes past a 256-byte boundary
    assert odd.data_ptr() % 16 == 8
    odd_s = torch.zeros(P * n * n + 1, dtype=torch.int32, device=DEV)[1:]
    good = torch.zeros_like(d)
    with pytest.raises(RuntimeError, match="16-byte"):
        eng.loss_grad(odd.data_ptr(), s.data_ptr(), P, 1, 1e-3, 0, good.data_ptr(), 0)
    with pytest.raises(RuntimeError, match="16-byte"):
        eng.loss_grad(d.data_ptr(), odd_s.data_ptr(), P, 1, 1e-3, 0, good.data_ptr(), 0)
    with pytest.raises(RuntimeError, match="16-byte"):
        eng.loss_grad_cols(d.data_ptr(), s.data_ptr(), P, odd.data_ptr(), 1, 1e-3, 0)
    with pytest.raises(RuntimeError, match="16-byte"):
        eng.grad_rows(odd.data_ptr(), s.data_ptr(), P, good.data_ptr())
    with pytest.raises(RuntimeError, match="16-byte"):
        eng.adam_step(d.data_ptr(), s.data_ptr(), odd.data_ptr(), good.data_ptr(), P)
    # the engine is unaffected
    loss = torch.empty(P, dtype=torch.float64, device=DEV)
    eng.loss_grad(d.data_ptr(), s.data_ptr(), P, 1, 1e-3, loss.data_ptr(), good.data_ptr(), 0)
    torch.cuda.synchronize(DEV)
    assert torch.isfinite(loss).all()
    eng.close()
    # side 100 (run-time kernels, plain loads): the same views are accepted
    n = 100
    eng, A, dens, S = setup(n, 1, seed=6)
    eng.set_stream(torch.cuda.current_stream(DEV).cuda_stream or 1)
    raw = torch.zeros(n * n + 1, dtype=torch.complex64, device=DEV)
    raw[1:] = torch.tensor(dens[0].ravel(), device=DEV)
    s = torch.tensor(S[0], device=DEV)
    loss_odd = torch.empty(1, dtype=torch.float64, device=DEV)
    loss_ref = torch.empty(1, dtype=torch.float64, device=DEV)
    eng.loss_grad(raw[1:].data_ptr(), s.data_ptr(), 1, 1, 1e-3, loss_odd.data_ptr(), 0, 0)
    d = torch.tensor(dens[:1], device=DEV)
    eng.loss_grad(d.data_ptr(), s.data_ptr(), 1, 1, 1e-3, loss_ref.data_ptr(), 0, 0)
    torch.cuda.synchronize(DEV)
    assert torch.equal(loss_odd, loss_ref)
    eng.close()
