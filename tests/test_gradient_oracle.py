"""The oracle's far-field loss gradient (gradient refinement) against FP64
finite differences and against torch autograd through torch.fft (FP64, CPU).
No reference counterpart: the reference has no gradient path."""
import numpy as np
import pytest
import torch

from oracle import spring_oracle as o


def case(n=32, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.uniform(0, 30, (n, n))
    A[rng.uniform(size=(n, n)) < 0.1] = -1.0  # unknown pixels
    A[0, 0] = -1.0
    S = np.zeros((n, n), np.int32)
    S[n // 4:3 * n // 4, n // 4:3 * n // 4] = 1
    rho = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.05
    return rho, S, A


@pytest.mark.parametrize("loss,eps", [("amplitude", 0.0), ("poisson", 1e-3)])
def test_gradient_matches_fp64_finite_differences(loss, eps):
    rho, S, A = case()
    L, G = o.farfield_loss_grad(rho, S, A, loss, eps)
    rng = np.random.default_rng(5)
    for _ in range(4):
        d = (rng.standard_normal(rho.shape) + 1j * rng.standard_normal(rho.shape)) * (S > 0)
        h = 1e-6
        Lp, _ = o.farfield_loss_grad(rho + h * d, S, A, loss, eps)
        Lm, _ = o.farfield_loss_grad(rho - h * d, S, A, loss, eps)
        fd = (Lp - Lm) / (2 * h)
        an = float(np.real(np.vdot(G, d)))  # dL = Re <G, d>
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an))


@pytest.mark.parametrize("loss,eps", [("amplitude", 0.0), ("poisson", 1e-3)])
def test_gradient_matches_torch_autograd(loss, eps):
    rho, S, A = case(seed=3)
    L, G = o.farfield_loss_grad(rho, S, A, loss, eps)
    r = torch.tensor(rho, dtype=torch.complex128, requires_grad=True)
    Sm = torch.tensor((S > 0).astype(np.float64))
    At = torch.tensor(A)
    n = rho.shape[0]
    F = torch.fft.ifft2(r * Sm) * (n * n)
    known = At >= 0
    if loss == "amplitude":
        Lt = ((F.abs() - At) ** 2)[known].sum()
    else:
        m2 = F.abs() ** 2
        Lt = (m2 - At ** 2 * torch.log(m2 + eps))[known].sum()
    Lt.backward()
    assert abs(Lt.item() - L) <= 1e-10 * abs(L)
    assert np.allclose(r.grad.numpy(), G, rtol=1e-9, atol=1e-9 * np.abs(G).max())


def test_zero_gradient_at_the_solution():
    rho, S, _ = case(seed=7)
    rho = rho * (S > 0)
    A = np.abs(o.ft(rho))
    A[3, 5] = -1.0
    L, G = o.farfield_loss_grad(rho, S, A, "amplitude")
    assert L < 1e-20 and np.abs(G).max() < 1e-9
