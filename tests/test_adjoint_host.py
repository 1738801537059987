"""Host-side pieces of the differentiable transport (no GPU): the checkpoint segments and
reinitialization schedule, the divergence-free velocity modes and the smoothed
Heaviside of the mismatch loss."""
import importlib
import math

import numpy as np
import pytest
import torch


@pytest.fixture(scope="module")
def A(pkg):
    return importlib.import_module(pkg.__name__ + ".adjoint")


@pytest.fixture(scope="module")
def S(pkg):
    return importlib.import_module(pkg.__name__ + ".sdf3")


def test_segments_cover_every_step_once(A):
    for steps, ck in ((40, 10), (7, 3), (5, 1), (4, 8)):
        plan = A.TransportPlan(steps=steps, checkpoint_every=ck)
        seen = [s for a, b in plan.segments() for s in range(a, b)]
        assert seen == list(range(steps))
        assert all(b - a <= ck for a, b in plan.segments())


def test_reinit_schedule(A):
    plan = A.TransportPlan(steps=40, reinit_every=10, reinit_iters=10)
    assert [s for s in range(40) if plan.reinit_after(s)] == [9, 19, 29, 39]
    assert not any(A.TransportPlan(steps=5, reinit_every=0).reinit_after(s) for s in range(5))
    assert not any(A.TransportPlan(steps=5, reinit_every=1, reinit_iters=0).reinit_after(s) for s in range(5))


def test_fourier_modes_divergence_free(A, S):
    n = 32
    v = np.linspace(-1.5, 1.5, n, endpoint=False)
    X, Y, Z = S.GD3.meshgrid(v, v, v, device="cpu")
    grid = S.GD3(X, Y, Z, device="cpu")
    modes = A.fourier_modes(grid, 8, 3.0, seed=0)
    assert modes.shape == (8, 3, n, n, n)
    h = float(v[1] - v[0])
    kap = 2 * np.pi * np.fft.fftfreq(n, d=h)

    def deriv(f, axis):  # spectral derivative, exact for these periodic band-limited modes
        shape = [1, 1, 1]
        shape[axis] = n
        return np.real(np.fft.ifft(1j * kap.reshape(shape) * np.fft.fft(f, axis=axis), axis=axis))

    for m in range(8):
        u = modes[m].numpy()
        assert np.isclose(np.sqrt((u ** 2).sum(0)).max(), 1.0, atol=0.05)  # unit polarisation
        # arrays are (rows = y, cols = x, pges = z)
        div = deriv(u[0], 1) + deriv(u[1], 0) + deriv(u[2], 2)
        scale = max(np.abs(deriv(u[a], ax)).max() for a in range(3) for ax in range(3))
        assert np.abs(div).max() <= 1e-12 * scale


def test_velocity_is_linear_in_amplitudes(A, S):
    v = np.linspace(-1, 1, 8)
    X, Y, Z = S.GD3.meshgrid(v, v, v, device="cpu")
    grid = S.GD3(X, Y, Z, device="cpu")
    modes = A.fourier_modes(grid, 4, 2.0, seed=1)
    a = torch.tensor([0.1, -0.2, 0.05, 0.3], dtype=torch.float64)
    b = torch.tensor([0.0, 0.4, -0.1, 0.2], dtype=torch.float64)
    va, vb, vab = A.velocity(a, modes), A.velocity(b, modes), A.velocity(a + b, modes)
    for q in range(3):
        assert torch.allclose(va[q] + vb[q], vab[q], atol=1e-14)
        assert S.is_colmajor(va[q])


def test_smoothed_heaviside(A):
    eps = 0.1
    phi = torch.linspace(-0.3, 0.3, 601, dtype=torch.float64)
    H = A.smoothed_heaviside(phi, eps)
    assert torch.all(H[phi <= -eps] == 0) and torch.all(H[phi >= eps] == 1)
    assert abs(float(A.smoothed_heaviside(torch.tensor(0.0, dtype=torch.float64), eps)) - 0.5) < 1e-15
    assert torch.all(torch.diff(H) >= -1e-15)  # monotone up to rounding
    # derivative (1 + cos(pi phi/eps)) / (2 eps) inside the band
    p = torch.tensor([0.03], dtype=torch.float64, requires_grad=True)
    A.smoothed_heaviside(p, eps).sum().backward()
    assert abs(float(p.grad) - (1 + math.cos(math.pi * 0.3)) / (2 * eps)) < 1e-12
