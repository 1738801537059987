"""Adjoint of the WENO5 TVD-RK3 advection and reinitialization steps (the
differentiation workload) against central finite differences.

* FP64 directional derivatives of a linear functional of the transported field, through
  advection alone and through reinitialization alone (including its interface-distance
  roots), against central differences of the GPU FP64 forward map;
* the gradient of the Heaviside-mismatch loss with respect to the 8 velocity-mode
  amplitudes against central differences with h = 1e-4 (FP64);
* the same gradient against central differences of the oracle's forward map (the
  reference kernels' arithmetic on the CPU): the reference-derived gradient;
* checkpoint spacing does not change the gradient (bitwise), and the FP32 adjoint agrees
  with the FP64 one.
"""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZE = (20, 18, 16)  # rows (y), cols (x), pges (z)


@pytest.fixture(scope="module")
def A(pkg, vsl):
    return importlib.import_module(pkg.__name__ + ".adjoint")


@pytest.fixture(scope="module")
def S(pkg):
    return importlib.import_module(pkg.__name__ + ".sdf3")


def make_grid(S, size=SIZE, lo=-1.0, hi=1.0):
    rows, cols, pges = size
    xv, yv, zv = np.linspace(lo, hi, cols), np.linspace(lo, hi, rows), np.linspace(lo, hi, pges)
    return S.GD3(*S.GD3.meshgrid(xv, yv, zv))


def initial_field(grid):
    X, Y, Z = grid.X, grid.Y, grid.Z
    r = torch.sqrt((X - 0.05) ** 2 + (Y + 0.03) ** 2 + (Z / 0.8) ** 2)
    return (r - 0.55) * (1.0 + 0.6 * (X - 0.2) ** 2 + 0.3 * Y * Z)  # not a distance function


def smooth_weight(grid, seed):
    rng = np.random.default_rng(seed)
    a, b, c, d = rng.uniform(0.5, 2.5, 4)
    X, Y, Z = grid.X, grid.Y, grid.Z
    return torch.cos(a * X + 0.3) * torch.sin(b * Y + c * Z + 0.1) + 0.2 * torch.cos(d * Z)


def colmajor(S, t, dtype=torch.float64):
    return S.as_field(t, dtype)


def directional_check(fwd, grad_dirs, dirs, h):
    """central difference of fwd along dirs versus sum of <grad, dir>"""
    plus = fwd([h * d for d in dirs])
    minus = fwd([-h * d for d in dirs])
    fd = (plus - minus) / (2 * h)
    an = sum(float((g * d).sum()) for g, d in zip(grad_dirs, dirs))
    return fd, an


def test_advection_adjoint_directional(A, S):
    grid = make_grid(S)
    phi0 = colmajor(S, initial_field(grid))
    modes = A.fourier_modes(grid, 8, 3.0, seed=3)
    a = torch.tensor(np.random.default_rng(4).normal(0, 0.3, 8), dtype=torch.float64, device="cuda")
    v = [colmajor(S, t) for t in A.velocity(a, modes)]
    dt = A.time_step(a, modes, grid)
    plan = A.TransportPlan(steps=3, reinit_every=0, reinit_iters=0, checkpoint_every=2)
    tr = A.Transport(grid, dt, plan, "f64")
    w = colmajor(S, smooth_weight(grid, 5))

    p0 = phi0.clone().requires_grad_(True)
    vv = [t.clone().requires_grad_(True) for t in v]
    L = (tr(p0, *vv) * w).sum()
    L.backward()
    grads = [p0.grad] + [t.grad for t in vv]

    d_phi = colmajor(S, smooth_weight(grid, 6))
    d_v = [colmajor(S, t) for t in A.velocity(torch.tensor(np.random.default_rng(7).normal(0, 0.3, 8),
                                                            device="cuda"), modes)]
    dirs = [d_phi] + d_v

    def fwd(delta):
        with torch.no_grad():
            out = tr(phi0 + delta[0], *[v[q] + delta[q + 1] for q in range(3)])
            return float((out * w).sum())

    fd, an = directional_check(fwd, grads, dirs, 1e-6)
    assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


def test_reinit_adjoint_directional(A, S):
    grid = make_grid(S)
    phi0 = colmajor(S, initial_field(grid))
    zero = [torch.zeros_like(phi0) for _ in range(3)]
    plan = A.TransportPlan(steps=1, reinit_every=1, reinit_iters=3, checkpoint_every=1)
    tr = A.Transport(grid, 1e-3, plan, "f64")
    w = colmajor(S, smooth_weight(grid, 8))
    p0 = phi0.clone().requires_grad_(True)
    L = (tr(p0, *zero) * w).sum()
    L.backward()
    d_phi = colmajor(S, smooth_weight(grid, 9))

    def fwd(delta):
        with torch.no_grad():
            return float((tr(phi0 + delta[0], *zero) * w).sum())

    fd, an = directional_check(fwd, [p0.grad], [d_phi], 1e-6)
    assert abs(fd - an) <= 1e-5 * abs(an), (fd, an)


def mismatch_setup(A, S, size=SIZE, steps=4):
    grid = make_grid(S, size)
    phi0 = colmajor(S, initial_field(grid))
    modes = A.fourier_modes(grid, 8, 3.0, seed=11)
    a0 = torch.tensor(np.random.default_rng(12).normal(0, 0.1, 8), dtype=torch.float64, device="cuda")
    a_tgt = torch.tensor(np.random.default_rng(13).normal(0, 0.1, 8), dtype=torch.float64, device="cuda")
    dt = A.time_step(a0, modes, grid)
    plan = A.TransportPlan(steps=steps, reinit_every=2, reinit_iters=2, checkpoint_every=2)
    eps = 1.5 * grid.Dx
    dv = grid.Dx * grid.Dy * grid.Dz
    return grid, phi0, modes, a0, a_tgt, dt, plan, eps, dv


def amplitude_gradient(A, S, precision, setup, plan=None):
    grid, phi0, modes, a0, a_tgt, dt, plan0, eps, dv = setup
    tr = A.Transport(grid, dt, plan or plan0, precision)
    dtype = tr.dtype
    with torch.no_grad():
        target = tr(phi0.to(dtype), *[t.to(dtype) for t in A.velocity(a_tgt, modes)])
    a = a0.clone().requires_grad_(True)
    v = [t.to(dtype) for t in A.velocity(a, modes)]
    L = A.heaviside_mismatch(tr(phi0.to(dtype), *v), target, eps, dv)
    L.backward()
    return float(L.detach()), a.grad.detach().cpu().numpy(), tr, target


def test_amplitude_gradient_vs_central_differences(A, S):
    setup = mismatch_setup(A, S)
    grid, phi0, modes, a0, a_tgt, dt, plan, eps, dv = setup
    L, g, tr, target = amplitude_gradient(A, S, "f64", setup)
    assert L > 0

    def loss(a):
        with torch.no_grad():
            return float(A.heaviside_mismatch(tr(phi0, *A.velocity(a, modes)), target, eps, dv))

    h = 1e-4
    fd = np.zeros(8)
    for m in range(8):
        e = torch.zeros(8, dtype=torch.float64, device="cuda")
        e[m] = h
        fd[m] = (loss(a0 + e) - loss(a0 - e)) / (2 * h)
    err = np.abs(fd - g).max() / np.abs(fd).max()
    assert err <= 1e-3, (fd, g)


def test_checkpoint_spacing_does_not_change_gradient(A, S):
    setup = mismatch_setup(A, S)
    plan = setup[6]
    _, g1, _, _ = amplitude_gradient(A, S, "f64", setup, A.TransportPlan(plan.steps, plan.reinit_every,
                                                                         plan.reinit_iters, 1))
    _, g4, _, _ = amplitude_gradient(A, S, "f64", setup, A.TransportPlan(plan.steps, plan.reinit_every,
                                                                         plan.reinit_iters, plan.steps))
    assert np.array_equal(g1, g4)


def test_fp32_adjoint_matches_fp64(A, S):
    setup = mismatch_setup(A, S)
    _, g64, _, _ = amplitude_gradient(A, S, "f64", setup)
    _, g32, _, _ = amplitude_gradient(A, S, "f32", setup)
    err = np.abs(g32 - g64).max() / np.abs(g64).max()
    assert err <= 1e-3, (g32, g64)


def test_gradient_vs_oracle_central_differences(A, S, oracle_mod):
    """Central differences of the oracle's forward map (the reference kernels' arithmetic
    on the CPU: advect_rk3, set_distance, reinit_weno5) against the GPU FP64 adjoint."""
    O = oracle_mod
    K = O.kernels("port")
    size = (14, 12, 10)
    setup = mismatch_setup(A, S, size=size, steps=2)
    grid, phi0, modes, a0, a_tgt, dt, plan, eps, dv = setup
    L, g, tr, target = amplitude_gradient(A, S, "f64", setup)
    og = O.Grid(*size, grid.Dx, grid.Dy, grid.Dz)
    m_np = modes.cpu().numpy()
    phi_np = S.to_numpy(phi0)
    tgt_np = S.to_numpy(target)

    def oracle_forward(a):
        v = [np.asfortranarray(np.tensordot(a, m_np[:, q], axes=1)) for q in range(3)]
        F = phi_np.copy(order="F")
        for s in range(plan.steps):
            F = O.advect_rk3(K, og, F, *v, dt, 1)
            if plan.reinit_after(s):
                F = O.reinit_weno5(K, og, F, plan.reinit_iters, O.set_distance(K, og, F))
        return F

    def H(f):
        t = np.clip(f / eps, -1.0, 1.0)
        return 0.5 * (1.0 + t + np.sin(np.pi * t) / np.pi)

    def loss(a):
        return float(((H(oracle_forward(a)) - H(tgt_np)) ** 2).sum() * dv)

    a_np = a0.cpu().numpy()
    assert abs(loss(a_np) - L) <= 1e-12 * abs(L)  # the oracle forward is the GPU forward
    h = 1e-4
    fd = np.array([(loss(a_np + h * e) - loss(a_np - h * e)) / (2 * h) for e in np.eye(8)])
    err = np.abs(fd - g).max() / np.abs(fd).max()
    assert err <= 1e-3, (fd, g)
