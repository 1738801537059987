"""The FP64 vesicle-step workload at 128^3: 50 steps of the oblate vesicle (axes
(1, 1, 0.55), l <= 6 harmonic noise of amplitude 0.02) on [-1.5, 1.5]^3, normal speed =
mean curvature, 30 extension + 1 advection (CFL 0.5) + 20 reinitialization pseudo-steps
per step, after the driver's set-up (setDistance and 500 reinitialization pseudo-steps).

The first two FP64 steps from the set-up state are compared with the oracle: bitwise
against the oracle built with integer powers rounded once (the FP64 form's arithmetic),
area and volume within 1e-14 (fixed-order tree against a correctly rounded sum).  The
50-step history is checked through properties that hold at any size.  Mean-curvature flow moves the surface
inward: the enclosed volume shrinks every step and the area shrinks overall.  The
advective CFL 0.5 time step is above the parabolic stability limit of an explicit
curvature flow (about dx^2 / 6), so after a few steps a grid-scale oscillation grows until
max |Vn| has risen about 15-fold and the CFL rule has shrunk dt to match; from then on the
flow runs at that saturated state.  Before the onset the mixed-precision history follows
the FP64 one to rounding level; after it the unstable modes amplify rounding, and the two
histories stay within a few per cent.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 50
N = 128


def setup(pkg, precision):
    S = importlib.import_module(pkg.__name__ + ".shapes")
    v = np.linspace(-1.5, 1.5, N)
    x, y, z = S.meshgrid(v, v, v, device="cuda")
    F0 = S.noisy_oblate(x, y, z, axes=(1.0, 1.0, 0.55), amplitude=0.02, seed=0)
    h = 3.0 / (N - 1)
    grid = pkg.GD3(x, y, z, spacing=(h, h, h))
    m = pkg.SDF3(grid, Val=F0, precision=precision)
    # the driver's set-up: setDistance, then 500 reinitialization pseudo-steps
    # (p00_test_singlephase_relax.m:27-28)
    m.setDistance()
    m.F = m.WENO5RK3Reinitialization(m.F, 500)
    m.setDistance()
    return m


def test_fp64_steps_match_oracle_128(pkg, vsl, oracle_mod):
    from gpu_util import host

    O = oracle_mod
    m = setup(pkg, "f64")
    h = 3.0 / (N - 1)  # the spacing the level-set object was given
    g = O.Grid(N, N, N, h, h, h)
    KC = O.kernels("port_crpow")
    Fo = host(m.F)
    do = O.Distances(*(host(t) for t in m._dist()))
    for _ in range(2):
        info = m.vesicle_step(30, 20, 0.5).cpu().numpy()
        Fo, do, oi = O.vesicle_step(KC, g, Fo, do, 30, 20, 0.5)
        assert abs(info[0] - oi["area"]) <= 1e-14 * oi["area"]
        assert abs(info[1] - oi["volume"]) <= 1e-14 * oi["volume"]
        assert info[2] == oi["dt"] and info[3] == oi["vmax"]
        assert np.array_equal(host(m.F), Fo)
        for a, b in zip(m._dist(), do.six()):
            assert np.array_equal(host(a), b)


def history(pkg, precision):
    import torch

    m = setup(pkg, precision)
    rows = []
    for _ in range(STEPS):
        rows.append(m.vesicle_step(30, 20, 0.5).cpu().numpy().copy())
    torch.cuda.synchronize()
    return np.array(rows)  # columns: area, volume (before the step), dt, max |Vn|


def test_area_volume_history_128(pkg, vsl):
    h64 = history(pkg, "f64")
    h32 = history(pkg, "f32")
    area, vol = h64[:, 0], h64[:, 1]
    print("\nstep area volume dt maxVn (FP64) | area, volume rel. diff FP32")
    for s in range(STEPS):
        print(s, area[s], vol[s], h64[s, 2], h64[s, 3], abs(h32[s, 0] / area[s] - 1), abs(h32[s, 1] / vol[s] - 1))
    assert np.all(np.isfinite(h64)) and np.all(h64[:, 2] > 0)
    assert np.all(np.diff(vol) < 0), vol
    assert area[-1] < 0.9 * area[0]
    # steps before the oscillation sets in: max |Vn| still within twice its first value
    calm = int(np.argmax(h64[:, 3] > 2 * h64[0, 3]))
    assert calm >= 2
    rel = np.abs(h32[:, :2] / h64[:, :2] - 1)
    print("onset step", calm, "max rel diff FP32 vs FP64 before:", rel[:calm].max(), "after:", rel[calm:].max())
    assert rel[:calm].max() <= 2e-5
    assert rel[calm:].max() <= 5e-2
