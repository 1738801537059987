"""The FP64 vesicle-step workload at 128^3: 50 steps of the oblate vesicle (axes
(1, 1, 0.55), l <= 6 harmonic noise of amplitude 0.02) on [-1.5, 1.5]^3, normal speed =
mean curvature, 30 extension + 1 advection (CFL 0.5) + 20 reinitialization pseudo-steps
per step, after the driver's set-up (setDistance and 500 reinitialization pseudo-steps).

At this size the oracle is too slow for a step-by-step comparison (the FP64 step is
bitwise equal to the oracle on the smaller grids of test_gpu_methods), so the history is
checked through properties that hold at any size.  Mean-curvature flow moves the surface
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


def history(pkg, precision):
    import torch

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
