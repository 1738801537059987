"""TMA plane loads of the FP32 tiled stage kernels (vsl_set_plane_loads(1)) against the
register plane loads (the default): the same build, the same inputs, every FP32 operator
that runs the tiled kernels.  The planes are the same; the two kernels are compiled apart
and fuse multiply-adds differently, so the outputs agree to a few ulp rather than bit for
bit.  Grids: the 128^3 vesicle (whole tiles), a ragged 100 x 75 x 41 grid (partial tiles:
TMA on every tile, the halo cells outside the grid filled from the clamped cells), and
102 x 64 x 33 (rows not a multiple of 4: no tensor map, registers in both modes, bitwise).
No bounded TMA wait may have given up.  GPU only."""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")
A = importlib.import_module("2018_7_vesicle_gb300.autotune")


def grid_case(size):
    rows, cols, pges = size
    h = 2.4 / (max(size) - 1)
    xv = (np.arange(cols) - (cols - 1) / 2) * h
    yv = (np.arange(rows) - (rows - 1) / 2) * h
    zv = (np.arange(pges) - (pges - 1) / 2) * h
    x, y, z = np.meshgrid(xv, yv, zv)
    F = np.asfortranarray(np.sqrt((x / 0.9) ** 2 + (y / 0.7) ** 2 + (z / 0.5) ** 2) - 0.6
                          + 0.02 * np.sin(5 * x) * np.cos(3 * y))
    return x, y, z, F


def run_all(pkg, x, y, z, F):
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    m.setDistance()
    out = {}
    out["reinit"] = m.WENO5RK3Reinitialization(m.F, 6)
    out["reinit_eno3"] = m.WENORK3Reinitialization(m.F, 4)
    out["enork2_reinit"] = m.ENORK2Reinitialization(m.F, 4)
    C = m.F * 0.5 + 0.25
    out["extend"] = m.WENO5RK3Extend(C, 6)
    out["extend_eno3"] = m.WENORK3Extend(C, 4)
    out["enork2_extend"] = m.ENORK2Extend(C, 4)
    v = torch.ones_like(m.F) * 0.4
    out["advect"] = m.WENO5RK3Advection(m.F, v, -0.5 * v, 0.7 * v, 2e-3, steps=2)
    out["redistance"] = m.WENO5RK3ClosetPointSurfaceRedistance(C, 2, 2)
    m.vesicle_step(6, 4, 0.5)
    out["step"] = m.F.clone()
    torch.cuda.synchronize()
    return {k: t.cpu().numpy() for k, t in out.items()}, float(m.GD3.Dx)


@pytest.mark.parametrize("size", [(128, 128, 128), (100, 75, 41), (102, 64, 33)])
def test_tma_planes_match_register_planes(pkg, vsl, size):
    if size == (128, 128, 128):
        x, y, z, F = S.vesicle_256(128, seed=0)
    else:
        x, y, z, F = grid_case(size)
    before = A.tma_wait_timeouts()
    got = {}
    try:
        for mode in (1, 0):
            A.set_plane_loads(mode)
            assert A.plane_loads() == mode
            got[mode], dx = run_all(pkg, x, y, z, F)
    finally:
        A.set_plane_loads(0)
    for k in got[0]:
        a, b = got[1][k].astype(np.float64), got[0][k].astype(np.float64)
        if size[0] % 4:
            assert np.array_equal(a, b), k  # no tensor map: the same kernel
            continue
        # a few ulp of the field's own scale (level sets: of dx-sized band values and of the
        # grid's largest distances)
        tol = 8 * np.finfo(np.float32).eps * max(float(np.max(np.abs(b))), dx)
        diff = float(np.max(np.abs(a - b)))
        assert diff <= tol, (k, diff, tol)
    assert A.tma_wait_timeouts() == before == 0
