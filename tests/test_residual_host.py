"""The residual-driven reinitialization without a GPU: argument checks of the C ABI (all
made before any CUDA call), and the oracle's loop stopping by its cap or its tolerance."""
import importlib

import numpy as np

from conftest import ROOT  # noqa: F401  (puts the repository on sys.path)

S = importlib.import_module("2018_7_vesicle_gb300.shapes")

FAKE = 0x1000  # never dereferenced: every call below fails its checks first
VSL_ERR_NULL, VSL_ERR_VALUE, VSL_ERR_WORKSPACE = 1, 3, 4
G = (16, 16, 16, 0.1, 0.1, 0.1)


def call(vsl, suf, max_iters=5, tol=1e-3, band=0.3, status=FAKE, ws=None, nbytes=0):
    d = [FAKE] * 6
    return vsl.raw(f"vsl_weno5_rk3_reinitialization_tol_{suf}", FAKE, max_iters, tol, band, *d, *G, status, None, ws,
                   nbytes, None)


def test_rejects_bad_arguments(vsl):
    for suf in ("f64", "f32"):
        assert call(vsl, suf, status=None) == VSL_ERR_NULL
        assert call(vsl, suf, max_iters=-1) == VSL_ERR_VALUE
        assert call(vsl, suf, tol=-1e-3) == VSL_ERR_VALUE
        assert call(vsl, suf, tol=float("nan")) == VSL_ERR_VALUE
        assert call(vsl, suf, band=0.0) == VSL_ERR_VALUE
        assert call(vsl, suf, band=float("nan")) == VSL_ERR_VALUE
        # valid arguments, no workspace: rejected before anything is recorded
        assert call(vsl, suf) == VSL_ERR_WORKSPACE
        assert call(vsl, suf, ws=FAKE + 1, nbytes=1 << 30) == VSL_ERR_WORKSPACE  # misaligned


def test_workspace_of_the_loop(vsl):
    r, c, p = 40, 36, 32
    for e in (4, 8):
        assert vsl.workspace_bytes("reinit_tol", r, c, p, e) > vsl.workspace_bytes("reinit_weno5", r, c, p, e)


def oracle_case(oracle_mod, n=24):
    O = oracle_mod
    x, y, z = S.cube_grid(n, -1.0, 1.0)
    F = S.perturbed_sphere(x, y, z)
    g = O.grid_from_mesh(x, y, z)
    K = O.kernels("port")
    return O, K, g, F, O.set_distance(K, g, F)


def test_oracle_loop_stops_at_its_cap(oracle_mod):
    O, K, g, F, d = oracle_case(oracle_mod)
    Fo, n, conv, hist = O.reinit_weno5_tol(K, g, F, 2, 0.0, 3 * g.dx, d)
    assert n == 2 and not conv and len(hist) == 3
    assert np.array_equal(Fo, O.reinit_weno5(K, g, F, 2, d))


def test_oracle_loop_stops_at_its_tolerance(oracle_mod):
    O, K, g, F, d = oracle_case(oracle_mod)
    Fo, n, conv, hist = O.reinit_weno5_tol(K, g, F, 200, 2e-3, 3 * g.dx, d)
    assert conv and 0 < n < 200
    assert hist[-1] <= 2e-3 < hist[-2]
    assert np.array_equal(Fo, O.reinit_weno5(K, g, F, n, d))
    # a zero cap takes no step and reports the input's residual
    F0, n0, conv0, hist0 = O.reinit_weno5_tol(K, g, F, 0, 2e-3, 3 * g.dx, d)
    assert n0 == 0 and not conv0 and hist0 == hist[:1] and np.array_equal(F0, F)
