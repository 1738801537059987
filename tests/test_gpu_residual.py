"""The residual-driven reinitialization (vsl_weno5_rk3_reinitialization_tol_*) against the
oracle's loop (oracle.reinit_weno5_tol), through the C ABI.

* FP64: the residual history within 1e-12 of the oracle's (relative to the first
  residual), the same number of pseudo-steps and the same convergence flag, and the field
  bitwise equal to the fixed-count entry point run for that many pseudo-steps;
* FP32: the residual (FP64 arithmetic on the promoted FP32 values) within 1e-4 of the
  oracle's at every pseudo-step, the step count within one of the oracle's, and the field
  bitwise equal to the FP32 fixed-count entry point run for that many pseudo-steps;
* the cap: with tol 0 the loop stops after max_iters pseudo-steps and reports no
  convergence; with max_iters 0 it takes no step and reports the input's residual;
* recorded inside the caller's own CUDA graph capture, a replay gives the direct call's
  result bit for bit.

GPU only."""
import importlib

import numpy as np
import pytest
import torch

from gpu_util import host

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")


@pytest.fixture(scope="module")
def case(oracle_mod):
    O = oracle_mod
    x, y, z = S.cube_grid(48, -1.0, 1.0)
    F = S.perturbed_sphere(x, y, z)
    g = O.grid_from_mesh(x, y, z)
    K = O.kernels("port")
    return O, K, g, x, y, z, F, O.set_distance(K, g, F)


def run(pkg, x, y, z, F, precision, max_iters, tol, band):
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision=precision)
    m.setDistance()
    out, status, res = m.WENO5RK3ReinitializationTol(m.F, max_iters, tol, band)
    torch.cuda.synchronize()
    return m, out, status.cpu().numpy(), res.cpu().numpy()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_converges_like_the_oracle(pkg, vsl, case, precision):
    O, K, g, x, y, z, F, d = case
    tol, band, cap = 2e-3, 3 * g.dx, 200
    Fo, n, conv, hist = O.reinit_weno5_tol(K, g, F, cap, tol, band, d)
    assert conv and 0 < n < cap
    m, out, st, res = run(pkg, x, y, z, F, precision, cap, tol, band)
    steps = int(st[0])
    assert st[1] == 1
    if precision == "f64":
        assert steps == n
        assert np.max(np.abs(res[: n + 1] - hist)) <= 1e-12 * hist[0]
    else:
        assert abs(steps - n) <= 1
        k = min(steps, n) + 1
        assert np.max(np.abs(res[:k] - hist[:k])) <= 1e-4 * hist[0]
    assert np.all(np.isnan(res[steps + 1:]))
    assert res[steps] <= tol < res[steps - 1]
    # the field is the fixed-count operation's after the same number of pseudo-steps
    assert np.array_equal(host(out), host(m.WENO5RK3Reinitialization(m.F, steps)))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_cap_and_zero_steps(pkg, vsl, case, precision):
    O, K, g, x, y, z, F, d = case
    band = 3 * g.dx
    m, out, st, res = run(pkg, x, y, z, F, precision, 3, 0.0, band)
    assert st[0] == 3 and st[1] == 0 and np.all(res > 0)
    assert np.array_equal(host(out), host(m.WENO5RK3Reinitialization(m.F, 3)))
    m, out, st, res = run(pkg, x, y, z, F, precision, 0, 1e-3, band)
    assert st[0] == 0 and st[1] == 0 and res.shape == (1,)
    r0 = O.reinit_residual(K, g, F, np.asfortranarray(F < 0), d, band)
    assert abs(res[0] - r0) <= (1e-12 if precision == "f64" else 1e-4) * r0
    assert np.array_equal(host(out), host(m.F))


def test_inside_a_caller_graph(pkg, vsl, case):
    O, K, g, x, y, z, F, d = case
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    m.setDistance()
    ref, st_ref, res_ref = m.WENO5RK3ReinitializationTol(m.F, 100, 2e-3, 3 * g.dx)
    torch.cuda.synchronize()
    src = m.F.clone()
    m.workspace("reinit_tol")
    graph = torch.cuda.CUDAGraph()
    out = None
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            out, st, res = m.WENO5RK3ReinitializationTol(src, 100, 2e-3, 3 * g.dx)
    torch.cuda.current_stream().wait_stream(s)
    for _ in range(2):
        graph.replay()
        torch.cuda.synchronize()
        assert np.array_equal(st.cpu().numpy(), st_ref.cpu().numpy())
        assert np.array_equal(host(out), host(ref))
        assert np.array_equal(res.cpu().numpy(), res_ref.cpu().numpy(), equal_nan=True)
