"""The reference's own CUDA kernels on the GPU (the plain FP64 reference GPU form of
oracle/refgpu.py: the reference's .cu files compiled for sm_103a with the reference's
Makefile flags, launched with its block and grid) against the CPU oracle, per grid value
relative to the field's scale.  The reference's Makefiles compile with nvcc's default
multiply-add contraction, the host oracle (the reference's kernels built for the host)
without it, so the two agree to rounding, not bit for bit: within 1e-12 for setDistance,
the reinitialization and the toolbox; within 1e-10 for the extension and the composite
step, whose crossing values evaluate the degree-5 interpolant from monomial coefficients
(boundary_interpolant.cu:78-99), which turns one-ulp differences of the contracted
products into ~1e-11 (measured 1.1e-11 after 30 extension pseudo-steps at 64^3; the dt of
a step 1.3e-12).  Skipped where the reference's PTX was not built (it is built from the
reference checkout, beside the host build of the oracle).  GPU only."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")
TOL = 1e-12
TOL_CROSSING = 1e-10


@pytest.fixture(scope="module")
def ref(oracle_mod):
    from oracle import refgpu

    if not refgpu.available():
        pytest.skip("the reference's PTX is not built here (it needs the reference checkout)")
    return refgpu


def host(t):
    import torch

    torch.cuda.synchronize()
    return np.asfortranarray(t.detach().cpu().numpy())


def rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.fixture(scope="module")
def config1(ref, oracle_mod):
    O = oracle_mod
    x, y, z = S.cube_grid(64, -1.0, 1.0)
    F = S.perturbed_sphere(x, y, z)
    g = O.grid_from_mesh(x, y, z)
    R = ref.RefGpu(ref.Grid(*g.args()))
    return O, O.kernels("port"), g, R, x, y, z, F


def ref_field(F):
    from oracle import refgpu

    return refgpu.field(F)


def test_set_distance_and_reinitialization(config1):
    O, K, g, R, x, y, z, F = config1
    d = O.set_distance(K, g, F)
    Fd = ref_field(F)
    dr = R.set_distance(Fd)
    for a, b in zip(dr, d.six()):
        assert rel(host(a), b) <= TOL
    got = host(R.reinit_weno5(Fd, 100, dr))
    assert rel(got, O.reinit_weno5(K, g, F, 100, d)) <= TOL
    got3 = host(R.reinit_eno3(Fd, 20))
    assert rel(got3, O.reinit_eno3(K, g, F, 20)) <= TOL


def test_extension_and_toolbox(config1):
    O, K, g, R, x, y, z, F = config1
    d = O.set_distance(K, g, F)
    C = S.surface_field(x, y, z)
    Fd = ref_field(F)
    dr = R.set_distance(Fd)
    got = host(R.extend_weno5(Fd, dr, ref_field(C), 30))
    assert rel(got, O.extend_weno5(K, g, F, d, C, 30)) <= TOL_CROSSING
    tb = R.calculus_toolbox(Fd)
    tbo = O.calculus_toolbox(K, g, F)
    for name in ("MeanCurvature", "GaussianCurvature", "Heaviside", "DiracDelta", "Nx"):
        assert rel(host(tb[name]), tbo[name]) <= TOL, name


def test_vesicle_steps(ref, oracle_mod):
    O = oracle_mod
    K = O.kernels("port")
    x, y, z = S.cube_grid(48, -1.5, 1.5)
    F = S.noisy_oblate(x, y, z, seed=3)
    g = O.grid_from_mesh(x, y, z)
    R = ref.RefGpu(ref.Grid(*g.args()))
    Fo, do = F, O.set_distance(K, g, F)
    Fr = ref.field(F)
    dr = R.set_distance(Fr)
    for _ in range(2):
        Fo, do, oi = O.vesicle_step(K, g, Fo, do, 30, 20, 0.5)
        Fr, dr, ri = R.vesicle_step(Fr, dr, 30, 20, 0.5)
        assert rel(host(Fr), Fo) <= TOL_CROSSING
        for k in ("area", "volume", "dt"):
            assert abs(ri[k] / oi[k] - 1) <= TOL_CROSSING, k
