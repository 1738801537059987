"""Parity of the method-level operations (the SD.SDF3 mirror over the C ABI, fused GB300
kernels) with the oracle's restatement of the MATLAB loops.

Plain FP64 form: every grid value within 1e-12 of the oracle, relative to the field's
scale (max(|field|, 1)), single stages and short loops; long loops (100 pseudo-steps at
the full 64^3 reinitialization size) within 1e-10, where one-ulp differences of FMA
contraction can move a WENO/Godunov switch.  GPU only."""
import importlib

import numpy as np
import pytest
import torch

from conftest import GOLDEN_CASES, load_golden
from gpu_util import dev, host, max_rel

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")
TOL = 1e-12
TOL_LONG = 1e-10


def make(pkg, x, y, z, F, precision="f64", spacing=None):
    grid = pkg.GD3(x, y, z, spacing=spacing)
    return pkg.SDF3(grid, x, y, z, F, precision=precision)


def ograd(O, x, y, z):
    return O.grid_from_mesh(x, y, z)


@pytest.fixture(scope="module")
def config1(pkg, vsl, oracle_mod):
    """The reinitialization workload at full size: 64^3 on [-1,1]^3, dx = 2/63."""
    x, y, z = S.cube_grid(64, -1.0, 1.0)
    F = S.perturbed_sphere(x, y, z)
    return x, y, z, F


def test_set_distance_config1(pkg, oracle_mod, config1):
    O = oracle_mod
    x, y, z, F = config1
    m = make(pkg, x, y, z, F)
    m.setDistance()
    d = O.set_distance(O.kernels("port"), ograd(O, x, y, z), F)
    for a, b in zip(m._dist(), d.six()):
        assert max_rel(host(a), b) <= TOL


@pytest.mark.parametrize("iters", [1, 100])
def test_weno5_reinit_config1(pkg, oracle_mod, config1, iters):
    O = oracle_mod
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    K = O.kernels("port")
    m = make(pkg, x, y, z, F)
    m.setDistance()
    got = host(m.WENO5RK3Reinitialization(m.F, iters))
    ref = O.reinit_weno5(K, g, F, iters, O.set_distance(K, g, F))
    assert max_rel(got, ref) <= (TOL if iters == 1 else TOL_LONG)


@pytest.mark.parametrize("iters", [1, 100])
def test_eno3_reinit_config1(pkg, oracle_mod, config1, iters):
    O = oracle_mod
    x, y, z, F = config1
    m = make(pkg, x, y, z, F)
    got = host(m.WENORK3Reinitialization(m.F, iters))
    ref = O.reinit_eno3(O.kernels("port"), ograd(O, x, y, z), F, iters)
    assert max_rel(got, ref) <= (TOL if iters == 1 else TOL_LONG)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_loops(pkg, vsl, name):
    """The reference's own loop outputs (4 reinit / 3 extension pseudo-steps, surface
    redistance 2x2) on the golden inputs, including grids smaller than the stencil."""
    G = load_golden(name)
    r, c, p, dx, dy, dz = G["grid"]
    shape = (int(r), int(c), int(p))
    x = np.zeros(shape, order="F")
    m = make(pkg, x, x, x, G["F"], spacing=(dx, dy, dz))
    m.setDistance()
    assert max_rel(host(m.WENO5RK3Reinitialization(m.F, 4)), G["reinit5_it4"]) <= TOL
    assert max_rel(host(m.WENORK3Reinitialization(m.F, 4)), G["reinit3_it4"]) <= TOL
    C = dev(G["C"])
    assert max_rel(host(m.WENO5RK3Extend(C, 3)), G["extend5_it3"]) <= TOL
    assert max_rel(host(m.WENORK3Extend(C, 3)), G["extend3_it3"]) <= TOL
    assert max_rel(host(m.WENO5RK3ClosetPointSurfaceRedistance(C, 2, 2)), G["redistance_2_2"]) <= TOL
    av = m.area_volume().cpu().numpy()
    assert abs(av[0] - float(G["area"])) <= 1e-12 * max(1.0, abs(float(G["area"])))
    assert abs(av[1] - float(G["volume"])) <= 1e-12 * max(1.0, abs(float(G["volume"])))


@pytest.mark.parametrize("eno3", [False, True])
def test_extend_config1(pkg, oracle_mod, config1, eno3):
    O = oracle_mod
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    K = O.kernels("port")
    C = S.surface_field(x, y, z)
    m = make(pkg, x, y, z, F)
    m.setDistance()
    if eno3:
        got = host(m.WENORK3Extend(dev(C), 30))
        ref = O.extend_eno3(K, g, F, C, 30)
    else:
        got = host(m.WENO5RK3Extend(dev(C), 30))
        ref = O.extend_weno5(K, g, F, O.set_distance(K, g, F), C, 30)
    assert max_rel(got, ref) <= TOL_LONG


def test_surface_redistance(pkg, oracle_mod):
    O = oracle_mod
    x, y, z = S.cube_grid(28, -1.0, 1.0)
    F = np.asfortranarray(np.sqrt(x**2 + y**2 + z**2) - 0.6)
    A = np.asfortranarray(np.exp(z) - 1)
    m = make(pkg, x, y, z, F)
    got = host(m.WENO5RK3ClosetPointSurfaceRedistance(dev(A), 3, 6))
    ref = O.surface_redistance(O.kernels("port"), ograd(O, x, y, z), F, A, 3, 6)
    assert max_rel(got, ref) <= TOL_LONG


def test_area_volume_and_toolbox(pkg, oracle_mod, config1):
    O = oracle_mod
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    m = make(pkg, x, y, z, F)
    tb = O.calculus_toolbox(O.kernels("port"), g, F)
    av = m.area_volume().cpu().numpy()
    assert abs(av[0] - O.cal_area(g, F, tb["DiracDelta"])) <= 1e-12 * abs(av[0])
    assert abs(av[1] - O.cal_volume(g, F, tb["Heaviside"])) <= 1e-12 * abs(av[1])
    # bitwise reproducible
    assert np.array_equal(av, m.area_volume().cpu().numpy())
    m.GPUsetCalculusToolBox()
    for k in O.TOOLBOX_FIELDS:
        assert max_rel(host(getattr(m, k)), tb[k]) <= TOL, k


def test_advection_rk3(pkg, oracle_mod, config1):
    O = oracle_mod
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    vx = np.asfortranarray(-y + 0.3 * np.sin(2 * z))
    vy = np.asfortranarray(x.copy())
    vz = np.asfortranarray(0.5 * np.cos(3 * x) * y)
    dt = 0.5 * g.ds / 1.5
    m = make(pkg, x, y, z, F)
    got = host(m.WENO5RK3Advection(m.F, dev(vx), dev(vy), dev(vz), dt, steps=3))
    ref = O.advect_rk3(O.kernels("port"), g, F, vx, vy, vz, dt, steps=3)
    assert max_rel(got, ref) <= TOL


def test_vesicle_step(pkg, oracle_mod):
    """The composite step (toolbox -> extension 30 -> dt -> advection -> setDistance ->
    reinit 20) on the noisy oblate vesicle at 48^3, two steps."""
    O = oracle_mod
    x, y, z = S.cube_grid(48, -1.5, 1.5)
    F = S.noisy_oblate(x, y, z, seed=3)
    g = ograd(O, x, y, z)
    K = O.kernels("port")
    m = make(pkg, x, y, z, F)
    m.setDistance()
    Fo, do = F, O.set_distance(K, g, F)
    for _ in range(2):
        info = m.vesicle_step(30, 20, 0.5).cpu().numpy()
        Fo, do, oi = O.vesicle_step(K, g, Fo, do, 30, 20, 0.5)
        assert abs(info[0] - oi["area"]) <= 1e-11 * oi["area"]
        assert abs(info[1] - oi["volume"]) <= 1e-11 * oi["volume"]
        assert abs(info[2] - oi["dt"]) <= 1e-10 * oi["dt"]
    assert max_rel(host(m.F), Fo) <= TOL_LONG
    for a, b in zip(m._dist(), do.six()):
        assert max_rel(host(a), b) <= TOL_LONG


def test_deterministic(pkg, config1):
    x, y, z, F = config1
    m = make(pkg, x, y, z, F)
    m.setDistance()
    a = m.WENO5RK3Reinitialization(m.F, 5)
    b = m.WENO5RK3Reinitialization(m.F, 5)
    assert torch.equal(a, b)
