"""Parity of the method-level operations (the SD.SDF3 mirror over the C ABI, fused GB300
kernels) with the oracle's restatement of the MATLAB loops, plain FP64 form.

Two bars, both per grid value:

* bit-identical to the oracle built with integer powers rounded once
  (``kernels("port_crpow")``), the rounding the CUDA plain form uses where the reference
  calls pow(t, n);
* within 1e-12 of the oracle with libm's pow and of the golden outputs of the reference's
  own kernels (relative to the field's scale, max(|field|, 1)).  libm's pow is accurate to
  0.52 ulp but not always correctly rounded; the closest-point surface redistance
  normalises upwind gradients with a 1e-14 floor, which turns such one-ulp differences of
  a crossing value into ~6e-12 (measured: the two oracle builds differ by 6.06e-12 on the
  pear14 window), so that one operation is held to 1e-10 against libm pow.

GPU only."""
import importlib

import numpy as np
import pytest
import torch

from conftest import GOLDEN_CASES, load_golden
from gpu_util import dev, host, max_rel

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")
TOL = 1e-12
TOL_REDIST_LIBM = 1e-10


def make(pkg, x, y, z, F, precision="f64", spacing=None):
    grid = pkg.GD3(x, y, z, spacing=spacing)
    return pkg.SDF3(grid, x, y, z, F, precision=precision)


def ograd(O, x, y, z):
    return O.grid_from_mesh(x, y, z)


def same(a, b):
    """bitwise equality of two float64 fields (NaN-free)."""
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all(a == b))


@pytest.fixture(scope="module")
def oracles(oracle_mod):
    return oracle_mod, oracle_mod.kernels("port"), oracle_mod.kernels("port_crpow")


@pytest.fixture(scope="module")
def config1(pkg, vsl):
    """The reinitialization workload at full size: 64^3 on [-1,1]^3, dx = 2/63."""
    x, y, z = S.cube_grid(64, -1.0, 1.0)
    return x, y, z, S.perturbed_sphere(x, y, z)


def test_set_distance_config1(pkg, oracles, config1):
    O, K, KC = oracles
    x, y, z, F = config1
    m = make(pkg, x, y, z, F)
    m.setDistance()
    for a, b, c in zip(m._dist(), O.set_distance(KC, ograd(O, x, y, z), F).six(),
                       O.set_distance(K, ograd(O, x, y, z), F).six()):
        assert same(host(a), b)
        assert max_rel(host(a), c) <= TOL


@pytest.mark.parametrize("iters", [1, 100])
def test_weno5_reinit_config1(pkg, oracles, config1, iters):
    O, K, KC = oracles
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    m = make(pkg, x, y, z, F)
    m.setDistance()
    got = host(m.WENO5RK3Reinitialization(m.F, iters))
    assert same(got, O.reinit_weno5(KC, g, F, iters, O.set_distance(KC, g, F)))
    assert max_rel(got, O.reinit_weno5(K, g, F, iters, O.set_distance(K, g, F))) <= TOL


@pytest.mark.parametrize("iters", [1, 100])
def test_eno3_reinit_config1(pkg, oracles, config1, iters):
    O, K, KC = oracles
    x, y, z, F = config1
    m = make(pkg, x, y, z, F)
    got = host(m.WENORK3Reinitialization(m.F, iters))
    assert same(got, O.reinit_eno3(KC, ograd(O, x, y, z), F, iters))
    assert max_rel(got, O.reinit_eno3(K, ograd(O, x, y, z), F, iters)) <= TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_loops(pkg, vsl, oracles, name):
    """The reference's own loop outputs (4 reinit / 3 extension pseudo-steps, surface
    redistance 2x2) on the golden inputs, including grids smaller than the stencil."""
    O, K, KC = oracles
    G = load_golden(name)
    r, c, p, dx, dy, dz = G["grid"]
    g = O.Grid(int(r), int(c), int(p), dx, dy, dz)
    x = np.zeros((int(r), int(c), int(p)), order="F")
    F, Cn = O.F64(G["F"]), O.F64(G["C"])
    m = make(pkg, x, x, x, F, spacing=(dx, dy, dz))
    m.setDistance()
    C = dev(Cn)
    dC = O.set_distance(KC, g, F)
    got = host(m.WENO5RK3Reinitialization(m.F, 4))
    assert same(got, O.reinit_weno5(KC, g, F, 4, dC)) and max_rel(got, G["reinit5_it4"]) <= TOL
    got = host(m.WENORK3Reinitialization(m.F, 4))
    assert same(got, O.reinit_eno3(KC, g, F, 4)) and max_rel(got, G["reinit3_it4"]) <= TOL
    got = host(m.WENO5RK3Extend(C, 3))
    assert same(got, O.extend_weno5(KC, g, F, dC, Cn, 3)) and max_rel(got, G["extend5_it3"]) <= TOL
    got = host(m.WENORK3Extend(C, 3))
    assert same(got, O.extend_eno3(KC, g, F, Cn, 3)) and max_rel(got, G["extend3_it3"]) <= TOL
    got = host(m.WENO5RK3ClosetPointSurfaceRedistance(C, 2, 2))
    assert same(got, O.surface_redistance(KC, g, F, Cn, 2, 2))
    assert max_rel(got, G["redistance_2_2"]) <= TOL_REDIST_LIBM
    av = m.area_volume().cpu().numpy()
    assert abs(av[0] - float(G["area"])) <= 1e-12 * max(1.0, abs(float(G["area"])))
    assert abs(av[1] - float(G["volume"])) <= 1e-12 * max(1.0, abs(float(G["volume"])))


@pytest.mark.parametrize("eno3", [False, True])
def test_extend_config1(pkg, oracles, config1, eno3):
    O, K, KC = oracles
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    C = S.surface_field(x, y, z)
    m = make(pkg, x, y, z, F)
    m.setDistance()
    if eno3:
        got = host(m.WENORK3Extend(dev(C), 30))
        assert same(got, O.extend_eno3(KC, g, F, C, 30))
        assert max_rel(got, O.extend_eno3(K, g, F, C, 30)) <= TOL
    else:
        got = host(m.WENO5RK3Extend(dev(C), 30))
        assert same(got, O.extend_weno5(KC, g, F, O.set_distance(KC, g, F), C, 30))
        assert max_rel(got, O.extend_weno5(K, g, F, O.set_distance(K, g, F), C, 30)) <= TOL


@pytest.mark.parametrize("eno3", [False, True])
def test_surface_redistance(pkg, oracles, eno3):
    """WENO5RK3ClosetPointSurfaceRedistance and its WENORK3 form (cubic distances, WENORK3
    normals, crossing values and extension, ENO3 reinitialization)."""
    O, K, KC = oracles
    x, y, z = S.cube_grid(28, -1.0, 1.0)
    F = np.asfortranarray(np.sqrt(x**2 + y**2 + z**2) - 0.6)
    A = np.asfortranarray(np.exp(z) - 1)
    m = make(pkg, x, y, z, F)
    method = m.WENORK3ClosetPointSurfaceRedistance if eno3 else m.WENO5RK3ClosetPointSurfaceRedistance
    got = host(method(dev(A), 3, 6))
    assert same(got, O.surface_redistance(KC, ograd(O, x, y, z), F, A, 3, 6, eno3=eno3))
    assert max_rel(got, O.surface_redistance(K, ograd(O, x, y, z), F, A, 3, 6, eno3=eno3)) <= TOL_REDIST_LIBM


def test_area_volume_and_toolbox(pkg, oracles, config1):
    O, K, KC = oracles
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    m = make(pkg, x, y, z, F)
    tb = O.calculus_toolbox(KC, g, F)
    av = m.area_volume().cpu().numpy()
    # fixed-order tree vs correctly rounded sum: a few ulps of the total
    assert abs(av[0] - O.cal_area(g, F, tb["DiracDelta"])) <= 1e-14 * abs(av[0])
    assert abs(av[1] - O.cal_volume(g, F, tb["Heaviside"])) <= 1e-14 * abs(av[1])
    assert np.array_equal(av, m.area_volume().cpu().numpy())  # bitwise reproducible
    m.GPUsetCalculusToolBox()
    tbl = O.calculus_toolbox(K, g, F)
    for k in O.TOOLBOX_FIELDS:
        assert same(host(getattr(m, k)), tb[k]), k
        assert max_rel(host(getattr(m, k)), tbl[k]) <= TOL, k


def test_advection_rk3(pkg, oracles, config1):
    O, K, KC = oracles
    x, y, z, F = config1
    g = ograd(O, x, y, z)
    vx = np.asfortranarray(-y + 0.3 * np.sin(2 * z))
    vy = np.asfortranarray(x.copy())
    vz = np.asfortranarray(0.5 * np.cos(3 * x) * y)
    dt = 0.5 * g.ds / 1.5
    m = make(pkg, x, y, z, F)
    got = host(m.WENO5RK3Advection(m.F, dev(vx), dev(vy), dev(vz), dt, steps=3))
    assert same(got, O.advect_rk3(KC, g, F, vx, vy, vz, dt, steps=3))


def test_vesicle_step(pkg, oracles):
    """The composite step (toolbox -> extension 30 -> dt -> advection -> setDistance ->
    reinit 20) on the noisy oblate vesicle at 48^3, three steps."""
    O, K, KC = oracles
    x, y, z = S.cube_grid(48, -1.5, 1.5)
    F = S.noisy_oblate(x, y, z, seed=3)
    g = ograd(O, x, y, z)
    m = make(pkg, x, y, z, F)
    m.setDistance()
    Fo, do = F, O.set_distance(KC, g, F)
    for _ in range(3):
        info = m.vesicle_step(30, 20, 0.5).cpu().numpy()
        Fo, do, oi = O.vesicle_step(KC, g, Fo, do, 30, 20, 0.5)
        assert abs(info[0] - oi["area"]) <= 1e-14 * oi["area"]
        assert abs(info[1] - oi["volume"]) <= 1e-14 * oi["volume"]
        assert info[2] == oi["dt"] and info[3] == oi["vmax"]
        assert same(host(m.F), Fo)
        for a, b in zip(m._dist(), do.six()):
            assert same(host(a), b)


def test_deterministic(pkg, config1):
    x, y, z, F = config1
    m = make(pkg, x, y, z, F)
    m.setDistance()
    a = m.WENO5RK3Reinitialization(m.F, 5)
    b = m.WENO5RK3Reinitialization(m.F, 5)
    assert torch.equal(a, b)
