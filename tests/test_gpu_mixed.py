"""Mixed-precision form (FP32 fields and stencils, FP64 interface roots and reductions)
against the FP64 oracle.  Tolerances, written per test:

* reinitialization: max error over the interface band |phi| < 3dx below 1e-5*dx (the
  target of the mixed form), after 1, 20 and 100 pseudo-steps at the full 64^3 size;
* extension and advection (fields of arbitrary scale): max error below 5e-5 of the
  field's scale, i.e. a few hundred FP32 ulps after 30 pseudo-steps;
* area and volume: relative error below 1e-8 (FP64 terms on the promoted FP32 values,
  against the oracle's correctly rounded sums); the composite step at most 1e-5 dx over
  the band, 1e-8 on area and volume.

GPU only; everything goes through the C ABI."""
import importlib

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from gpu_util import dev, host

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")


def band_err(a, ref, phi, dx, width=3):
    m = np.abs(phi) < width * dx
    return float(np.max(np.abs(a[m] - ref[m]))) / dx


def rel_err(a, ref):
    return float(np.max(np.abs(a - ref))) / max(1.0, float(np.max(np.abs(ref))))


@pytest.fixture(scope="module")
def config1(pkg, vsl, oracle_mod):
    O = oracle_mod
    x, y, z = S.cube_grid(64, -1.0, 1.0)
    F = S.perturbed_sphere(x, y, z)
    g = O.grid_from_mesh(x, y, z)
    return x, y, z, F, g, O.kernels("port")


def f32(pkg, x, y, z, F):
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    m.setDistance()
    return m


@pytest.mark.parametrize("iters", [1, 20, 100])
def test_reinit_weno5_band_error(pkg, oracle_mod, config1, iters):
    O = oracle_mod
    x, y, z, F, g, K = config1
    ref = O.reinit_weno5(K, g, F, iters, O.set_distance(K, g, F))
    m = f32(pkg, x, y, z, F)
    got = host(m.WENO5RK3Reinitialization(m.F, iters))
    assert band_err(got, ref, ref, g.dx) <= 1e-5
    assert rel_err(got, ref) <= 5e-5


def test_reinit_eno3_band_error(pkg, oracle_mod, config1):
    O = oracle_mod
    x, y, z, F, g, K = config1
    ref = O.reinit_eno3(K, g, F, 100)
    m = f32(pkg, x, y, z, F)
    got = host(m.WENORK3Reinitialization(m.F, 100))
    assert band_err(got, ref, ref, g.dx) <= 1e-5


@pytest.mark.parametrize("eno3", [False, True])
def test_extend(pkg, oracle_mod, config1, eno3):
    O = oracle_mod
    x, y, z, F, g, K = config1
    C = S.surface_field(x, y, z)
    m = f32(pkg, x, y, z, F)
    if eno3:
        ref = O.extend_eno3(K, g, F, C, 30)
        got = host(m.WENORK3Extend(dev(C), 30))
    else:
        ref = O.extend_weno5(K, g, F, O.set_distance(K, g, F), C, 30)
        got = host(m.WENO5RK3Extend(dev(C), 30))
    assert rel_err(got, ref) <= 5e-5


def test_advection(pkg, oracle_mod, config1):
    O = oracle_mod
    x, y, z, F, g, K = config1
    vx = np.asfortranarray(-y + 0.3 * np.sin(2 * z))
    vy = np.asfortranarray(x.copy())
    vz = np.asfortranarray(0.5 * np.cos(3 * x) * y)
    dt = 0.5 * g.ds / 1.5
    ref = O.advect_rk3(K, g, F, vx, vy, vz, dt, steps=3)
    m = f32(pkg, x, y, z, F)
    got = host(m.WENO5RK3Advection(m.F, dev(vx), dev(vy), dev(vz), dt, steps=3))
    assert rel_err(got, ref) <= 5e-5


def test_area_volume(pkg, oracle_mod, config1):
    O = oracle_mod
    x, y, z, F, g, K = config1
    tb = O.calculus_toolbox(K, g, F)
    m = f32(pkg, x, y, z, F)
    av = m.area_volume().cpu().numpy()
    a, v = O.cal_area(g, F, tb["DiracDelta"]), O.cal_volume(g, F, tb["Heaviside"])
    assert abs(av[0] - a) <= 1e-8 * a
    assert abs(av[1] - v) <= 1e-8 * v


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_cases_fp32(pkg, vsl, name):
    """The reference's own outputs on the golden inputs (kinks, nodes on the interface,
    grids smaller than the stencil), within FP32 tolerance.

    The merged-spheres input is mirror-symmetric about x = 0.  On the symmetry plane the
    reference's upwind normal (upwind_normal.cu:10) picks the forward derivative only if
    |phi(+1)| < |phi(-1)|; the two values agree to within an ulp in FP64 and are equal
    once rounded to FP32, so the FP32 form takes the other one-sided derivative of the
    kink, of opposite sign.  That case is checked for the reinitialization only."""
    G = load_golden(name)
    r, c, p, dx, dy, dz = G["grid"]
    x = np.zeros((int(r), int(c), int(p)), order="F")
    m = pkg.SDF3(pkg.GD3(x, x, x, spacing=(dx, dy, dz)), Val=G["F"], precision="f32")
    m.setDistance()
    C = dev(G["C"])
    assert rel_err(host(m.WENO5RK3Reinitialization(m.F, 4)), G["reinit5_it4"]) <= 5e-5
    assert rel_err(host(m.WENORK3Reinitialization(m.F, 4)), G["reinit3_it4"]) <= 5e-5
    if name == "merge15":
        return
    assert rel_err(host(m.WENO5RK3Extend(C, 3)), G["extend5_it3"]) <= 5e-5
    assert rel_err(host(m.WENORK3Extend(C, 3)), G["extend3_it3"]) <= 5e-5


@pytest.mark.parametrize("eno3", [False, True])
def test_surface_redistance(pkg, oracle_mod, eno3):
    O = oracle_mod
    x, y, z = S.cube_grid(28, -1.0, 1.0)
    F = np.asfortranarray(np.sqrt(x**2 + y**2 + z**2) - 0.6)
    A = np.asfortranarray(np.exp(z) - 1)
    m = f32(pkg, x, y, z, F)
    method = m.WENORK3ClosetPointSurfaceRedistance if eno3 else m.WENO5RK3ClosetPointSurfaceRedistance
    got = host(method(dev(A), 3, 6))
    ref = O.surface_redistance(O.kernels("port"), O.grid_from_mesh(x, y, z), F, A, 3, 6, eno3=eno3)
    assert rel_err(got, ref) <= 5e-5


def test_vesicle_steps(pkg, oracle_mod):
    """The composite step, one step at a time from the FP64 oracle's state (field and its
    cached distances rounded to FP32), three steps of the noisy oblate vesicle at 48^3.

    Per step: interface-band error at most 1e-5*dx at the worst node and 1e-6*dx RMS, area
    and volume within 1e-8, dt within 1e-6 (the tolerances of the mixed form).  Consecutive
    FP32 steps are not compared with consecutive FP64 steps: the two trajectories drift
    apart through dt."""
    O = oracle_mod
    x, y, z = S.cube_grid(48, -1.5, 1.5)
    F = S.noisy_oblate(x, y, z, seed=3)
    g = O.grid_from_mesh(x, y, z)
    K = O.kernels("port")
    Fo, do = F, O.set_distance(K, g, F)
    for _ in range(3):
        m = f32(pkg, x, y, z, Fo)
        for t, a in zip(m._dist(), do.six()):
            t.copy_(dev(a, t.dtype))
        info = m.vesicle_step(30, 20, 0.5).cpu().numpy()
        Fn, dn, oi = O.vesicle_step(K, g, Fo, do, 30, 20, 0.5)
        got = host(m.F)
        band = np.abs(Fn) < 3 * g.dx
        e = np.abs(got[band] - Fn[band]) / g.dx
        da, dv, ddt = abs(info[0] / oi["area"] - 1), abs(info[1] / oi["volume"] - 1), abs(info[2] / oi["dt"] - 1)
        print(f"\nstep: band max {e.max():.2e} dx, rms {np.sqrt(np.mean(e**2)):.2e} dx, area {da:.1e}, "
              f"volume {dv:.1e}, dt {ddt:.1e}")
        assert da <= 1e-8 and dv <= 1e-8 and ddt <= 1e-6
        assert e.max() <= 1e-5 and np.sqrt(np.mean(e**2)) <= 1e-6
        Fo, do = Fn, dn


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_vesicle_step_graph_replay(pkg, precision):
    """The CUDA-graph replay of a vesicle step gives bitwise the result of direct launches."""
    x, y, z = S.cube_grid(40, -1.5, 1.5)
    F = S.noisy_oblate(x, y, z, seed=5)
    runs = []
    for graph in (False, True):
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision=precision)
        m.setDistance()
        infos = [m.vesicle_step(10, 6, 0.5, graph=graph).cpu().numpy().copy() for _ in range(3)]
        runs.append((host(m.F), infos))
    assert np.array_equal(runs[0][0], runs[1][0])
    for a, b in zip(runs[0][1], runs[1][1]):
        assert np.array_equal(a, b)
