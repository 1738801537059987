"""ENORK2 (second-order ENO with the sub-cell fix, Heun RK2; the reference's
CUDA_Code/1_0_ENORK2_Reinitialization and 2_0_ENORK2_Extend with the drivers
ENORK2Reinitialization.m / ENORK2Extend.m) on the GPU.

* FP64 drop-in kernels against the golden fixtures of the reference's own kernels
  (1e-12 relative per grid value);
* the fused FP64 methods (reinitialization, extension, closest-point surface
  redistance) bit-identical to the oracle built with integer powers rounded once, and
  within 1e-12 of the golden loop outputs and of the oracle with libm's pow (1e-10 for
  the redistance, whose 1e-14 normal floor amplifies one-ulp pow differences);
* the FP32 form against the FP64 oracle: reinitialization within 1e-5 dx over the band
  |phi| < 3 dx, extension within 5e-5 relative to the field's scale.
GPU only; calls go through the C ABI."""
import importlib

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from gpu_util import dev, empty, host, max_rel, ptr, stream

pytestmark = pytest.mark.gpu

DIRS = ("xpr", "xpl", "ypf", "ypb", "zpu", "zpd")
CROSS = ("cpr", "cpl", "cpf", "cpb", "cpu", "cpd")
TOL = 1e-12
S = importlib.import_module("2018_7_vesicle_gb300.shapes")


@pytest.fixture(scope="module", params=GOLDEN_CASES)
def golden(request, vsl):
    G = load_golden(request.param)
    r, c, p, dx, dy, dz = G["grid"]
    return request.param, G, (int(r), int(c), int(p)), (float(dx), float(dy), float(dz))


def test_dropin_kernels(golden, vsl, oracle_mod):
    name, G, shape, h = golden
    n = shape[0] * shape[1] * shape[2]
    F, C = dev(G["F"]), dev(G["C"])
    # boundary_correction on spacing-filled arrays (ENORK2Reinitialization.m:10-19)
    d = [empty(shape, fill=h[q // 2]) for q in range(6)]
    vsl.call("vsl_enork2_boundary_correction", *map(ptr, d), ptr(F), n, *shape, *h, stream())
    for q, nm in enumerate(DIRS):
        assert max_rel(host(d[q]), G["dist2_" + nm]) <= TOL, nm
    md = np.minimum(np.minimum(G["dist2_xpr"], G["dist2_xpl"]),
                    np.minimum(np.minimum(G["dist2_ypf"], G["dist2_ypb"]), np.minimum(G["dist2_zpu"], G["dist2_zpd"])))
    step = empty(shape, fill=np.nan)
    mask, dt_d = dev(G["F"] < 0), dev(0.3 * md)  # kept alive until the kernel has run
    vsl.call("vsl_enork2_re_step", ptr(step), ptr(F), ptr(mask), ptr(dt_d), *map(ptr, d), *shape, *h, n, stream())
    assert max_rel(host(step), G["re_step2"], scale=max(1e-300, float(np.abs(G["re_step2"]).max()))) <= 1e-11
    nrm = [empty(shape, fill=np.nan) for _ in range(3)]
    vsl.call("vsl_enork2_upwind_normal", *map(ptr, nrm), ptr(F), *map(ptr, d), *shape, *h, n, stream())
    for a, ax in zip(nrm, "xyz"):
        assert max_rel(host(a), G[f"normal2_{ax}"]) <= TOL
    cp = [empty(shape, fill=np.nan) for _ in range(6)]
    vsl.call("vsl_enork2_boundary_interpolate", *map(ptr, cp), *map(ptr, d), ptr(C), *shape, *h, n, stream())
    for a, nm in zip(cp, CROSS):
        assert max_rel(host(a), G[f"cross2_{nm}"]) <= TOL
    # one extend_step with the oracle's velocity, against the oracle's kernel
    O = oracle_mod
    K = O.kernels("port")
    g = O.Grid(*shape, *h)
    dd = O.Distances(*[O.F64(G["dist2_" + nm]) for nm in DIRS])
    v = O.extension_velocity(K, g, O.F64(G["F"]), dd, enork2=True)
    dt = O.F64(0.3 * md)
    ref = O.zeros(g)
    K.enork2_extend_step(ref, dt, O.F64(G["C"]), *v, *dd.six(), *[O.F64(G[f"cross2_{nm}"]) for nm in CROSS],
                         *g.args(), g.num_ele)
    got = empty(shape, fill=np.nan)
    dt_g, v_g = dev(dt), [dev(a) for a in v]
    vsl.call("vsl_enork2_extend_step", ptr(got), ptr(dt_g), ptr(C), *map(ptr, v_g), *map(ptr, d), *map(ptr, cp),
             *shape, *h, n, stream())
    assert max_rel(host(got), ref, scale=max(1e-300, float(np.abs(ref).max()))) <= 1e-11


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all(a == b))


def test_golden_loops(golden, pkg, oracle_mod):
    name, G, shape, h = golden
    O = oracle_mod
    K, KC = O.kernels("port"), O.kernels("port_crpow")
    g = O.Grid(*shape, *h)
    F, Cn = O.F64(G["F"]), O.F64(G["C"])
    x = np.zeros(shape, order="F")
    m = pkg.SDF3(pkg.GD3(x, x, x, spacing=h), Val=F, precision="f64")
    got = host(m.ENORK2Reinitialization(m.F, 4))
    assert same(got, O.reinit_enork2(KC, g, F, 4))
    assert max_rel(got, G["reinit2_it4"]) <= TOL and max_rel(got, O.reinit_enork2(K, g, F, 4)) <= TOL
    got = host(m.ENORK2Extend(dev(Cn), 3))
    assert same(got, O.extend_enork2(KC, g, F, Cn, 3))
    assert max_rel(got, G["extend2_it3"]) <= TOL and max_rel(got, O.extend_enork2(K, g, F, Cn, 3)) <= TOL
    got = host(m.ENORK2ClosetPointSurfaceRedistance(dev(Cn), 2, 2))
    assert same(got, O.surface_redistance_enork2(KC, g, F, Cn, 2, 2))
    # the 1e-14 normal floor amplifies one-ulp differences of libm's pow (see test_gpu_methods)
    assert max_rel(got, G["redistance2_2_2"]) <= 1e-10


@pytest.fixture(scope="module")
def config1(pkg, vsl):
    x, y, z = S.cube_grid(64, -1.0, 1.0)
    return x, y, z, S.perturbed_sphere(x, y, z)


def test_config1_fp64(pkg, oracle_mod, config1):
    """64^3 non-distance sphere: 100 reinitialization and 30 extension pseudo-steps."""
    O = oracle_mod
    KC = O.kernels("port_crpow")
    x, y, z, F = config1
    g = O.grid_from_mesh(x, y, z)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f64")
    assert same(host(m.ENORK2Reinitialization(m.F, 100)), O.reinit_enork2(KC, g, F, 100))
    C = S.surface_field(x, y, z)
    assert same(host(m.ENORK2Extend(dev(C), 30)), O.extend_enork2(KC, g, F, C, 30))


def test_config1_fp32(pkg, oracle_mod, config1):
    O = oracle_mod
    K = O.kernels("port")
    x, y, z, F = config1
    g = O.grid_from_mesh(x, y, z)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    band = np.abs(F) < 3 * g.dx
    ref = O.reinit_enork2(K, g, F, 100)
    got = host(m.ENORK2Reinitialization(m.F, 100))
    err = np.abs(got - ref)[band].max() / g.dx
    print("ENORK2 FP32 reinit band error / dx", err)
    assert err <= 1e-5
    C = S.surface_field(x, y, z)
    ref = O.extend_enork2(K, g, F, C, 30)
    got = host(m.ENORK2Extend(dev(C), 30))
    rel = max_rel(got, ref)
    print("ENORK2 FP32 extension rel error", rel)
    assert rel <= 5e-5


def test_fp32_extension_ragged_tiles(pkg, oracle_mod):
    """FP32 ENORK2 extension on a grid with partial tiles in every axis (37 rows, 29
    columns, 11 pages: 32 x 8 tiles and fewer pages than a block marches): tiled uniform
    nodes and the flagged list together, against the oracle."""
    O = oracle_mod
    K = O.kernels("port")
    x, y, z = S.meshgrid(np.linspace(-1, 1, 29), np.linspace(-0.95, 0.95, 37), np.linspace(-0.7, 0.7, 11))
    F = S.perturbed_sphere(x, y, z, r=0.55, centre=(0.1, -0.05, 0.02))
    g = O.grid_from_mesh(x, y, z)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    C = S.surface_field(x, y, z)
    ref = O.extend_enork2(K, g, F, C, 20)
    got = host(m.ENORK2Extend(dev(C), 20))
    rel = max_rel(got, ref)
    print("ENORK2 FP32 extension (ragged tiles) rel error", rel)
    assert rel <= 5e-5


def test_fp32_reinitialization_ragged_tiles(pkg, oracle_mod):
    """FP32 ENORK2 reinitialization on the ragged grid: tiled uniform nodes and the flagged
    list together, within 1e-5 dx of the oracle over the band |phi| < 3 dx."""
    O = oracle_mod
    K = O.kernels("port")
    x, y, z = S.meshgrid(np.linspace(-1, 1, 29), np.linspace(-0.95, 0.95, 37), np.linspace(-0.7, 0.7, 11))
    F = S.perturbed_sphere(x, y, z, r=0.55, centre=(0.1, -0.05, 0.02))
    g = O.grid_from_mesh(x, y, z)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    ref = O.reinit_enork2(K, g, F, 30)
    got = host(m.ENORK2Reinitialization(m.F, 30))
    h = min(g.dx, g.dy, g.dz)
    band = np.abs(ref) < 3 * h
    err = np.abs(got - ref)[band].max() / h
    print("ENORK2 FP32 reinitialization (ragged tiles) band error / dx", err)
    assert err <= 1e-5
