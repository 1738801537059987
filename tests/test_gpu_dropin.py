"""Parity of the FP64 drop-in kernels (reference argument order, in/out semantics) with
the golden fixtures of the reference's own kernels and with the oracle.  GPU only; calls
go through the C ABI."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from gpu_util import dev, empty, host, max_rel, ptr, stream

pytestmark = pytest.mark.gpu

DIRS = ("xpr", "xpl", "ypf", "ypb", "zpu", "zpd")
CROSS = ("cpr", "cpl", "cpf", "cpb", "cpu", "cpd")
TOL = 1e-12  # plain FP64 form: relative to the field's scale, per grid value


@pytest.fixture(scope="module", params=GOLDEN_CASES)
def case(request, vsl):
    G = load_golden(request.param)
    r, c, p, dx, dy, dz = G["grid"]
    return G, (int(r), int(c), int(p)), (float(dx), float(dy), float(dz)), vsl


def test_boundary_location_inout_semantics(case):
    G, shape, h, vsl = case
    n = shape[0] * shape[1] * shape[2]
    F = dev(G["F"])
    for fn, tag in (("vsl_boundary_location", "dist5_"), ("vsl_cubic_boundary_correction", "dist3_")):
        # caller-initialised to the spacing (setDistance.m:5-10): equals the reference output
        d = [empty(shape, fill=h[q // 2]) for q in range(6)]
        vsl.call(fn, *map(ptr, d), ptr(F), n, *shape, *h, stream())
        for q, nm in enumerate(DIRS):
            assert max_rel(host(d[q]), G[tag + nm]) <= TOL, (fn, nm)
        # entries the kernel does not write keep whatever the caller put there
        d2 = [empty(shape, fill=-7.0) for _ in range(6)]
        vsl.call(fn, *map(ptr, d2), ptr(F), n, *shape, *h, stream())
        for q, nm in enumerate(DIRS):
            ref, got = G[tag + nm], host(d2[q])
            written = got != -7.0
            assert max_rel(got[written], ref[written], scale=1.0) <= TOL
            assert np.all(written[ref != h[q // 2]])


def test_re_step(case):
    G, shape, h, vsl = case
    n = shape[0] * shape[1] * shape[2]
    F = dev(G["F"])
    mask = dev(G["F"] < 0)
    for fn, tag, out in (("vsl_re_step", "dist5_", "re_step5"), ("vsl_re_step_eno3", "dist3_", "re_step3")):
        d = [dev(G[tag + nm]) for nm in DIRS]
        md = np.minimum(np.minimum(G[tag + "xpr"], G[tag + "xpl"]),
                        np.minimum(np.minimum(G[tag + "ypf"], G[tag + "ypb"]), np.minimum(G[tag + "zpu"], G[tag + "zpd"])))
        dt = dev(0.3 * md)
        step = empty(shape, fill=np.nan)
        vsl.call(fn, ptr(step), ptr(F), ptr(mask), ptr(dt), *map(ptr, d), *shape, *h, n, stream())
        assert max_rel(host(step), G[out], scale=max(1e-300, float(np.max(np.abs(G[out]))))) <= 1e-11, fn


def test_normals_crossings_extend_step(case, oracle_mod):
    G, shape, h, vsl = case
    n = shape[0] * shape[1] * shape[2]
    O = oracle_mod
    F, C = dev(G["F"]), dev(G["C"])
    for e3, tag in ((False, "5"), (True, "3")):
        d = [dev(G[f"dist{tag}_" + nm]) for nm in DIRS]
        nrm = [empty(shape, fill=np.nan) for _ in range(3)]
        vsl.call("vsl_upwind_normal_eno3" if e3 else "vsl_upwind_normal", *map(ptr, nrm), ptr(F), *map(ptr, d), *shape,
                 *h, n, stream())
        for a, ax in zip(nrm, "xyz"):
            assert max_rel(host(a), G[f"normal{tag}_{ax}"]) <= TOL
        cp = [empty(shape, fill=np.nan) for _ in range(6)]
        vsl.call("vsl_boundary_interpolate_eno3" if e3 else "vsl_boundary_interpolant", *map(ptr, cp), *map(ptr, d),
                 ptr(C), *shape, *h, n, stream())
        for a, nm in zip(cp, CROSS):
            assert max_rel(host(a), G[f"cross{tag}_{nm}"]) <= TOL
        # one extend_step with the oracle's velocity, against the oracle's kernel
        g = O.Grid(*shape, *h)
        K = O.kernels("port")
        dd = O.Distances(*[O.F64(G[f"dist{tag}_" + nm]) for nm in DIRS])
        v = O.extension_velocity(K, g, O.F64(G["F"]), dd, eno3=e3)
        cpo = O.crossing_values(K, g, O.F64(G["C"]), dd, eno3=e3)
        dt = O.F64(0.3 * dd.min_dist)
        ref = O.zeros(g)
        (K.extend_step_eno3 if e3 else K.extend_step)(ref, dt, O.F64(G["C"]), *v, *dd.six(), *cpo, *g.args(), g.num_ele)
        step = empty(shape, fill=np.nan)
        dt_d, v_d, cp_d = dev(dt), [dev(a) for a in v], [dev(a) for a in cpo]  # kept alive across the call
        vsl.call("vsl_extend_step_eno3" if e3 else "vsl_extend_step", ptr(step), ptr(dt_d), ptr(C),
                 *map(ptr, v_d), *map(ptr, d), *map(ptr, cp_d), *shape, *h, n, stream())
        assert max_rel(host(step), ref, scale=max(1e-300, float(np.max(np.abs(ref))))) <= 1e-11


def test_toolbox_advection_weno_derivative(case):
    G, shape, h, vsl = case
    n = shape[0] * shape[1] * shape[2]
    F = dev(G["F"])
    hp = dev(np.maximum(G["F"], 0))
    outs = [empty(shape, fill=np.nan) for _ in range(18)]
    ds = sum(h) / 3
    vsl.call("vsl_set_calculus_toolbox", *map(ptr, outs), ptr(F), ptr(hp), *shape, *h, ds, n, stream())
    from oracle.oracle import TOOLBOX_FIELDS

    for a, nm in zip(outs, TOOLBOX_FIELDS):
        assert max_rel(host(a), G["tb_" + nm]) <= TOL, nm
    v = [dev(G["v" + ax]) for ax in "xyz"]
    out = empty(shape, fill=np.nan)
    vsl.call("vsl_advection_step", ptr(out), *map(ptr, v), ptr(F), *shape, *h, stream())
    assert max_rel(host(out), G["advection_step"]) <= TOL
    wd = [empty(shape, fill=np.nan) for _ in range(6)]
    vsl.call("vsl_weno_derivative", *map(ptr, wd), ptr(F), *shape, *h, stream())
    for a, nm in zip(wd, ("back_x", "fore_x", "back_y", "fore_y", "back_z", "fore_z")):
        assert max_rel(host(a), G["wd_" + nm]) <= TOL
