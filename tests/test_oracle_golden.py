"""The oracle (C restatement) against the golden fixtures made by the reference's own
kernels compiled for the host (tests/golden/gen_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

DIRS = ("xpr", "xpl", "ypf", "ypb", "zpu", "zpd")
CROSS = ("cpr", "cpl", "cpf", "cpb", "cpu", "cpd")

# The restatement keeps the reference's operation order; on the machine that made the
# fixtures it is bit-exact, elsewhere (another libm) it agrees to a few ulps.
RTOL = 1e-13


def close(a, b, scale=None):
    a = np.asarray(a)
    b = np.asarray(b)
    s = scale if scale is not None else max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    err = float(np.max(np.abs(a - b))) if a.size else 0.0
    assert err <= RTOL * s, f"max |diff| {err:.3e} > {RTOL * s:.3e}"


def setup(O, G):
    r, c, p, dx, dy, dz = G["grid"]
    g = O.Grid(int(r), int(c), int(p), float(dx), float(dy), float(dz))
    return g, O.F64(G["F"]), O.F64(G["C"])


@pytest.fixture(scope="module", params=GOLDEN_CASES)
def case(request, oracle_mod):
    return request.param, load_golden(request.param), oracle_mod


def test_distances(case):
    name, G, O = case
    K = O.kernels("port")
    g, F, _ = setup(O, G)
    d5 = O.set_distance(K, g, F)
    d3 = O.set_distance(K, g, F, cubic=True)
    for nm, a, b in zip(DIRS, d5.six(), d3.six()):
        close(a, G["dist5_" + nm])
        close(b, G["dist3_" + nm])


def test_re_step_single_stage(case):
    name, G, O = case
    K = O.kernels("port")
    g, F, _ = setup(O, G)
    mask = np.asfortranarray(F < 0)
    d5 = O.Distances(*[O.F64(G["dist5_" + n]) for n in DIRS])
    d3 = O.Distances(*[O.F64(G["dist3_" + n]) for n in DIRS])
    step = O.zeros(g)
    K.re_step(step, F, mask, O.F64(0.3 * d5.min_dist), *d5.six(), *g.args(), g.num_ele)
    close(step, G["re_step5"])
    K.re_step_eno3(step, F, mask, O.F64(0.3 * d3.min_dist), *d3.six(), *g.args(), g.num_ele)
    close(step, G["re_step3"])


def test_reinit_loops(case):
    name, G, O = case
    K = O.kernels("port")
    g, F, _ = setup(O, G)
    d5 = O.set_distance(K, g, F)
    close(O.reinit_weno5(K, g, F, 4, d5), G["reinit5_it4"])
    close(O.reinit_eno3(K, g, F, 4), G["reinit3_it4"])


def test_normals_crossings_extension(case):
    name, G, O = case
    K = O.kernels("port")
    g, F, C = setup(O, G)
    for tag, e3 in (("5", False), ("3", True)):
        d = O.set_distance(K, g, F, cubic=e3)
        n = [O.zeros(g) for _ in range(3)]
        (K.upwind_normal_eno3 if e3 else K.upwind_normal)(*n, F, *d.six(), *g.args(), g.num_ele)
        for ax, a in zip("xyz", n):
            close(a, G[f"normal{tag}_{ax}"])
        for nm, a in zip(CROSS, O.crossing_values(K, g, C, d, eno3=e3)):
            close(a, G[f"cross{tag}_{nm}"])
    d5 = O.set_distance(K, g, F)
    close(O.extend_weno5(K, g, F, d5, C, 3), G["extend5_it3"])
    close(O.extend_eno3(K, g, F, C, 3), G["extend3_it3"])


def test_toolbox_advection_derivatives(case):
    name, G, O = case
    K = O.kernels("port")
    g, F, _ = setup(O, G)
    tb = O.calculus_toolbox(K, g, F)
    for k in O.TOOLBOX_FIELDS:
        close(tb[k], G["tb_" + k])
    v = [O.F64(G["v" + ax]) for ax in "xyz"]
    close(O.weno_dot_grad(K, g, *v, F), G["advection_step"])
    wd = [O.zeros(g) for _ in range(6)]
    K.weno_derivative(*wd, F, *g.args())
    for nm, a in zip(("back_x", "fore_x", "back_y", "fore_y", "back_z", "fore_z"), wd):
        close(a, G["wd_" + nm])
    assert abs(O.cal_area(g, F, tb["DiracDelta"]) - float(G["area"])) <= 1e-13 * max(1.0, abs(float(G["area"])))
    assert abs(O.cal_volume(g, F, tb["Heaviside"]) - float(G["volume"])) <= 1e-13 * max(1.0, abs(float(G["volume"])))


def test_surface_redistance(case):
    name, G, O = case
    K = O.kernels("port")
    g, F, C = setup(O, G)
    close(O.surface_redistance(K, g, F, C, 2, 2), G["redistance_2_2"])


def test_enork2(case):
    """ENORK2 (second-order ENO with the sub-cell fix, Heun RK2): distances, one re_step,
    upwind normals, crossing values, and the reinitialization and extension loops."""
    name, G, O = case
    K = O.kernels("port")
    g, F, C = setup(O, G)
    d2 = O.set_distance_enork2(K, g, F)
    for nm, a in zip(DIRS, d2.six()):
        close(a, G["dist2_" + nm])
    step = O.zeros(g)
    K.enork2_re_step(step, F, np.asfortranarray(F < 0), O.F64(0.3 * d2.min_dist), *d2.six(), *g.args(), g.num_ele)
    close(step, G["re_step2"])
    n = [O.zeros(g) for _ in range(3)]
    K.enork2_upwind_normal(*n, F, *d2.six(), *g.args(), g.num_ele)
    for ax, a in zip("xyz", n):
        close(a, G[f"normal2_{ax}"])
    cp = [O.zeros(g) for _ in range(6)]
    K.enork2_boundary_interpolate(*cp, *d2.six(), C, *g.args(), g.num_ele)
    for nm, a in zip(CROSS, cp):
        close(a, G[f"cross2_{nm}"])
    close(O.reinit_enork2(K, g, F, 4), G["reinit2_it4"])
    close(O.extend_enork2(K, g, F, C, 3), G["extend2_it3"])
    close(O.surface_redistance_enork2(K, g, F, C, 2, 2), G["redistance2_2_2"])
