"""Generate the golden fixtures of the level-set hot path from the reference's own kernels.

The reference's CUDA kernel files are compiled for the host by ``oracle/ref/Makefile``
(``oracle/_ref/libvsl_ref.so``); this script runs them, with the MATLAB glue restated in
``oracle/oracle.py``, on seeded inputs and writes ``golden_<case>.npz`` beside itself.
It needs the reference checkout, so it runs in the development container only; the
fixtures it writes are committed and read by the tests everywhere.

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402
from oracle import oracle as O  # noqa: E402

PEAR = os.path.join(build_oracle.reference_vesicle(), "pear.mat")


def reference_digest() -> str:
    h = hashlib.sha256()
    base = build_oracle.reference_kernels()
    for sub in sorted(os.listdir(base)):
        d = os.path.join(base, sub)
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".hpp", ".cuh", ".cup")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode())
                    h.update(fh.read())
    return h.hexdigest()


def cases():
    """(name, x, y, z, F, C): seeded inputs in MATLAB meshgrid layout."""
    out = []
    # config-1 family: non-distance sphere on [-1,1]^3 (uniform spacing)
    n = 14
    xv = np.linspace(-1, 1, n)
    x, y, z = O.meshgrid(xv, xv, xv)
    F = (np.sqrt(x**2 + y**2 + z**2) - 0.6) * (0.1 + (x - 0.35) ** 2 + (y - 0.35) ** 2 + (z - 0.35) ** 2)
    C = np.sin(3 * x) * np.cos(2 * y) + 0.5 * z**2
    out.append(("sphere14", x, y, z, F, C))
    # anisotropic box: rows != cols != pges and dx != dy != dz (catches axis mix-ups)
    xv = np.linspace(-1.0, 1.0, 13)
    yv = np.linspace(-0.8, 0.9, 11)
    zv = np.linspace(-1.1, 1.0, 9)
    x, y, z = O.meshgrid(xv, yv, zv)
    F = np.sqrt(x**2 / 0.7**2 + y**2 / 0.6**2 + z**2 / 0.45**2) - 1
    rng = np.random.default_rng(7)
    C = np.exp(z) - 1 + 0.1 * rng.standard_normal(x.shape)
    out.append(("aniso", x, y, z, F, C))
    # two merging spheres: kinks where the fronts meet (nodes exactly on the interface too)
    xv = np.linspace(-1, 1, 15)
    x, y, z = O.meshgrid(xv, xv, xv)
    F = np.minimum(np.sqrt((x - 0.3) ** 2 + y**2 + z**2) - 0.4, np.sqrt((x + 0.3) ** 2 + y**2 + z**2) - 0.4)
    F[np.abs(F) < 0.02] = 0.0
    C = x * y + z
    out.append(("merge15", x, y, z, F, C))
    # tiny grids smaller than the 7-point stencil, and a single page
    xv = np.linspace(-1, 1, 4)
    x, y, z = O.meshgrid(xv, xv, np.linspace(-1, 1, 3))
    F = x**2 + y**2 + z**2 - 0.5
    out.append(("tiny", x, y, z, F, x + 2 * y))
    x, y, z = O.meshgrid(np.linspace(-1, 1, 9), np.linspace(-1, 1, 8), np.array([0.0, 0.1]))
    F = np.sqrt(x**2 + y**2) - 0.5
    out.append(("slab", x, y, z, F, np.cos(x) * y))
    # the reference's shipped 64^3 input field (V/pear.mat), a 14^3 window across the surface
    if os.path.exists(PEAR):
        import scipy.io

        Fp = scipy.io.loadmat(PEAR)["F"]
        xv = np.linspace(-1, 1, 64)
        x, y, z = O.meshgrid(xv, xv, xv)
        sl = (slice(25, 39), slice(8, 22), slice(25, 39))
        out.append(("pear14", x[sl], y[sl], z[sl], Fp[sl], np.sin(2 * x[sl]) + y[sl]))
    return out


def run_case(K, name, x, y, z, F, C):
    g = O.grid_from_mesh(x, y, z)
    F = O.F64(F)
    C = O.F64(C)
    rec = {"grid": np.array([g.rows, g.cols, g.pges, g.dx, g.dy, g.dz]), "F": F, "C": C}
    d5 = O.set_distance(K, g, F)
    d3 = O.set_distance(K, g, F, cubic=True)
    for nm, a in zip(("xpr", "xpl", "ypf", "ypb", "zpu", "zpd"), d5.six()):
        rec["dist5_" + nm] = a
    for nm, a in zip(("xpr", "xpl", "ypf", "ypb", "zpu", "zpd"), d3.six()):
        rec["dist3_" + nm] = a
    mask = np.asfortranarray(F < 0)
    deltat = O.F64(0.3 * d5.min_dist)
    step = O.zeros(g)
    K.re_step(step, F, mask, deltat, *d5.six(), *g.args(), g.num_ele)
    rec["re_step5"] = step.copy(order="F")
    deltat3 = O.F64(0.3 * d3.min_dist)
    K.re_step_eno3(step, F, mask, deltat3, *d3.six(), *g.args(), g.num_ele)
    rec["re_step3"] = step.copy(order="F")
    rec["reinit5_it4"] = O.reinit_weno5(K, g, F, 4, d5)
    rec["reinit3_it4"] = O.reinit_eno3(K, g, F, 4)
    for tag, dd, e3 in (("5", d5, False), ("3", d3, True)):
        n3 = [O.zeros(g) for _ in range(3)]
        (K.upwind_normal_eno3 if e3 else K.upwind_normal)(*n3, F, *dd.six(), *g.args(), g.num_ele)
        for ax, a in zip("xyz", n3):
            rec[f"normal{tag}_{ax}"] = a
        cp = O.crossing_values(K, g, C, dd, eno3=e3)
        for nm, a in zip(("cpr", "cpl", "cpf", "cpb", "cpu", "cpd"), cp):
            rec[f"cross{tag}_{nm}"] = a
    rec["extend5_it3"] = O.extend_weno5(K, g, F, d5, C, 3)
    rec["extend3_it3"] = O.extend_eno3(K, g, F, C, 3)
    tb = O.calculus_toolbox(K, g, F)
    for k in O.TOOLBOX_FIELDS:
        rec["tb_" + k] = tb[k]
    rng = np.random.default_rng(11)
    v = [O.F64(rng.standard_normal(g.size)) for _ in range(3)]
    for ax, a in zip("xyz", v):
        rec["v" + ax] = a
    rec["advection_step"] = O.weno_dot_grad(K, g, *v, F)
    wd = [O.zeros(g) for _ in range(6)]
    K.weno_derivative(*wd, F, *g.args())
    for nm, a in zip(("back_x", "fore_x", "back_y", "fore_y", "back_z", "fore_z"), wd):
        rec["wd_" + nm] = a
    rec["redistance_2_2"] = O.surface_redistance(K, g, F, C, 2, 2)
    # ENORK2: quadratic-ENO distances, re_step, Heun RK2 reinitialization and extension
    d2 = O.set_distance_enork2(K, g, F)
    for nm, a in zip(("xpr", "xpl", "ypf", "ypb", "zpu", "zpd"), d2.six()):
        rec["dist2_" + nm] = a
    K.enork2_re_step(step, F, mask, O.F64(0.3 * d2.min_dist), *d2.six(), *g.args(), g.num_ele)
    rec["re_step2"] = step.copy(order="F")
    n3 = [O.zeros(g) for _ in range(3)]
    K.enork2_upwind_normal(*n3, F, *d2.six(), *g.args(), g.num_ele)
    for ax, a in zip("xyz", n3):
        rec[f"normal2_{ax}"] = a
    cp = [O.zeros(g) for _ in range(6)]
    K.enork2_boundary_interpolate(*cp, *d2.six(), C, *g.args(), g.num_ele)
    for nm, a in zip(("cpr", "cpl", "cpf", "cpb", "cpu", "cpd"), cp):
        rec[f"cross2_{nm}"] = a
    rec["reinit2_it4"] = O.reinit_enork2(K, g, F, 4)
    rec["extend2_it3"] = O.extend_enork2(K, g, F, C, 3)
    rec["redistance2_2_2"] = O.surface_redistance_enork2(K, g, F, C, 2, 2)
    rec["area"] = np.array(O.cal_area(g, F, tb["DiracDelta"]))
    rec["volume"] = np.array(O.cal_volume(g, F, tb["Heaviside"]))
    return rec


def main():
    build_oracle.build()
    K = O.kernels("ref")
    digest = reference_digest()
    for name, x, y, z, F, C in cases():
        rec = run_case(K, name, x, y, z, F, C)
        rec["reference_sha256"] = np.array(digest)
        path = os.path.join(HERE, f"golden_{name}.npz")
        np.savez_compressed(path, **rec)
        print(f"{path}: {len(rec)} arrays, {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
