"""Generate the golden fixture of the auxiliary level set toolbox from the reference's own
kernel (auxi_set_calculus_toolbox.cu, compiled for the host by ``oracle/ref/Makefile``),
with F's toolbox from the reference's set_calculus_toolbox.cu, on two seeded cases, and
write ``golden_auxi.npz`` beside this script: the axis vectors, F, A and the kernel's 27
fields.  The integrals of SDF3.m:82-85, 212-227 are stored too, evaluated with the
oracle's numpy restatement of the MATLAB glue (AFDiracDelta of GPUAsetCalculusToolBox.m
and the masked sums), which has no other form outside MATLAB.

It needs the reference checkout, so it runs in the development container only; the
fixture it writes is committed and read by the tests everywhere.

    python tests/golden/gen_golden_auxi.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    rng = np.random.default_rng(7)
    # a sphere cut by a tilted plane: the domain boundary is a circle
    xv, yv, zv = np.linspace(-1, 1, 14), np.linspace(-0.95, 0.95, 13), np.linspace(-0.9, 0.9, 12)
    x, y, z = np.meshgrid(xv, yv, zv)
    F = np.sqrt(x**2 + y**2 + z**2) - 0.62
    A = z - 0.12 + 0.25 * x + 0.01 * rng.standard_normal(x.shape)
    yield "plane", (xv, yv, zv), x, y, z, F, A
    # an oblate ellipsoid with a spherical-cap domain around the +x pole
    v = np.linspace(-1, 1, 12)
    x, y, z = np.meshgrid(v, v, v)
    F = np.sqrt(x**2 / 0.7**2 + y**2 / 0.7**2 + z**2 / 0.4**2) - 1
    A = np.sqrt((x - 0.7) ** 2 + y**2 + (z - 0.05) ** 2) - 0.45
    yield "cap", (v, v, v), x, y, z, F, A


def main():
    build_oracle.build_port()
    if build_oracle.build_ref() is None:
        raise SystemExit("the reference checkout is needed to generate the fixture")
    R = O.kernels("ref")
    out = {}
    for name, (xv, yv, zv), x, y, z, F, A in cases():
        F, A = O.F64(F), O.F64(A)
        g = O.grid_from_mesh(x, y, z)
        aux, tb = O.auxiliary_toolbox(R, g, F, A)
        out[f"{name}/xv"], out[f"{name}/yv"], out[f"{name}/zv"] = xv, yv, zv
        out[f"{name}/F"], out[f"{name}/A"] = F, A
        for n in O.AUX_FIELDS:
            out[f"{name}/{n}"] = O.F64(aux[n])
        fld = O.F64(np.sin(2 * x) * np.cos(y) + z)
        out[f"{name}/calLength"] = np.array(O.cal_length(g, F, A, aux))
        out[f"{name}/LineIntegral"] = np.array(O.line_integral(g, F, A, fld, aux))
        out[f"{name}/AcalArea"] = np.array(O.a_cal_area(g, F, tb, aux))
        out[f"{name}/AsurfaceIntegral"] = np.array(O.a_surface_integral(g, F, fld, tb, aux))
        out[f"{name}/surfaceIntegral"] = np.array(
            O.surface_integral_mask(g, F, fld, tb["DiracDelta"], tb["FGradMag"]))
    path = os.path.join(HERE, "golden_auxi.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays")


if __name__ == "__main__":
    main()
