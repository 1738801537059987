"""Known-answer tests: the convergence studies of the reference's WENO paper scripts
(src/7_0_paper/1_0_WENO/p07_test_curvature.m, p08_test_extend.m, p20_test_merging_front.m,
p11_test_surface_redistance_table.m) re-run on the GPU at 16^3, 32^3 and 64^3 on [-1, 1]^3.

Each error is the script's: the difference from the exact answer, extended off the
surface with WENORK3Extend(., 100) (WENO5RK3Extend for the geodesic curvature), then
L1 = surfaceIntegral(|D|), L2 = sqrt(surfaceIntegral(D^2)) and the maximum over
|F| < 1.5 Ds.  The surface measure comes from the second-order GPU toolbox (the scripts use
the CPU fourth-order setCalculusToolBox4; only the quadrature weights differ).

* p07: the non-distance sphere x^2+y^2+z^2-0.36, setDistance and 1000 WENO5 RK3
  reinitialization pseudo-steps: F against the distance (order >= 4), the mean curvature
  against -2/r and the Gaussian curvature against 1/r^2 (order >= 1.8);
* p08: z extended off the sphere of radius 0.5 (WENO5RK3Extend 100) against
  r0 sin(elevation) (order >= 4), and GD3.Laplacian of it (extended) against
  -2/r0^2 r0 sin(elevation) (order >= 1.8);
* p20: two merged spheres min(f1, f2) reinitialized (1000) against min(F1, F2) (order
  >= 1.3 at the finest pair: the kink limits it);
* p11: A = exp(z) - 1 on the sphere of radius 0.6, WENO5 closest-point surface
  redistance (200 x 100) against the geodesic distance r0 elevation (order >= 4) and the
  geodesic curvature of its level sets (auxiliary toolbox) against tan(elevation) / r0
  (order >= 1.7), both away from the caps where that curvature exceeds 2; FP32 only (the
  FP64 form takes minutes here).
The absolute bounds are 1.5 times the errors measured with the FP64 form (bitwise the
oracle) at 32^3 and 64^3; the FP32 form meets the same bounds.
GPU only."""
import importlib
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
SIZES = (16, 32, 64)


def _mesh(pkg, n, zv=None):
    S = importlib.import_module(pkg.__name__ + ".shapes")
    v = np.linspace(-1, 1, n)
    return S.meshgrid(v, v, v if zv is None else zv, device="cuda")


def _errors(m, D, extend=None):
    """(L1, L2, max) of D extended off F = 0, as the scripts measure them."""
    D = (extend or m.WENORK3Extend)(D.to(m.dtype), 100)
    m.GPUsetCalculusToolBox()
    Dd = D.double()
    band = m.F.double().abs() < 1.5 * m.GD3.Ds
    return (m.surfaceIntegral(Dd.abs()), math.sqrt(max(m.surfaceIntegral(Dd * Dd), 0.0)),
            float(Dd[band].abs().max()))


def p07(pkg, n, prec):
    x, y, z = _mesh(pkg, n)
    r = 0.6
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=x**2 + y**2 + z**2 - r * r, precision=prec)
    m.setDistance()
    m.F = m.WENO5RK3Reinitialization(m.F, 1000)
    m.setDistance()
    m.GPUsetCalculusToolBox()
    H, K = m.MeanCurvature.clone(), m.GaussianCurvature.clone()
    return {"F": _errors(m, m.F.double() - (torch.sqrt(x**2 + y**2 + z**2) - r)),
            "H": _errors(m, m.WENORK3Extend(H, 100).double() + 2.0 / r),
            "K": _errors(m, m.WENORK3Extend(K, 100).double() - 1.0 / r**2)}


def p08(pkg, n, prec):
    x, y, z = _mesh(pkg, n)
    r0 = 0.5
    rr = torch.sqrt(x**2 + y**2 + z**2)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=rr - r0, precision=prec)
    m.setDistance()
    exact = r0 * z / rr  # r0 sin(elevation)
    G = m.WENO5RK3Extend(z, 100)
    L = m.WENO5RK3Extend(m.GD3.Laplacian(G, precision=prec), 100)
    return {"G": _errors(m, G.double() - exact), "lapG": _errors(m, L.double() + 2 / r0**2 * exact)}


def p20(pkg, n, prec):
    v = np.linspace(-1, 1, n)
    nz = int(1.5 * n)
    zv = (np.arange(nz) + (1 - nz) / 2.0) * (v[1] - v[0])
    x, y, z = _mesh(pkg, n, zv)
    r, z0 = 0.6, 0.3
    f = torch.minimum(x**2 + y**2 + (z - z0) ** 2 - r * r, x**2 + y**2 + (z + z0) ** 2 - r * r)
    exact = torch.minimum(torch.sqrt(x**2 + y**2 + (z - z0) ** 2) - r, torch.sqrt(x**2 + y**2 + (z + z0) ** 2) - r)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=f, precision=prec)
    m.setDistance()
    m.F = m.WENO5RK3Reinitialization(m.F, 1000)
    m.setDistance()
    return {"F": _errors(m, m.F.double() - exact)}


def p11(pkg, n, prec):
    x, y, z = _mesh(pkg, n)
    r0 = 0.6
    rr = torch.sqrt(x**2 + y**2 + z**2)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=rr - r0, precision=prec)
    m.setDistance()
    elev = torch.asin(torch.clamp(z / rr.clamp(min=1e-30), -1, 1))
    G = m.WENO5RK3ClosetPointSurfaceRedistance(torch.exp(z) - 1, 200, 100)
    m.A = G
    m.GPUAsetCalculusToolBox(fields=("GeodesicCurvature",))
    kexact = torch.tan(elev) / r0
    cap = kexact.abs() > 2
    out = {}
    for name, D, ext in (("G", G.double() - r0 * elev, m.WENORK3Extend),
                         ("kg", kexact - m.GeodesicCurvature.double(), m.WENO5RK3Extend)):
        D = D.clone()
        D[cap] = 0
        D = ext(D.to(m.dtype), 100).double()
        D[cap] = 0
        m.GPUsetCalculusToolBox()
        band = (m.F.double().abs() < 1.5 * m.GD3.Ds) & ~cap
        out[name] = (m.surfaceIntegral(D.abs()), math.sqrt(max(m.surfaceIntegral(D * D), 0.0)),
                     float(D[band].abs().max()))
    return out


# measured with the FP64 form: case -> quantity -> {n: (L1, L2, max)}, and the least order
# (16 -> 32 -> 64, each of L1 and L2 at the finest pair; the maximum is reported)
MEASURED = {
    "p07": {"F": ({32: (1.03e-7, 6.75e-8, 9.3e-8), 64: (2.85e-9, 1.73e-9, 2.26e-9)}, 4.0),
            "H": ({32: (1.15e-2, 7.50e-3, 9.53e-3), 64: (2.72e-3, 1.79e-3, 2.33e-3)}, 1.8),
            "K": ({32: (1.97e-2, 1.29e-2, 1.64e-2), 64: (4.56e-3, 2.99e-3, 3.91e-3)}, 1.8)},
    "p08": {"G": ({32: (3.40e-6, 2.72e-6, 4.54e-6), 64: (3.04e-8, 2.80e-8, 1.48e-7)}, 4.0),
            "lapG": ({32: (6.07e-2, 4.04e-2, 5.29e-2), 64: (1.45e-2, 9.68e-3, 1.19e-2)}, 1.8)},
    "p20": {"F": ({32: (1.53e-4, 2.37e-4, 7.75e-4), 64: (4.10e-5, 7.98e-5, 2.69e-4)}, 1.3)},
    "p11": {"G": ({32: (3.90e-5, 3.24e-5, 4.62e-5), 64: (1.26e-6, 8.87e-7, 1.42e-6)}, 4.0),
            "kg": ({32: (3.30e-2, 2.33e-2, 3.57e-2), 64: (7.90e-3, 6.07e-3, 1.71e-2)}, 1.7)},
}
# the FP32 form's extra rounding at 64^3 where the FP64 errors are near 1e-8 (p07 F,
# p08 G, p11 G): its bound is 4x the FP64 measurement there
FP32_SLACK = {("p07", "F"): 4.0, ("p08", "G"): 4.0, ("p11", "G"): 4.0}


def _check(case, prec, table):
    for q, (bounds, order) in MEASURED[case].items():
        for n, ref in bounds.items():
            slack = 1.5 * (FP32_SLACK.get((case, q), 1.0) if prec == "f32" else 1.0)
            got = table[n][q]
            assert all(g <= slack * b for g, b in zip(got, ref)), (case, q, n, prec, got, ref)
        # convergence order of L1 and L2 between 32^3 and 64^3 (spacing ratio 63/31)
        for k in (0, 1):
            o = math.log(table[32][q][k] / table[64][q][k]) / math.log(63 / 31)
            assert o >= order, (case, q, prec, k, o)


def _run(pkg, case, prec):
    fn = {"p07": p07, "p08": p08, "p20": p20, "p11": p11}[case]
    table = {n: fn(pkg, n, prec) for n in SIZES}
    for n in SIZES:
        print(case, prec, n, {q: tuple(f"{v:.2e}" for v in e) for q, e in table[n].items()})
    return table


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("case", ["p07", "p08", "p20"])
def test_convergence(pkg, vsl, case, prec):
    _check(case, prec, _run(pkg, case, prec))


def test_surface_redistance_geodesics_fp32(pkg, vsl):
    _check("p11", "f32", _run(pkg, "p11", "f32"))
