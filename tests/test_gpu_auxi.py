"""The auxiliary level set of multiphase vesicles on the GPU (auxi_set_calculus_toolbox.cu,
GPUAsetCalculusToolBox.m, SDF3.m:82-85, 212-227) against the oracle.

* the drop-in vsl_auxi_set_calculus_toolbox (FP64): bit for bit the oracle built with
  correctly rounded powers, given the same F toolbox inputs;
* the fused method (reads only A and F; FP64): the 27 kernel fields bit for bit, and
  AFDiracDelta / ADiracDeltaDn (periodic GD3 operators) within 1e-12;
* the integrals (calLength, LineIntegral, AcalArea, AsurfaceIntegral, surfaceIntegral):
  FP64 sums within 1e-12 of the oracle's correctly rounded sums (relative to max(|value|, 1):
  an odd field's surface integral is 0 up to rounding);
* FP32 against FP64: the integrals within 1e-4 relative;
* known answers on a sphere of radius R = 0.6 cut by the plane z = z0 at 64^3: the circle
  length 2 pi sqrt(R^2 - z0^2), the area 2 pi R (R + z0) of the part below the plane, the
  normal curvature -1/R and the geodesic curvature magnitude z0 / (R sqrt(R^2 - z0^2))
  along the circle, within 1-3%.
GPU only."""
import importlib
import os

import numpy as np
import pytest
import torch

from gpu_util import dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("plane", "cap")


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "golden_auxi.npz"))


def case(O, G, name):
    x, y, z = np.meshgrid(G[f"{name}/xv"], G[f"{name}/yv"], G[f"{name}/zv"])
    return O.grid_from_mesh(x, y, z), x, y, z, G[f"{name}/F"], G[f"{name}/A"]


@pytest.mark.parametrize("name", CASES)
def test_dropin_bitwise(vsl, oracle_mod, golden, name):
    O = oracle_mod
    K = O.kernels("port_crpow")
    g, x, y, z, F, A = case(O, golden, name)
    ref, tb = O.auxiliary_toolbox(K, g, F, A)
    shape = (g.rows, g.cols, g.pges)
    outs = [empty(shape, fill=np.nan) for _ in range(27)]
    ins = [dev(tb[n]) for n in O.AUX_INPUTS]
    Ad, hp = dev(A), dev(np.maximum(A, 0))
    vsl.call("vsl_auxi_set_calculus_toolbox", *map(ptr, outs), ptr(Ad), ptr(hp), *map(ptr, ins), *g.args(), g.ds,
             g.num_ele, stream())
    for t, n in zip(outs, O.AUX_FIELDS):
        assert np.array_equal(host(t), ref[n]), n


@pytest.mark.parametrize("name", CASES)
def test_fused_fp64(pkg, vsl, oracle_mod, golden, name):
    O = oracle_mod
    g, x, y, z, F, A = case(O, golden, name)
    ref, tb = O.auxiliary_toolbox(O.kernels("port_crpow"), g, F, A)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f64")
    m.A = dev(A)
    m.GPUAsetCalculusToolBox()
    for n in O.AUX_FIELDS:
        assert np.array_equal(host(getattr(m, n)), ref[n]), n
    for n in ("AFDiracDelta", "ADiracDeltaDn"):
        got, want = host(getattr(m, n)), ref[n]
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), n
    # the integrals, with F's toolbox on the object
    m.GPUsetCalculusToolBox()
    fld = np.sin(2 * x) * np.cos(y) + z
    got = {"calLength": m.calLength(), "LineIntegral": m.LineIntegral(dev(fld)), "AcalArea": m.AcalArea(),
           "AsurfaceIntegral": m.AsurfaceIntegral(dev(fld)), "surfaceIntegral": m.surfaceIntegral(dev(fld))}
    for k, v in got.items():
        want = float(golden[f"{name}/{k}"])
        assert abs(v - want) <= 1e-12 * max(abs(want), 1.0), (k, v, want)  # some are 0 up to rounding


def test_subset_of_fields(pkg, vsl, oracle_mod, golden):
    """Asking for a few fields writes those alone, with the same values."""
    O = oracle_mod
    g, x, y, z, F, A = case(O, golden, "cap")
    ref, _ = O.auxiliary_toolbox(O.kernels("port_crpow"), g, F, A)
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f64")
    m.A = dev(A)
    m.GPUAsetCalculusToolBox(fields=("GeodesicCurvature", "AFDiracDelta"))
    assert np.array_equal(host(m.GeodesicCurvature), ref["GeodesicCurvature"])
    assert np.abs(host(m.AFDiracDelta) - ref["AFDiracDelta"]).max() <= 1e-12 * np.abs(ref["AFDiracDelta"]).max()
    assert not hasattr(m, "NormalCurvature")


def sphere_plane(pkg, n, precision, z0=0.2, R=0.6):
    S = importlib.import_module(pkg.__name__ + ".shapes")
    v = np.linspace(-1, 1, n)
    x, y, z = S.meshgrid(v, v, v, device="cuda")
    F = torch.sqrt(x**2 + y**2 + z**2) - R
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision=precision)
    m.A = z - z0
    m.GPUsetCalculusToolBox()
    m.GPUAsetCalculusToolBox()
    return m


def test_fp32_integrals_against_fp64(pkg, vsl):
    m64 = sphere_plane(pkg, 64, "f64")
    m32 = sphere_plane(pkg, 64, "f32")
    for f in ("calLength", "AcalArea"):
        a, b = getattr(m32, f)(), getattr(m64, f)()
        print("FP32 vs FP64", f, a, b, abs(a / b - 1))
        assert abs(a / b - 1) <= 1e-4, f
    a = m32.LineIntegral(m32.GeodesicCurvature)
    b = m64.LineIntegral(m64.GeodesicCurvature)
    assert abs(a / b - 1) <= 1e-3


def test_sphere_plane_known_answers(pkg, vsl):
    R, z0 = 0.6, 0.2
    m = sphere_plane(pkg, 64, "f64", z0, R)
    r = np.sqrt(R * R - z0 * z0)
    length = m.calLength()
    area = m.AcalArea()
    kn = m.LineIntegral(m.NormalCurvature) / length
    kg = m.LineIntegral(m.GeodesicCurvature) / length
    print("length", length, 2 * np.pi * r, "area", area, 2 * np.pi * R * (R + z0), "kn", kn, -1 / R, "kg", kg,
          z0 / (R * r))
    assert abs(length / (2 * np.pi * r) - 1) <= 0.01
    assert abs(area / (2 * np.pi * R * (R + z0)) - 1) <= 0.01
    assert abs(kn * R + 1) <= 0.02
    assert abs(abs(kg) / (z0 / (R * r)) - 1) <= 0.03
