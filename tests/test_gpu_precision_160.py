"""The mixed-precision form against the FP64 oracle on the vesicle workload at 160^3
(the oblate vesicle of reduced volume 0.65 with l <= 6 harmonic noise on [-1.5, 1.5]^3,
seeded), at the tolerances the mixed form is specified to: interface-band error at most
1e-5 dx relative to the FP64 oracle, area and volume within 1e-8 per step.

Per operation, errors over the band |phi| < 3 dx of the oracle's result:

* 20 WENO5 TVD-RK3 reinitialization pseudo-steps: max 1e-5 dx, rms 1e-6 dx;
* 30 WENO5 extension pseudo-steps of the mean curvature: max 5e-5 of the band's max |H|
  (the FP32 rounding of the extended field itself is 6e-8 of it);
* one whole vesicle step (toolbox, extension, time step, advection, setDistance,
  reinitialization): field max 1e-5 dx, rms 1e-6 dx; area and volume of the step's input
  within 1e-8 relative, the time step within 1e-6.

The FP32 form's distances come from its own setDistance on the FP32 field (FP64 roots of
the promoted values).  GPU only."""
import importlib

import numpy as np
import pytest

from gpu_util import dev, host

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")
N = 160


@pytest.fixture(scope="module")
def vesicle(oracle_mod):
    O = oracle_mod
    x, y, z, F = S.vesicle_256(N, seed=0)
    g = O.grid_from_mesh(x, y, z)
    K = O.kernels("port")
    return O, K, g, x, y, z, F, O.set_distance(K, g, F)


def f32(pkg, x, y, z, F):
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
    m.setDistance()
    return m


def band_errors(got, ref, dx):
    band = np.abs(ref) < 3 * dx
    e = np.abs(got[band] - ref[band]) / dx
    return float(e.max()), float(np.sqrt(np.mean(e**2)))


def test_reinitialization_20(pkg, vsl, vesicle):
    O, K, g, x, y, z, F, d = vesicle
    ref = O.reinit_weno5(K, g, F, 20, d)
    m = f32(pkg, x, y, z, F)
    mx, rms = band_errors(host(m.WENO5RK3Reinitialization(m.F, 20)), ref, g.dx)
    print(f"\nreinitialization 20 at {N}^3: band max {mx:.2e} dx, rms {rms:.2e} dx")
    assert mx <= 1e-5 and rms <= 1e-6


def test_extension_30(pkg, vsl, vesicle):
    O, K, g, x, y, z, F, d = vesicle
    H = O.calculus_toolbox(K, g, F)["MeanCurvature"]
    ref = O.extend_weno5(K, g, F, d, H, 30)
    m = f32(pkg, x, y, z, F)
    got = host(m.WENO5RK3Extend(dev(H), 30))
    band = np.abs(F) < 3 * g.dx
    scale = float(np.max(np.abs(H[band])))
    e = np.abs(got[band] - ref[band]) / scale
    print(f"\nextension 30 at {N}^3: band max {e.max():.2e}, rms {np.sqrt(np.mean(e**2)):.2e} of max |H|")
    assert e.max() <= 5e-5


def test_vesicle_step(pkg, vsl, vesicle):
    O, K, g, x, y, z, F, d = vesicle
    Fn, dn, oi = O.vesicle_step(K, g, F, d, 30, 20, 0.5)
    m = f32(pkg, x, y, z, F)
    info = m.vesicle_step(30, 20, 0.5).cpu().numpy()
    mx, rms = band_errors(host(m.F), Fn, g.dx)
    da, dv, ddt = abs(info[0] / oi["area"] - 1), abs(info[1] / oi["volume"] - 1), abs(info[2] / oi["dt"] - 1)
    print(f"\nvesicle step at {N}^3: band max {mx:.2e} dx, rms {rms:.2e} dx; area {da:.1e}, volume {dv:.1e}, "
          f"dt {ddt:.1e}")
    assert mx <= 1e-5 and rms <= 1e-6
    assert da <= 1e-8 and dv <= 1e-8 and ddt <= 1e-6
