"""Known answer for the oracle's restatement of WENORK3ClosetPointSurfaceRedistance (the
checker of vsl_wenork3_surface_redistance_*): the setting of
src/7_0_paper/1_0_WENO/p11_test_surface_redistance_table.m with the WENORK3 form, which
p17_test_surface_redistance_table3.m names as its alternative.  A = exp(z) - 1 on the sphere
of radius 0.6 centred in [-1, 1]^3, redistanced on the sphere (60 x 30 iterations), against
the geodesic distance r0 * elevation, at the nodes within 1.5 dx of the sphere away from the
caps where the geodesic curvature tan(elevation) / r0 exceeds 2.

The oracle's kernels are bitwise the reference's own (test_oracle_vs_reference); this pins
the composition: it converges to the geodesic distance at third order or better.  Bounds:
1.5 times the errors measured here (1.88e-3 at 16^3, 4.38e-4 at 24^3; order 3.4).  CPU only,
about 10 s."""
import numpy as np
import pytest


def geodesic_error(O, K, n, eno3):
    v = np.linspace(-1, 1, n)
    x, y, z = O.meshgrid(v, v, v)
    g = O.grid_from_mesh(x, y, z)
    r0 = 0.6
    rr = np.sqrt(x**2 + y**2 + z**2)
    F = O.F64(rr - r0)
    elev = np.arcsin(np.clip(z / np.maximum(rr, 1e-30), -1, 1))
    G = O.surface_redistance(K, g, F, O.F64(np.exp(z) - 1), 60, 30, eno3=eno3)
    band = (np.abs(F) < 1.5 * g.dx) & ~(np.abs(np.tan(elev) / r0) > 2)
    return float(np.abs(G - r0 * elev)[band].max()), g.dx


@pytest.fixture(scope="module")
def port(oracle_mod):
    return oracle_mod, oracle_mod.kernels("port")


def test_wenork3_redistance_converges_to_the_geodesic_distance(port):
    O, K = port
    e16, h16 = geodesic_error(O, K, 16, eno3=True)
    e24, h24 = geodesic_error(O, K, 24, eno3=True)
    assert e16 <= 1.5 * 1.88e-3
    assert e24 <= 1.5 * 4.38e-4
    assert np.log(e16 / e24) / np.log(h16 / h24) >= 3.0
