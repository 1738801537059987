"""SD.Shape.Ellipsoid (Ellipsoid.m:5-85) on the host: the reduced-volume function on both
branches the reference uses, against the spheroids' independent closed-form areas, and the
shape's half axes from the interpolated table.  CPU only."""
import importlib
import math

import numpy as np
import pytest

S = importlib.import_module("2018_7_vesicle_gb300.shapes")


def rv_of(area, volume):
    return (3 * volume / 4 / math.pi) * (4 * math.pi / area) ** 1.5


@pytest.mark.parametrize("c", [0.05, 0.3, 0.55, 0.8, 0.99])
def test_oblate_branch_matches_the_oblate_spheroid(c):
    e = math.sqrt(1 - c * c)
    area = 2 * math.pi * (1 + c * c / e * math.atanh(e))
    assert S.ellipsoid_reduced_volume(1.0, 1.0, c) == pytest.approx(rv_of(area, 4 * math.pi * c / 3), rel=1e-13)


@pytest.mark.parametrize("c", [0.05, 0.3, 0.55, 0.8, 0.99])
def test_prolate_branch_matches_the_prolate_spheroid(c):
    # half axes (1, c, c): area 2 pi c^2 (1 + arcsin(e) / (c e)), e^2 = 1 - c^2
    e = math.sqrt(1 - c * c)
    area = 2 * math.pi * c * c * (1 + math.asin(e) / (c * e))
    assert S.ellipsoid_reduced_volume(1.0, c, c) == pytest.approx(rv_of(area, 4 * math.pi * c * c / 3), rel=1e-13)


@pytest.mark.parametrize("kind,rv", [("O", 0.6), ("O", 0.8), ("P", 0.6), ("P", 0.9)])
def test_shape_axes_and_field(kind, rv):
    size = (40, 36, 44)
    x, y, z, f, (a, b, c) = S.ellipsoid(size, rv, kind, 0.35)
    assert f.shape == (36, 40, 44)  # meshgrid(xv, yv, zv): rows y, columns x, pages z
    dx = 2.0 / 39
    zv = (np.arange(44) - 21.5) * dx
    if kind == "O":
        assert a == b == pytest.approx(0.7) and c < a
        got = S.ellipsoid_reduced_volume(1.0, 1.0, c / a)
        want = np.sqrt(x**2 / a**2 + y**2 / b**2 + z**2 / c**2) - 1
    else:
        assert a == pytest.approx(0.35 * (zv[-1] - zv[0])) and b == c < a
        got = S.ellipsoid_reduced_volume(1.0, b / a, b / a)
        want = np.sqrt(x**2 / b**2 + y**2 / c**2 + z**2 / a**2) - 1
    # cq is interpolated linearly in a table at steps of 0.01
    assert got == pytest.approx(rv, abs=2e-3)
    assert np.array_equal(f, np.asfortranarray(want))
    assert np.allclose(z[0, 0, :], zv) and np.allclose(y[:, 0, 0], (np.arange(36) - 17.5) * dx)


def test_oblate_wrapper_is_the_oblate_branch():
    x, y, z, f = S.oblate_ellipsoid((24, 26, 28), 0.6, 0.35)
    assert np.array_equal(f, S.ellipsoid((24, 26, 28), 0.6, "O", 0.35)[3])
