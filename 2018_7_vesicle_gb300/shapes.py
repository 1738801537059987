"""Initial level-set fields of the benchmark and test workloads (host-side numpy setup,
the role of the reference's SD.Shape package, src/7_0_paper/2_0_Vesicle/+SD/+Shape/).

All fields are float64 numpy arrays of shape (rows, cols, pges) = (y, x, z) in Fortran
order, the MATLAB meshgrid layout.
"""
from __future__ import annotations

import math

import numpy as np


def meshgrid(xv, yv, zv):
    x, y, z = np.meshgrid(np.asarray(xv, float), np.asarray(yv, float), np.asarray(zv, float))
    return np.asfortranarray(x), np.asfortranarray(y), np.asfortranarray(z)


def cube_grid(n: int, lo: float, hi: float):
    """n^3 nodes on [lo, hi]^3 (x = linspace(lo, hi, n) on every axis)."""
    v = np.linspace(lo, hi, n)
    return meshgrid(v, v, v)


def perturbed_sphere(x, y, z, r: float = 0.6, centre=(0.35, 0.35, 0.35)):
    """The non-distance sphere of the reinitialization workload:
    (sqrt(x^2+y^2+z^2) - r) * (0.1 + (x-cx)^2 + (y-cy)^2 + (z-cz)^2)."""
    cx, cy, cz = centre
    return np.asfortranarray((np.sqrt(x**2 + y**2 + z**2) - r) * (0.1 + (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2))


def oblate_reduced_volume(c: float) -> float:
    """Reduced volume of the oblate spheroid with half axes (1, 1, c), c < 1
    (Ellipsoid.m:73-85 for a = b = 1, where the elliptic integrals reduce to closed form)."""
    e = math.sqrt(1 - c * c)
    area = 2 * math.pi * (1 + c * c / e * math.atanh(e))
    volume = 4 * math.pi * c / 3
    return (3 * volume / 4 / math.pi) * (4 * math.pi / area) ** 1.5


def oblate_c_for_reduced_volume(rv: float) -> float:
    """Half axis c of the (1, 1, c) oblate spheroid with reduced volume rv (bisection)."""
    lo, hi = 1e-4, 1 - 1e-9
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if oblate_reduced_volume(mid) < rv:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def _legendre_all(lmax: int, t):
    """Associated Legendre P_l^m(t), 0 <= m <= l <= lmax, (no Condon-Shortley phase)."""
    s = np.sqrt(np.maximum(0.0, 1 - t * t))
    P = {}
    P[(0, 0)] = np.ones_like(t)
    for m in range(1, lmax + 1):
        P[(m, m)] = (2 * m - 1) * s * P[(m - 1, m - 1)]
    for m in range(0, lmax):
        P[(m + 1, m)] = (2 * m + 1) * t * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * t * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    return P


def sh_noise(x, y, z, lmax: int, seed: int):
    """Real spherical-harmonic series sum_{l<=lmax, |m|<=l} a_lm Y_lm(theta, phi) with
    a_lm ~ N(0, 1) from numpy's default_rng(seed), normalised to max |.| = 1 on the grid."""
    rng = np.random.default_rng(seed)
    r = np.sqrt(x**2 + y**2 + z**2)
    t = np.where(r > 0, z / np.where(r > 0, r, 1), 1.0)
    ph = np.arctan2(y, x)
    P = _legendre_all(lmax, t)
    out = np.zeros_like(x)
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            ang = np.cos(am * ph) if m >= 0 else np.sin(am * ph)
            if m != 0:
                norm *= math.sqrt(2)
            out += rng.standard_normal() * norm * P[(l, am)] * ang
    return np.asfortranarray(out / np.max(np.abs(out)))


def noisy_oblate(x, y, z, axes=(1.0, 1.0, 0.55), amplitude: float = 0.02, lmax: int = 6, seed: int = 0):
    """Oblate ellipsoid sqrt(x^2/a^2+y^2/b^2+z^2/c^2) - 1 (Ellipsoid.m:45) with its radius
    perturbed by `amplitude` times a seeded spherical-harmonic series (l <= lmax)."""
    a, b, c = axes
    base = np.sqrt(x**2 / a**2 + y**2 / b**2 + z**2 / c**2)
    return np.asfortranarray(base - 1 - amplitude * sh_noise(x, y, z, lmax, seed))


def vesicle_256(n: int = 256, seed: int = 0, reduced_volume: float = 0.65):
    """The mixed-precision vesicle workload: n^3 on [-1.5, 1.5]^3, oblate ellipsoid with
    half axes (1, 1, c(reduced volume)) plus l <= 6 spherical-harmonic noise of 0.02."""
    x, y, z = cube_grid(n, -1.5, 1.5)
    c = oblate_c_for_reduced_volume(reduced_volume)
    return x, y, z, noisy_oblate(x, y, z, axes=(1.0, 1.0, c), seed=seed)


def surface_field(x, y, z):
    """The scalar field redistanced on the interface: sin(3x) cos(2y) + 0.5 z^2."""
    return np.asfortranarray(np.sin(3 * x) * np.cos(2 * y) + 0.5 * z**2)
