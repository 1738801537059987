"""Initial level-set fields of the benchmark and test workloads (host-side numpy setup,
the role of the reference's SD.Shape package, src/7_0_paper/2_0_Vesicle/+SD/+Shape/).

All fields have shape (rows, cols, pges) = (y, x, z), the MATLAB meshgrid layout:
float64 numpy arrays in Fortran order, or, where a torch device is given, float64 torch
tensors computed on that device (same values, the pointwise formulas run on the GPU).
"""
from __future__ import annotations

import math

import numpy as np


def meshgrid(xv, yv, zv, device=None):
    if device is not None:
        import torch

        t = [torch.as_tensor(np.asarray(v, float), device=device) for v in (xv, yv, zv)]
        return torch.meshgrid(t[0], t[1], t[2], indexing="xy")
    x, y, z = np.meshgrid(np.asarray(xv, float), np.asarray(yv, float), np.asarray(zv, float))
    return np.asfortranarray(x), np.asfortranarray(y), np.asfortranarray(z)


class _Ops:
    """The few array functions the shape formulas need, for numpy arrays or torch tensors."""

    def __init__(self, a):
        self.torch = not isinstance(a, np.ndarray)
        if self.torch:
            import torch

            self.m = torch
        else:
            self.m = np

    def atan2(self, y, x):
        return self.m.atan2(y, x) if self.torch else np.arctan2(y, x)

    def fortran(self, a):
        return a if self.torch else np.asfortranarray(a)

    def __getattr__(self, name):
        return getattr(self.m, name)


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
    xp = _Ops(t)
    s = xp.sqrt(xp.clamp(1 - t * t, min=0.0)) if xp.torch else np.sqrt(np.maximum(0.0, 1 - t * t))
    P = {(0, 0): xp.ones_like(t)}
    for m in range(1, lmax + 1):
        P[(m, m)] = (2 * m - 1) * s * P[(m - 1, m - 1)]
    for m in range(0, lmax):
        P[(m + 1, m)] = (2 * m + 1) * t * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * t * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    return P


def _sh_series(coef, lmax, t, ph):
    xp = _Ops(t)
    P = _legendre_all(lmax, t)
    out = xp.zeros_like(t)
    q = 0
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            ang = xp.cos(am * ph) if m >= 0 else xp.sin(am * ph)
            if m != 0:
                norm *= math.sqrt(2)
            out = out + float(coef[q]) * norm * P[(l, am)] * ang
            q += 1
    return out


def sh_noise(x, y, z, lmax: int, seed: int):
    """Real spherical-harmonic series sum_{l<=lmax, |m|<=l} a_lm Y_lm(theta, phi) of the
    direction of (x, y, z), a_lm ~ N(0, 1) from numpy's default_rng(seed), normalised to
    max |.| = 1 over a 1-degree sphere grid (so any sub-grid sees the same field)."""
    coef = np.random.default_rng(seed).standard_normal((lmax + 1) ** 2)
    th, phs = np.meshgrid(np.linspace(0, np.pi, 181), np.linspace(-np.pi, np.pi, 361), indexing="ij")
    scale = float(np.max(np.abs(_sh_series(coef, lmax, np.cos(th), phs))))
    xp = _Ops(x)
    r = xp.sqrt(x**2 + y**2 + z**2)
    safe = xp.where(r > 0, r, xp.ones_like(r))
    t = xp.where(r > 0, z / safe, xp.ones_like(r))
    return xp.fortran(_sh_series(coef, lmax, t, xp.atan2(y, x)) / scale)


def noisy_oblate(x, y, z, axes=(1.0, 1.0, 0.55), amplitude: float = 0.02, lmax: int = 6, seed: int = 0):
    """Oblate ellipsoid sqrt(x^2/a^2+y^2/b^2+z^2/c^2) - 1 (Ellipsoid.m:45) with its radius
    perturbed by `amplitude` times a seeded spherical-harmonic series (l <= lmax)."""
    a, b, c = axes
    xp = _Ops(x)
    base = xp.sqrt(x**2 / a**2 + y**2 / b**2 + z**2 / c**2)
    return xp.fortran(base - 1 - amplitude * sh_noise(x, y, z, lmax, seed))


def vesicle_256(n: int = 256, seed: int = 0, reduced_volume: float = 0.65, pages=None, device=None):
    """The mixed-precision vesicle workload: n^3 on [-1.5, 1.5]^3, oblate ellipsoid with
    half axes (1, 1, c(reduced volume)) plus l <= 6 spherical-harmonic noise of 0.02.
    `pages` (a slice of z indices) restricts it to a slab of the same field; `device`
    computes it as torch tensors on that device."""
    v = np.linspace(-1.5, 1.5, n)
    x, y, z = meshgrid(v, v, v if pages is None else v[pages], device=device)
    c = oblate_c_for_reduced_volume(reduced_volume)
    return x, y, z, noisy_oblate(x, y, z, axes=(1.0, 1.0, c), seed=seed)


def ellipsoid_reduced_volume(a: float, b: float, c: float) -> float:
    """Reduced volume (3V/4pi)(4pi/A)^(3/2) of the ellipsoid with half axes a >= b >= c
    (Ellipsoid.m:74-85).  The area is Legendre's form 2 pi c^2 + 2 pi a b (E(phi, m) sin^2 phi
    + F(phi, m) cos^2 phi) / sin phi with cos phi = c / a; as in the reference, the value
    k = a sqrt(b^2 - c^2) / (b sqrt(a^2 - c^2)) is passed as the integrals' second argument
    (the parameter m of MATLAB's ellipticE/ellipticF and of scipy's ellipeinc/ellipkinc).
    Both branches the reference uses have k = 0 (prolate, b = c) or k = 1 (oblate, a = b),
    where the integrals are elementary and taken in closed form; other axes go through
    scipy."""
    volume = 4 * math.pi * a * b * c / 3
    phi = math.atan2(math.sqrt(a * a - c * c), c)
    cos_phi = c / a
    sin_phi = math.sqrt(a * a - c * c) / a
    if b == c:  # k = 0: E(phi, 0) = F(phi, 0) = phi
        e_int = f_int = phi
    elif a == b:  # k = 1: E(phi, 1) = sin phi, F(phi, 1) = atanh(sin phi)
        e_int, f_int = sin_phi, math.atanh(sin_phi)
    else:
        from scipy.special import ellipeinc, ellipkinc

        k = a * math.sqrt(b * b - c * c) / b / math.sqrt(a * a - c * c)
        e_int, f_int = float(ellipeinc(phi, k)), float(ellipkinc(phi, k))
    area = 2 * math.pi * c * c + 2 * math.pi * a * b * (e_int * sin_phi**2 + f_int * cos_phi**2) / sin_phi
    return (3 * volume / 4 / math.pi) * (4 * math.pi / area) ** 1.5


def ellipsoid(size=(96, 96, 96), reduced_volume: float = 0.6, kind: str = "O", ratio: float = 0.35, device=None):
    """SD.Shape.Ellipsoid(Size, reducedVolume, TYPE, ratio) (Ellipsoid.m:5-72):
    x = linspace(-1, 1, size[0]), y and z centred on 0 with the same spacing
    ((1-n)/2 : (n-1)/2 times dx).  The axis ratio cq is interpolated linearly in the table
    of reduced volumes at c = 0.01 : 0.01 : 0.99 (interp1 of the reference).
      kind 'O' (oblate): half axes a = b = ratio (xmax - xmin) = 2 ratio, c = a cq, table of
        ReducedVolume(1, 1, c); field sqrt(x^2/a^2 + y^2/b^2 + z^2/c^2) - 1.
      kind 'P' (prolate): a = ratio (zmax - zmin), b = c = a cq, table of
        ReducedVolume(1, c, c); field sqrt(x^2/b^2 + y^2/c^2 + z^2/a^2) - 1 (long axis z).
    Returns x, y, z, the field and the half axes (a, b, c)."""
    nx, ny, nz = size
    xv = np.linspace(-1.0, 1.0, nx)
    dx = xv[1] - xv[0]
    yv = (np.arange(ny) + (1 - ny) / 2.0) * dx
    zv = (np.arange(nz) + (1 - nz) / 2.0) * dx
    x, y, z = meshgrid(xv, yv, zv, device=device)
    cs = np.arange(1, 100) / 100.0
    kind = kind.upper()[:1]
    xp = _Ops(x)
    if kind == "O":
        rv = np.array([ellipsoid_reduced_volume(1.0, 1.0, c) for c in cs])
        a = ratio * 2.0
        b = a
        c = a * float(np.interp(reduced_volume, rv, cs))
        f = xp.sqrt(x**2 / a**2 + y**2 / b**2 + z**2 / c**2) - 1
    elif kind == "P":
        rv = np.array([ellipsoid_reduced_volume(1.0, c, c) for c in cs])
        a = ratio * (float(zv[-1]) - float(zv[0]))
        b = a * float(np.interp(reduced_volume, rv, cs))
        c = b
        f = xp.sqrt(x**2 / b**2 + y**2 / c**2 + z**2 / a**2) - 1
    else:
        raise ValueError("kind must be 'O' (oblate) or 'P' (prolate)")
    return x, y, z, xp.fortran(f), (a, b, c)


def oblate_ellipsoid(size=(96, 96, 96), reduced_volume: float = 0.6, ratio: float = 0.35, device=None):
    """The relaxation driver's initial shape, SD.Shape.Ellipsoid(size, rv, 'O', ratio)
    (p00_test_singlephase_relax.m:24); see `ellipsoid`.  Returns x, y, z and the field."""
    return ellipsoid(size, reduced_volume, "O", ratio, device)[:4]


def surface_field(x, y, z):
    """The scalar field redistanced on the interface: sin(3x) cos(2y) + 0.5 z^2."""
    return np.asfortranarray(np.sin(3 * x) * np.cos(2 * y) + 0.5 * z**2)


EDGE_CHOICES = (48, 64, 96, 128, 160)


def random_vesicles(count: int = 64, seed: int = 0, half_width: float = 1.2, edges=EDGE_CHOICES):
    """The batched workload: `count` ellipsoids sqrt(x^2/a^2+y^2/b^2+z^2/c^2) - 1 with half
    axes a, b, c ~ U[0.4, 1.0], each on its own box [-half_width, half_width]^3 with node
    counts per axis drawn uniformly from `edges` (anisotropic grids).  Returns a list of
    (xv, yv, zv, axes) -- the coordinate vectors of the columns (x), rows (y) and pages
    (z) and the half axes; `ellipsoid_field` turns one into a field."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx, ny, nz = (int(v) for v in rng.choice(edges, size=3))
        axes = tuple(float(v) for v in rng.uniform(0.4, 1.0, size=3))
        out.append((np.linspace(-half_width, half_width, nx), np.linspace(-half_width, half_width, ny),
                    np.linspace(-half_width, half_width, nz), axes))
    return out


def ellipsoid_field(xv, yv, zv, axes, device=None):
    """Mesh (x, y, z) and field of one batched vesicle (see random_vesicles)."""
    x, y, z = meshgrid(xv, yv, zv, device=device)
    a, b, c = axes
    xp = _Ops(x)
    return x, y, z, xp.fortran(xp.sqrt(x**2 / a**2 + y**2 / b**2 + z**2 / c**2) - 1)
