"""The oracle's SD.GD3 operators (the checker of the GPU's vsl_gradient_* and vsl_laplacian_*)
pinned to their definitions in GD3.m without a GPU:

* Gradient (GD3.m:314-318 over Fx/Fy/Fz, :218-240): (F(next) - F(previous)) / (2 h) along
  x = columns, y = rows, z = pages, where next and previous are the circshift neighbours
  (GD3.m:111-116), so the first and last nodes of an axis are neighbours of each other;
* Laplacian (GD3.m:344-346): (F(next) - 2 F + F(previous)) / h^2 summed over the axes, with
  the same neighbours.

Checked entry by entry with explicit index arithmetic, and on data whose central
differences are exact (linear and quadratic fields in the interior).  CPU only."""
import numpy as np

from oracle import oracle as O


def grid_and_field(shape=(5, 7, 4), seed=3):
    rng = np.random.default_rng(seed)
    g = O.Grid(shape[0], shape[1], shape[2], 0.3, 0.2, 0.45)
    return g, np.asfortranarray(rng.standard_normal(shape))


def test_gradient_entries_use_circshift_neighbours():
    g, f = grid_and_field()
    fx, fy, fz = O.gradient(g, f)
    r, c, p = f.shape
    for i in range(r):
        for j in range(c):
            for k in range(p):
                assert fx[i, j, k] == (f[i, (j + 1) % c, k] - f[i, (j - 1) % c, k]) / (2 * g.dx)
                assert fy[i, j, k] == (f[(i + 1) % r, j, k] - f[(i - 1) % r, j, k]) / (2 * g.dy)
                assert fz[i, j, k] == (f[i, j, (k + 1) % p] - f[i, j, (k - 1) % p]) / (2 * g.dz)


def test_laplacian_entries_use_circshift_neighbours():
    g, f = grid_and_field()
    lap = O.laplacian(g, f)
    r, c, p = f.shape
    for i in range(r):
        for j in range(c):
            for k in range(p):
                fxx = (f[i, (j + 1) % c, k] - 2 * f[i, j, k] + f[i, (j - 1) % c, k]) / (g.dx * g.dx)
                fyy = (f[(i + 1) % r, j, k] - 2 * f[i, j, k] + f[(i - 1) % r, j, k]) / (g.dy * g.dy)
                fzz = (f[i, j, (k + 1) % p] - 2 * f[i, j, k] + f[i, j, (k - 1) % p]) / (g.dz * g.dz)
                assert lap[i, j, k] == fxx + fyy + fzz


def test_central_differences_are_exact_on_polynomials_in_the_interior():
    g = O.Grid(9, 11, 8, 0.25, 0.5, 0.125)
    i, j, k = np.meshgrid(np.arange(9), np.arange(11), np.arange(8), indexing="ij")
    x, y, z = j * g.dx, i * g.dy, k * g.dz  # x along columns, y along rows, z along pages
    fx, fy, fz = O.gradient(g, np.asfortranarray(3 * x - 2 * y + 0.5 * z))
    inner = (slice(1, -1), slice(1, -1), slice(1, -1))
    assert np.allclose(fx[inner], 3.0, rtol=0, atol=1e-12)
    assert np.allclose(fy[inner], -2.0, rtol=0, atol=1e-12)
    assert np.allclose(fz[inner], 0.5, rtol=0, atol=1e-12)
    lap = O.laplacian(g, np.asfortranarray(x * x + 2 * y * y - z * z))
    assert np.allclose(lap[inner], 2.0 + 4.0 - 2.0, rtol=0, atol=1e-9)
