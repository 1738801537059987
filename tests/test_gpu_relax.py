"""The single-phase relaxation step of the vesicle driver (p00_test_singlephase_relax.m:
60-196) and its SD.GD3 operators on the GPU, against the oracle.

* GD3.Laplacian (periodic 7-point) and GD3.Gradient (periodic central differences):
  bitwise equal to the oracle's numpy restatement;
* GD3.smoothGMRES: the GPU's exact spectral solve of (I + alpha Dt L^2) x = rhs against
  the reference's own algorithm, GMRES with the FFT preconditioner to relative
  tolerance 1e-12 (scipy), within 1e-9 of max|x|, and against a numpy direct spectral
  solve within 1e-12;
* GD3.smoothFFT: against numpy's FFTs within 1e-12, on an odd-sized grid too (the
  reference's half-integer wave numbers there);
* one relaxation step, FP64: against the oracle's composition within 1e-9 (field,
  relative to max|F|) and 1e-8 (the scalars: area, volume, Dt, the integrals, tension,
  pressure, energy); the differences come from summation order and the GMRES tolerance;
* the FP32 step against the FP64 step, the bounds of the composite vesicle step: field
  within 1e-3 dx at the worst node and 2e-5 dx RMS over the band |phi| < 3 dx, area and
  volume within 1e-6.
GPU only."""
import importlib

import numpy as np
import pytest
import torch

from gpu_util import dev, host

pytestmark = pytest.mark.gpu
S = importlib.import_module("2018_7_vesicle_gb300.shapes")


def grid_and_field(pkg, size=(28, 26, 24), axes=(0.75, 0.6, 0.5)):
    rows, cols, pges = size
    xv, yv, zv = np.linspace(-1, 1, cols), np.linspace(-0.9, 0.9, rows), np.linspace(-0.8, 0.8, pges)
    x, y, z = S.meshgrid(xv, yv, zv)
    F = np.sqrt(x**2 / axes[0] ** 2 + y**2 / axes[1] ** 2 + z**2 / axes[2] ** 2) - 1
    return pkg.GD3(x, y, z), x, y, z, np.asfortranarray(F)


def test_periodic_laplacian(pkg, vsl, oracle_mod):
    O = oracle_mod
    gd, x, y, z, F = grid_and_field(pkg)
    g = O.grid_from_mesh(x, y, z)
    f = np.asfortranarray(np.sin(3 * x) * np.cos(2 * y + z) + F)
    got = host(gd.Laplacian(dev(f)))
    assert np.array_equal(got, O.laplacian(g, f))
    got32 = host(gd.Laplacian(dev(f), precision="f32"))
    ref = O.laplacian(g, f)
    assert np.abs(got32 - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("size", [(28, 26, 24), (3, 2, 5)])
def test_periodic_gradient(pkg, vsl, oracle_mod, size):
    """GD3.Gradient: bitwise the oracle in FP64 (grids down to 2 nodes on an axis, where both
    periodic neighbours are the same node), within 1e-6 of max|grad| in FP32."""
    O = oracle_mod
    gd, x, y, z, F = grid_and_field(pkg, size)
    g = O.grid_from_mesh(x, y, z)
    f = np.asfortranarray(np.sin(3 * x) * np.cos(2 * y + z) + F)
    ref = O.gradient(g, f)
    for got, r in zip(gd.Gradient(dev(f)), ref):
        assert np.array_equal(host(got), r)
    for got, r in zip(gd.Gradient(dev(f), precision="f32"), ref):
        assert np.abs(host(got) - r).max() <= 1e-6 * max(np.abs(r).max(), 1.0)


@pytest.mark.parametrize("size", [(28, 26, 24), (21, 19, 17)])
def test_smoothing(pkg, vsl, oracle_mod, size):
    O = oracle_mod
    gd, x, y, z, F = grid_and_field(pkg, size)
    g = O.grid_from_mesh(x, y, z)
    rhs = np.asfortranarray(np.exp(-4 * F**2) * np.cos(5 * x) + 0.1 * np.random.default_rng(0).standard_normal(F.shape))
    dt, alpha = 1e-5, 0.5
    got = host(gd.smoothGMRES(dev(rhs), dt, alpha))
    ref = O.smooth_gmres(g, rhs, dt, alpha)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
    # the same system solved directly with numpy's FFTs and the discrete symbol
    n = [np.arange(m) for m in (g.rows, g.cols, g.pges)]
    ly = (2 * np.cos(2 * np.pi * n[0] / g.rows) - 2) / (g.dy * g.dy)
    lx = (2 * np.cos(2 * np.pi * n[1] / g.cols) - 2) / (g.dx * g.dx)
    lz = (2 * np.cos(2 * np.pi * n[2] / g.pges) - 2) / (g.dz * g.dz)
    lam = lx[None, :, None] + ly[:, None, None] + lz[None, None, :]
    direct = np.real(np.fft.ifftn(np.fft.fftn(rhs) / (1 + alpha * dt * lam**2)))
    assert np.abs(got - direct).max() <= 1e-12 * np.abs(direct).max()
    got = host(gd.smoothFFT(dev(rhs), dt, alpha))
    ref = O.smooth_fft(g, rhs, dt, alpha)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    got32 = host(gd.smoothGMRES(dev(rhs), dt, alpha, precision="f32"))
    assert np.abs(got32 - direct).max() <= 1e-5 * np.abs(direct).max()


def relax_setup(pkg, precision, F, x, y, z):
    m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision=precision)
    m.setDistance()
    av = m.area_volume().cpu().numpy()
    return m, float(av[0]), float(av[1])


def test_relax_step_fp64_vs_oracle(pkg, vsl, oracle_mod):
    O = oracle_mod
    K = O.kernels("port")
    gd, x, y, z, F = grid_and_field(pkg)
    g = O.grid_from_mesh(x, y, z)
    m, A0, V0 = relax_setup(pkg, "f64", F, x, y, z)
    A0, V0 = 1.001 * A0, 0.999 * V0  # targets away from the current values: nonzero correction terms
    params = dict(kappa=1.0, spon_c=-2.0, cfl=0.5, alpha=0.5, ext_iters=20, reinit_iters=3)
    Fo = F
    for _ in range(2):
        info = m.relax_step(A0, V0, **params).cpu().numpy()
        Fo, dist, oinfo = O.relax_step(K, g, Fo, A0, V0, **params)
        assert np.all(np.abs(info - oinfo) <= 1e-8 * np.maximum(np.abs(oinfo), 1e-300)), (info, oinfo)
        got = host(m.F)
        assert np.abs(got - Fo).max() <= 1e-9 * np.abs(Fo).max()


def test_relax_step_fp32_vs_fp64(pkg, vsl):
    gd, x, y, z, F = grid_and_field(pkg)
    m64, A0, V0 = relax_setup(pkg, "f64", F, x, y, z)
    m32, _, _ = relax_setup(pkg, "f32", F, x, y, z)
    params = dict(kappa=1.0, spon_c=0.0, cfl=0.5, alpha=0.5, ext_iters=20, reinit_iters=3)
    for _ in range(2):
        i64 = m64.relax_step(A0, V0, **params).cpu().numpy()
        i32 = m32.relax_step(A0, V0, **params).cpu().numpy()
        dx = float(x[0, 1, 0] - x[0, 0, 0])
        d = (m32.F.double() - m64.F).abs()
        band = m64.F.abs() < 3 * dx
        err, rms = float(d.max()) / dx, float(d[band].pow(2).mean().sqrt()) / dx
        print("relax FP32 vs FP64: field max", err, "dx, band rms", rms, "dx; area/volume rel",
              abs(i32[0] / i64[0] - 1), abs(i32[1] / i64[1] - 1))
        assert err <= 1e-3 and rms <= 2e-5
        assert abs(i32[0] / i64[0] - 1) <= 1e-6 and abs(i32[1] / i64[1] - 1) <= 1e-6


def test_relax_step_graph_replay_is_bitwise(pkg, vsl):
    """graph=True records the step once and replays it: same fields and scalars, bit for
    bit, as the direct launches, over three steps (FP32, the driver's initial shape)."""
    x, y, z, F = S.oblate_ellipsoid((32, 30, 28), 0.6, 0.35)
    ms = []
    for graph in (False, True):
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
        m.setDistance()
        av = m.area_volume().cpu().numpy()
        infos = []
        for _ in range(3):
            infos.append(m.relax_step(av[0], av[1], cfl=0.5, ext_iters=10, reinit_iters=5, graph=graph)
                         .cpu().numpy())
        ms.append((host(m.F), np.array(infos)))
    assert np.array_equal(ms[0][0], ms[1][0])
    assert np.array_equal(ms[0][1], ms[1][1])
