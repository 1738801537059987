"""Pages-per-block autotuning of the FP32 tiled kernels: the tuner fills the library's
table, the choice changes only the launch shape (results agree to rounding: a block's
first page computes the z smoothness weights directly instead of reusing those of the
page before, which can round differently), and a tuned batch steps the same way through
its graph as through its launch loop."""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def T(pkg, vsl):
    return importlib.import_module(pkg.__name__ + ".autotune")


def make(pkg, size=(40, 36, 52), axes=(0.8, 0.6, 0.7)):
    S = importlib.import_module(pkg.__name__ + ".shapes")
    rows, cols, pges = size
    xv, yv, zv = np.linspace(-1.1, 1.1, cols), np.linspace(-1.0, 1.0, rows), np.linspace(-1.2, 1.2, pges)
    x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes, device="cuda")
    spacing = (float(xv[1] - xv[0]), float(yv[1] - yv[0]), float(zv[1] - zv[0]))
    m = pkg.SDF3(pkg.GD3(x, y, z, spacing=spacing), Val=F, precision="f32")
    m.setDistance()
    return m


def test_tune_shape_fills_table(pkg, T):
    m = make(pkg)
    size = m.GD3.Size
    report = T.tune_shape(m, candidates=(4, 8, 16, 64))
    for kind in T.KINDS:
        assert report[kind]["pages"] in (4, 8, 16, 64)
        assert T.get_pages(size, kind) == report[kind]["pages"]
        assert all(ms > 0 for ms in report[kind]["ms"].values())
    T.clear_shape(size)
    assert all(T.get_pages(size, k) == T.DEFAULT_PAGES for k in T.KINDS)


def test_pages_change_only_the_launch_shape(pkg, T):
    m = make(pkg)
    size = m.GD3.Size
    v = [torch.full_like(m.F, 0.4) for _ in range(3)]
    outs = {}
    for pages in (2, 64):
        for kind in T.KINDS:
            T.set_pages(size, kind, pages)
        outs[pages] = [m.WENO5RK3Reinitialization(m.F, 4), m.WENO5RK3Extend(m.F * 0.5 + 1.0, 4),
                       m.WENO5RK3Advection(m.F, *v, 0.01, 2)]
    T.clear_shape(size)
    for a, b in zip(outs[2], outs[64]):
        diff = float((a.double() - b.double()).abs().max())
        assert diff <= 1e-5 * max(1.0, float(b.double().abs().max())), diff


def same(x, y):
    """bitwise equal, NaN positions included"""
    return torch.equal(torch.isnan(x), torch.isnan(y)) and torch.equal(torch.nan_to_num(x), torch.nan_to_num(y))


def test_tuned_batch_graph_matches_loop(pkg, T):
    B = importlib.import_module(pkg.__name__ + ".batch")
    shapes = [((40, 36, 52), (0.8, 0.6, 0.7)), ((48, 32, 40), (0.7, 0.8, 0.6)), ((40, 36, 52), (0.6, 0.7, 0.8))]
    ext, re = 12, 6
    a = B.VesicleBatch([make(pkg, s, ax) for s, ax in shapes], streams=2)
    b = B.VesicleBatch([make(pkg, s, ax) for s, ax in shapes], streams=2)
    rep = a.autotune(candidates=(4, 16), steps=1, ext_iters=ext, reinit_iters=re)
    assert rep["shapes"] == 2 and rep["kept"] in ("tuned", "default", "uniform")
    # same table for both batches from here on: b starts from a's state (field and cached
    # distances), then one step each way
    for m_a, m_b in zip(a.maps, b.maps):
        m_b.F.copy_(m_a.F)
        for db, da in zip(m_b._dist(), m_a._dist()):
            db.copy_(da)
    torch.cuda.synchronize()
    a2 = [t.clone() for t in a.step(ext, re, 0.5)]
    b2 = [t.clone() for t in b.step_loop(ext, re, 0.5)]
    for x, y in zip(a2, b2):
        assert same(x, y)
        assert torch.all(torch.isfinite(x))
    for m_a, m_b in zip(a.maps, b.maps):
        assert same(m_a.F, m_b.F)
    for s, _ in shapes:
        T.clear_shape(s)
