"""Batched vesicles: the graph with parallel branches gives bitwise the results of the
per-vesicle launch loop.  GPU only."""
import importlib

import numpy as np
import pytest

from gpu_util import host

pytestmark = pytest.mark.gpu

S = importlib.import_module("2018_7_vesicle_gb300.shapes")
B = importlib.import_module("2018_7_vesicle_gb300.batch")


def make_batch(pkg, n, precision):
    maps = []
    for xv, yv, zv, axes in S.random_vesicles(n, seed=2, edges=(24, 32, 40)):
        x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes)
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision=precision)
        m.setDistance()
        maps.append(m)
    return maps


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_batch_graph_matches_loop(pkg, vsl, precision):
    loop = B.VesicleBatch(make_batch(pkg, 6, precision), streams=3)
    graph = B.VesicleBatch(make_batch(pkg, 6, precision), streams=3)
    for _ in range(2):
        a = [i.cpu().numpy().copy() for i in loop.step_loop(8, 5, 0.5)]
        b = [i.cpu().numpy().copy() for i in graph.step(8, 5, 0.5)]
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
    for m1, m2 in zip(loop.maps, graph.maps):
        assert np.array_equal(host(m1.F), host(m2.F))
    # anisotropic grids really are anisotropic
    assert len({m.GD3.Size for m in loop.maps}) > 1
