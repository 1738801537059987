"""Batched vesicles: the graph with parallel branches gives bitwise the results of the
per-vesicle launch loop.  GPU only."""
import importlib

import numpy as np
import pytest

from gpu_util import dev, host

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


def oracle_steps(O, K, x, y, z, F, steps, ext, re):
    g = O.grid_from_mesh(x, y, z)
    d = O.set_distance(K, g, F)
    for _ in range(steps):
        F, d, info = O.vesicle_step(K, g, F, d, ext, re, 0.5)
    return g, F, info


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_batch_members_match_the_oracle(pkg, vsl, oracle_mod, precision):
    """Every member of a graph-replayed batch against the oracle's steps of the same vesicle:
    bitwise against the oracle built with integer powers rounded once (FP64 form), within
    1e-5 dx over the band |phi| < 3 dx (FP32 form)."""
    O = oracle_mod
    K = O.kernels("port_crpow")
    vs = S.random_vesicles(3, seed=5, edges=(24, 32, 40))
    fields = [S.ellipsoid_field(xv, yv, zv, axes) for xv, yv, zv, axes in vs]
    maps = []
    for x, y, z, F in fields:
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision=precision)
        m.setDistance()
        maps.append(m)
    batch = B.VesicleBatch(maps, streams=2)
    for _ in range(2):
        infos = [i.cpu().numpy().copy() for i in batch.step(8, 5, 0.5)]
    for (x, y, z, F), m, info in zip(fields, maps, infos):
        g, Fo, oi = oracle_steps(O, K, x, y, z, F, 2, 8, 5)
        got = host(m.F)
        if precision == "f64":
            assert np.array_equal(got, Fo)
            assert info[2] == oi["dt"]
        else:
            band = np.abs(Fo) < 3 * g.dx
            assert np.max(np.abs(got[band] - Fo[band])) <= 1e-5 * g.dx
            assert abs(info[2] / oi["dt"] - 1) <= 1e-5


def test_edge_mix_with_tuned_pages(pkg, vsl, oracle_mod):
    """The batched workload's edge mix {48, 64, 96, 128, 160} with a non-default pages-per-block
    table for every shape (as the autotuner leaves it): the graph replay equals the launch
    loop bit for bit, and the smallest member (FP32) is within 1e-5 dx of the oracle."""
    T = importlib.import_module("2018_7_vesicle_gb300.autotune")
    O = oracle_mod
    vs = S.random_vesicles(4, seed=7)
    fields = [S.ellipsoid_field(xv, yv, zv, axes) for xv, yv, zv, axes in vs]
    shapes = {f[3].shape for f in fields}
    assert len(shapes) > 1
    pages = {"reinit": 7, "extend": 13, "advect": 9}
    try:
        for sz in shapes:
            for kind, p in pages.items():
                T.set_pages(sz, kind, p)

        def make():
            out = []
            for x, y, z, F in fields:
                m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
                m.setDistance()
                out.append(m)
            return out

        loop = B.VesicleBatch(make(), streams=2)
        graph = B.VesicleBatch(make(), streams=2)
        a = [i.cpu().numpy().copy() for i in loop.step_loop(30, 20, 0.5)]
        b = [i.cpu().numpy().copy() for i in graph.step(30, 20, 0.5)]
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
        for m1, m2 in zip(loop.maps, graph.maps):
            assert np.array_equal(host(m1.F), host(m2.F))
        q = min(range(len(fields)), key=lambda t: fields[t][3].size)
        x, y, z, F = fields[q]
        g, Fo, oi = oracle_steps(O, O.kernels("port"), x, y, z, F, 1, 30, 20)
        got = host(graph.maps[q].F)
        band = np.abs(Fo) < 3 * g.dx
        err = float(np.max(np.abs(got[band] - Fo[band]))) / g.dx
        print(f"\nsmallest member {F.shape}: band max {err:.2e} dx")
        assert err <= 1e-5
    finally:
        for sz in shapes:
            for kind in pages:
                T.set_pages(sz, kind, 0)


@pytest.mark.parametrize("count,edges,iters", [(5, (24, 32, 40), (8, 5)), (66, (16, 20, 24), (4, 3))])
def test_batched_stages_match_loop(pkg, vsl, count, edges, iters):
    """vsl_vesicle_step_batch_f32 (each RK stage of all the vesicles as one launch;
    66 vesicles run as two launches' worth, 64 + 2) gives bitwise the per-vesicle steps,
    as a graph replay and as direct launches, over two batch steps."""
    loop = B.VesicleBatch(make_batch_edges(pkg, count, edges), streams=2)
    graph = B.VesicleBatch(make_batch_edges(pkg, count, edges), streams=2)
    direct = B.VesicleBatch(make_batch_edges(pkg, count, edges), streams=2)
    for _ in range(2):
        a = [i.cpu().numpy().copy() for i in loop.step_loop(*iters, 0.5)]
        b = [i.cpu().numpy().copy() for i in graph.step_batched(*iters, 0.5)]
        c = [i.cpu().numpy().copy() for i in direct.step_batched(*iters, 0.5, graph=False)]
        for u, v, w in zip(a, b, c):
            assert np.array_equal(u, v) and np.array_equal(u, w)
    for m1, m2, m3 in zip(loop.maps, graph.maps, direct.maps):
        f = host(m1.F)
        assert np.array_equal(f, host(m2.F)) and np.array_equal(f, host(m3.F))


def make_batch_edges(pkg, n, edges):
    maps = []
    for xv, yv, zv, axes in S.random_vesicles(n, seed=11, edges=edges):
        x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes)
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
        m.setDistance()
        maps.append(m)
    return maps


@pytest.mark.parametrize("count", [5, 66])
def test_reinitialize_batched_matches_per_object(pkg, vsl, count):
    """vsl_weno5_rk3_reinitialization_batch_f32 (each RK stage of every member as one
    launch; 66 members run as chunks of 64 and 2) against each object's own
    WENO5RK3Reinitialization: bitwise."""
    edges = (24, 32, 40) if count < 10 else (16, 20, 24)
    maps = []
    for xv, yv, zv, axes in S.random_vesicles(count, seed=4, edges=edges):
        x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes)
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
        m.setDistance()
        maps.append(m)
    fields = [m.F for m in maps]
    got = B.reinitialize_batched(maps, fields, 6)
    for m, F, g in zip(maps, fields, got):
        assert np.array_equal(host(g), host(m.WENO5RK3Reinitialization(F, 6)))
    assert len({m.GD3.Size for m in maps}) > 1


@pytest.mark.parametrize("count", [5, 66])
def test_extend_batched_matches_per_object(pkg, vsl, count):
    """vsl_weno5_rk3_extend_batch_f32 (each RK stage of every member, band blocks included,
    as one launch; 66 members run as chunks of 64 and 2) against each object's own
    WENO5RK3Extend: bitwise."""
    edges = (24, 32, 40) if count < 10 else (16, 20, 24)
    maps, fields = [], []
    for xv, yv, zv, axes in S.random_vesicles(count, seed=6, edges=edges):
        x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes)
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
        m.setDistance()
        maps.append(m)
        fields.append(dev(np.sin(3 * x) * np.cos(2 * y) + z))
    got = B.extend_batched(maps, fields, 8)
    for m, C, g in zip(maps, fields, got):
        assert np.array_equal(host(g), host(m.WENO5RK3Extend(C, 8)))


@pytest.mark.parametrize("count", [5, 66])
def test_advect_batched_matches_per_object(pkg, vsl, count):
    """vsl_weno5_rk3_advection_batch_f32 (each RK stage of every member as one launch; 66
    members run as chunks of 64 and 2) against each object's own WENO5RK3Advection, two steps
    of a rotation-plus-shear velocity with each member's own time step: bitwise."""
    edges = (24, 32, 40) if count < 10 else (16, 20, 24)
    maps, vels, dts = [], [], []
    for q, (xv, yv, zv, axes) in enumerate(S.random_vesicles(count, seed=8, edges=edges)):
        x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes)
        m = pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32")
        maps.append(m)
        vels.append((dev(-y + 0.2 * z), dev(x), dev(0.3 * np.sin(2 * x))))
        dts.append(0.3 * float(xv[1] - xv[0]) * (1 + 0.01 * q))
    fields = [m.F for m in maps]
    got = B.advect_batched(maps, fields, vels, dts, 2)
    for m, F, v, dt, g in zip(maps, fields, vels, dts, got):
        assert np.array_equal(host(g), host(m.WENO5RK3Advection(F, *v, dt, 2)))


@pytest.mark.parametrize("eno3", [False, True])
@pytest.mark.parametrize("count", [5, 66])
def test_redistance_batched_matches_per_object(pkg, vsl, count, eno3):
    """vsl_{weno5_rk3,wenork3}_surface_redistance_batch_f32 (each RK stage of every member's
    extensions and reinitialization as one launch; 66 members run as chunks of 64 and 2)
    against each object's own closest-point surface redistance: bitwise."""
    edges = (24, 32, 40) if count < 10 else (16, 20, 24)
    maps, fields = [], []
    for xv, yv, zv, axes in S.random_vesicles(count, seed=10, edges=edges):
        x, y, z, F = S.ellipsoid_field(xv, yv, zv, axes)
        maps.append(pkg.SDF3(pkg.GD3(x, y, z), Val=F, precision="f32"))
        fields.append(dev(np.exp(z) - 1 + 0.1 * x))
    got = B.redistance_batched(maps, fields, 2, 3, eno3=eno3)
    for m, A, g in zip(maps, fields, got):
        method = m.WENORK3ClosetPointSurfaceRedistance if eno3 else m.WENO5RK3ClosetPointSurfaceRedistance
        assert np.array_equal(host(g), host(method(A, 2, 3)))
