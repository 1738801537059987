"""Many independent vesicles advanced together.

Two batch steps:

* `step_batched` (FP32): vsl_vesicle_step_batch_f32, one launch per RK stage
  running that stage of every vesicle (a work list of all the vesicles' tiles), with the
  per-vesicle set-up passes between them; recorded once as a CUDA graph and replayed.  A
  batch step of 64 vesicles is then ~1,300 launches instead of ~20,000, and the small
  grids share the GPU inside each launch.
* `step` (either precision): one CUDA graph that forks into `streams` parallel branches,
  each vesicle's whole vesicle-step launch sequence recorded on one branch, vesicles dealt
  round-robin.

The vesicles share nothing: each has its own field, distances and workspace.

`reinitialize_batched`, `extend_batched`, `advect_batched` and `redistance_batched` (FP32)
run WENO5RK3Reinitialization, WENO5RK3Extend, WENO5RK3Advection and the closest-point
surface redistance (WENO5 or WENORK3 form) on a list of level sets the same way
(vsl_weno5_rk3_{reinitialization,extend,advection}_batch_f32,
vsl_{weno5_rk3,wenork3}_surface_redistance_batch_f32), bitwise the per-object calls.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import AdvectF32, ExtendF32, RedistanceF32, ReinitF32, VesicleF32, lib
from .sdf3 import SDF3


class VesicleBatch:
    def __init__(self, maps: list[SDF3], streams: int = 8):
        if not maps:
            raise ValueError("empty batch")
        self.maps = list(maps)
        self.nstreams = max(1, min(int(streams), len(self.maps)))
        self._streams = [torch.cuda.Stream() for _ in range(self.nstreams)]
        self._graph = None
        self._key = None
        self.infos = [torch.zeros(4, dtype=torch.float64, device="cuda") for _ in self.maps]
        self._tuning = {}

    def _descriptors(self):
        arr = (VesicleF32 * len(self.maps))()
        for d, m, info in zip(arr, self.maps, self.infos):
            ws = m.workspace("vesicle_step")
            dist = m._dist()
            d.F = m.F.data_ptr()
            d.xpr, d.xpl, d.ypf, d.ypb, d.zpu, d.zpd = (t.data_ptr() for t in dist)
            d.info = info.data_ptr()
            d.rows, d.cols, d.pges = m.GD3.Size
            d.dx, d.dy, d.dz = m.GD3.Dx, m.GD3.Dy, m.GD3.Dz
            d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
        return arr

    def step_batched(self, ext_iters: int = 30, reinit_iters: int = 20, cfl: float = 0.5, graph: bool = True):
        """One batch step with each RK stage of all the vesicles as one launch
        (vsl_vesicle_step_batch_f32; FP32 vesicles only).  graph=True records the step's
        launches once as a CUDA graph and replays it (re-recorded when the arguments
        change); bitwise the results of `step_loop`."""
        if any(m.precision != "f32" for m in self.maps):
            raise ValueError("step_batched runs the FP32 mixed form")
        key = (int(ext_iters), int(reinit_iters), float(cfl))

        def launch():
            arr = self._descriptors()
            lib().call("vsl_vesicle_step_batch_f32", ctypes.addressof(arr), len(self.maps), *key,
                       torch.cuda.current_stream().cuda_stream)

        if not graph:
            launch()
            return self.infos
        if getattr(self, "_bkey", None) != key:
            for m in self.maps:
                m.workspace("vesicle_step")  # allocated before recording
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                launch()
            self._bgraph, self._bkey = g, key
        self._bgraph.replay()
        return self.infos

    def nodes(self) -> int:
        return sum(m.GD3.NumElt for m in self.maps)

    def step_loop(self, ext_iters: int = 30, reinit_iters: int = 20, cfl: float = 0.5):
        """The per-vesicle launch loop: each vesicle's step launched in turn on the current
        stream (the baseline the graph is compared with)."""
        for m, info in zip(self.maps, self.infos):
            m.vesicle_step(ext_iters, reinit_iters, cfl, info=info)
        return self.infos

    def autotune(self, candidates=None, steps: int = 2, ext_iters: int = 30, reinit_iters: int = 20,
                 cfl: float = 0.5, mode: str = "graph") -> dict:
        """Pick pages per block of the tiled kernels for the batch's grid shapes by the
        batch step's own time (graph replay of `step`, mode "graph", or of `step_batched`,
        mode "batched").  Configurations compared: the per-shape choices (each shape timed
        alone on one of its vesicles), every candidate applied to all shapes, and the
        default.  Concurrent vesicles favour other choices than a vesicle timed alone, which
        is why the whole step decides.  Returns the timings and the configuration kept."""
        from . import autotune as T

        cand = T.CANDIDATES if candidates is None else candidates
        shapes = {}
        for m in self.maps:
            shapes.setdefault(tuple(m.GD3.Size), m)
        per_shape = {s: T.tune_shape(m, cand, kinds=T.STEP_KINDS) for s, m in shapes.items()}
        configs = {"tuned": {s: {k: r["pages"] for k, r in c.items()} for s, c in per_shape.items()},
                   "default": {s: {k: 0 for k in T.STEP_KINDS} for s in shapes}}
        for c in cand:
            configs[f"uniform_{c}"] = {s: {k: c for k in T.STEP_KINDS} for s in shapes}

        def apply(cfg):
            for s, kinds in cfg.items():
                for k, p in kinds.items():
                    T.set_pages(s, k, p)

        fn = self.step_batched if mode == "batched" else self.step

        def batch_ms():
            self._graph, self._key = None, None  # re-record with the current table
            self._bgraph, self._bkey = None, None
            fn(ext_iters, reinit_iters, cfl)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(steps):
                fn(ext_iters, reinit_iters, cfl)
            b.record()
            torch.cuda.synchronize()
            return a.elapsed_time(b) / steps

        times = {}
        for name, cfg in configs.items():
            apply(cfg)
            times[name] = batch_ms()
        best = min(times, key=times.get)
        apply(configs[best])
        self._graph, self._key = None, None
        self._bgraph, self._bkey = None, None
        self._tuning = configs
        return {"mode": mode, "shapes": len(shapes), "ms": times, "kept": best.split("_")[0] if best.startswith("uniform") else best,
                "config": best,
                "pages": {"x".join(map(str, s)): v for s, v in configs[best].items()}}

    def apply_tuning(self, name: str) -> None:
        """Put one of the configurations `autotune` compared ("tuned": per-shape choices,
        "default", "uniform_<pages>") back into the library's table."""
        from . import autotune as T

        for s, kinds in self._tuning[name].items():
            for k, p in kinds.items():
                T.set_pages(s, k, p)
        self._graph, self._key = None, None
        self._bgraph, self._bkey = None, None

    def step(self, ext_iters: int = 30, reinit_iters: int = 20, cfl: float = 0.5):
        """One batch step by graph replay (recorded on first use or when arguments change)."""
        key = (int(ext_iters), int(reinit_iters), float(cfl))
        if self._key != key:
            for m in self.maps:
                m.workspace("vesicle_step")  # allocated before recording
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                cap = torch.cuda.current_stream()
                for s in self._streams:
                    s.wait_stream(cap)
                for idx, (m, info) in enumerate(zip(self.maps, self.infos)):
                    with torch.cuda.stream(self._streams[idx % self.nstreams]):
                        m.vesicle_step(*key, info=info)
                for s in self._streams:
                    cap.wait_stream(s)
            self._graph, self._key = g, key
        self._graph.replay()
        return self.infos


def reinitialize_batched(maps: list[SDF3], fields, iteration: int):
    """WENO5RK3Reinitialization(F, iteration) of every (level set, field) pair, each RK stage
    of all of them as one launch (vsl_weno5_rk3_reinitialization_batch_f32; FP32 objects,
    cached distances of setDistance).  Returns new fields, bitwise those of
    `m.WENO5RK3Reinitialization(F, iteration)` per object."""
    maps = list(maps)
    if len(maps) != len(fields):
        raise ValueError("one field per level set")
    if any(m.precision != "f32" for m in maps):
        raise ValueError("reinitialize_batched runs the FP32 mixed form")
    outs = [m._field(F).clone() for m, F in zip(maps, fields)]
    arr = (ReinitF32 * len(maps))()
    keep = []
    for d, m, out in zip(arr, maps, outs):
        ws = m.workspace("reinit_weno5")
        dist = m._dist()
        keep.append((ws, dist))
        d.F = out.data_ptr()
        d.xpr, d.xpl, d.ypf, d.ypb, d.zpu, d.zpd = (t.data_ptr() for t in dist)
        d.rows, d.cols, d.pges = m.GD3.Size
        d.dx, d.dy, d.dz = m.GD3.Dx, m.GD3.Dy, m.GD3.Dz
        d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
    lib().call("vsl_weno5_rk3_reinitialization_batch_f32", ctypes.addressof(arr), len(maps), int(iteration),
               torch.cuda.current_stream().cuda_stream)
    return outs


def extend_batched(maps: list[SDF3], fields, iteration: int):
    """WENO5RK3Extend(C, iteration) of every (level set, field) pair off the level set's zero
    set, each RK stage of all of them as one launch (vsl_weno5_rk3_extend_batch_f32; FP32
    objects, cached distances of setDistance).  Returns new fields, bitwise those of
    `m.WENO5RK3Extend(C, iteration)` per object."""
    maps = list(maps)
    if len(maps) != len(fields):
        raise ValueError("one field per level set")
    if any(m.precision != "f32" for m in maps):
        raise ValueError("extend_batched runs the FP32 mixed form")
    outs = [m._field(C).clone() for m, C in zip(maps, fields)]
    arr = (ExtendF32 * len(maps))()
    keep = []
    for d, m, out in zip(arr, maps, outs):
        ws = m.workspace("extend_weno5")
        dist = m._dist()
        keep.append((ws, dist))
        d.C, d.F = out.data_ptr(), m.F.data_ptr()
        d.xpr, d.xpl, d.ypf, d.ypb, d.zpu, d.zpd = (t.data_ptr() for t in dist)
        d.rows, d.cols, d.pges = m.GD3.Size
        d.dx, d.dy, d.dz = m.GD3.Dx, m.GD3.Dy, m.GD3.Dz
        d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
    lib().call("vsl_weno5_rk3_extend_batch_f32", ctypes.addressof(arr), len(maps), int(iteration),
               torch.cuda.current_stream().cuda_stream)
    return outs


def advect_batched(maps: list[SDF3], fields, velocities, dts, steps: int = 1):
    """WENO5RK3Advection(F, vx, vy, vz, dt, steps) of every level set's grid, each RK stage of
    all of them as one launch (vsl_weno5_rk3_advection_batch_f32; FP32 objects).
    velocities: one (vx, vy, vz) per object; dts: one time step per object (a float or a
    device tensor of one double).  Returns new fields, bitwise those of
    `m.WENO5RK3Advection(F, vx, vy, vz, dt, steps)` per object."""
    maps = list(maps)
    if not (len(maps) == len(fields) == len(velocities) == len(dts)):
        raise ValueError("one field, velocity and time step per level set")
    if any(m.precision != "f32" for m in maps):
        raise ValueError("advect_batched runs the FP32 mixed form")
    outs = [m._field(F).clone() for m, F in zip(maps, fields)]
    arr = (AdvectF32 * len(maps))()
    keep = []
    for d, m, out, vel, dt in zip(arr, maps, outs, velocities, dts):
        v = [m._field(a) for a in vel]
        dtt = dt if isinstance(dt, torch.Tensor) else torch.tensor([float(dt)], dtype=torch.float64, device="cuda")
        ws = m.workspace("advection")
        keep.append((v, dtt, ws))
        d.F = out.data_ptr()
        d.vx, d.vy, d.vz = (t.data_ptr() for t in v)
        d.dt = dtt.data_ptr()
        d.rows, d.cols, d.pges = m.GD3.Size
        d.dx, d.dy, d.dz = m.GD3.Dx, m.GD3.Dy, m.GD3.Dz
        d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
    lib().call("vsl_weno5_rk3_advection_batch_f32", ctypes.addressof(arr), len(maps), int(steps),
               torch.cuda.current_stream().cuda_stream)
    return outs


def redistance_batched(maps: list[SDF3], fields, iter1: int, iter2: int, eno3: bool = False):
    """WENO5RK3ClosetPointSurfaceRedistance(A, iter1, iter2) (eno3: the WENORK3 form) of every
    (level set, field) pair on the level set's zero set, each RK stage of all of them as one
    launch (vsl_weno5_rk3_surface_redistance_batch_f32 / vsl_wenork3_surface_redistance_batch_f32;
    FP32 objects).  Returns new fields, bitwise those of the per-object method."""
    maps = list(maps)
    if len(maps) != len(fields):
        raise ValueError("one field per level set")
    if any(m.precision != "f32" for m in maps):
        raise ValueError("redistance_batched runs the FP32 mixed form")
    op = "surface_redistance_eno3" if eno3 else "surface_redistance"
    fn = "vsl_wenork3_surface_redistance_batch_f32" if eno3 else "vsl_weno5_rk3_surface_redistance_batch_f32"
    outs = [m._field(A).clone() for m, A in zip(maps, fields)]
    arr = (RedistanceF32 * len(maps))()
    keep = []
    for d, m, out in zip(arr, maps, outs):
        ws = m.workspace(op)
        keep.append(ws)
        d.A, d.F = out.data_ptr(), m.F.data_ptr()
        d.rows, d.cols, d.pges = m.GD3.Size
        d.dx, d.dy, d.dz = m.GD3.Dx, m.GD3.Dy, m.GD3.Dz
        d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
    lib().call(fn, ctypes.addressof(arr), len(maps), int(iter1), int(iter2), torch.cuda.current_stream().cuda_stream)
    return outs
