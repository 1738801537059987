"""Many independent vesicles advanced together.

A batch step is one CUDA graph: the graph forks into `streams` parallel branches and each
vesicle's whole vesicle-step launch sequence (toolbox, extension, time step, advection,
setDistance, reinitialization) is recorded on one branch, vesicles dealt round-robin.
Small grids, which cannot fill the GPU alone, then run concurrently, and the host issues
one graph launch per batch step instead of a few hundred launches per vesicle.  The
vesicles share nothing: each has its own field, distances and workspace.
"""
from __future__ import annotations

import torch

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

    def nodes(self) -> int:
        return sum(m.GD3.NumElt for m in self.maps)

    def step_loop(self, ext_iters: int = 30, reinit_iters: int = 20, cfl: float = 0.5):
        """The per-vesicle launch loop: each vesicle's step launched in turn on the current
        stream (the baseline the graph is compared with)."""
        for m, info in zip(self.maps, self.infos):
            m.vesicle_step(ext_iters, reinit_iters, cfl, info=info)
        return self.infos

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
