"""Autotuner of the FP32 tiled stage kernels.

Each tiled kernel block marches `pages` pages of the grid (a launch parameter): fewer
pages mean more blocks and more parallelism on small grids, more pages mean fewer halo
reloads per node on large ones.  The library keeps a table of pages per (grid shape,
stage kind) (vsl_set_tile_pages / vsl_tile_pages of the C ABI); `tune_shape` fills it for
one level-set object by timing each kind's own operation (extension, reinitialization,
advection, ENORK2 extension and reinitialization) on that object's field for every candidate, with CUDA events, and keeping
the fastest.  Tune before recording CUDA graphs: a graph keeps the launch shapes it was
recorded with.
"""
from __future__ import annotations

import torch

from ._lib import lib
from .sdf3 import SDF3, colmajor_full

KINDS = {"reinit": 0, "extend": 1, "advect": 2, "enork2_extend": 3, "enork2_reinit": 4}
CANDIDATES = (4, 8, 10, 15, 16, 20, 25, 30, 32, 40, 64)
DEFAULT_PAGES = 20  # pages per block of a shape not in the table
# tile of one block of the tiled kernels, fixed at compile time: 32x4, 32x16 and 64x4 tiles
# gave bitwise the same results and ran -1 % / +4 % / +1 % on the 256^3 vesicle step and
# +1 % / +3 % / +10 % on a batch of 64 vesicles of 48..160 nodes per axis
TILE_ROWS, TILE_COLS = 32, 8
BLOCKS_PER_SM = 4  # resident blocks per SM of the tiled kernels (launch bounds; 5 for the ENORK2 extension)


def wave_candidates(size, sms: int | None = None, fill: float = 0.85, max_waves: float = 4.0, lo: int = 2,
                    hi: int = 64):
    """Pages per block whose launch of at most `max_waves` waves of resident blocks fills
    its last wave to at least `fill` (a launch of 1.42 waves leaves 29% of the second wave
    idle; beyond a few waves the quantization hardly matters), together with CANDIDATES.
    size = (rows, cols, pges)."""
    rows, cols, pges = size
    if sms is None:
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    slots = sms * BLOCKS_PER_SM
    tiles = -(-rows // TILE_ROWS) * -(-cols // TILE_COLS)
    out = set(CANDIDATES)
    for kz in range(lo, hi + 1):
        waves = tiles * -(-pges // kz) / slots
        if waves <= max_waves and waves / -(-waves // 1) >= fill:
            out.add(kz)
    return tuple(sorted(out))


def get_pages(size, kind: str) -> int:
    return int(lib().raw("vsl_tile_pages", *size, KINDS[kind]))


def set_pages(size, kind: str, pages: int) -> None:
    """pages = 0 restores the default."""
    lib().call("vsl_set_tile_pages", *size, KINDS[kind], int(pages))


def set_plane_loads(mode: int) -> None:
    """Plane loads of the tiled kernels, process-wide: 1 TMA tensor copies (where the field
    allows), 0 through registers; the results are the same either way."""
    lib().call("vsl_set_plane_loads", int(mode))


def plane_loads() -> int:
    return int(lib().raw("vsl_plane_loads"))


def tma_wait_timeouts() -> int:
    """Bounded waits for a tensor copy that gave up since the library was loaded (0 unless a
    copy failed to complete)."""
    import ctypes

    n = ctypes.c_uint(0)
    lib().call("vsl_tma_wait_timeouts", ctypes.addressof(n))
    return int(n.value)


def _elapsed_ms(fn, reps: int) -> float:
    fn()  # warm-up (workspace, first launch of the shape)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def _candidates(pges: int, candidates):
    """Candidates that give distinct launch shapes (pages beyond pges all mean one block)."""
    out, seen = [], set()
    for c in sorted(candidates):
        blocks = -(-pges // c)
        if blocks not in seen:
            seen.add(blocks)
            out.append(c)
    return out


# the kinds a vesicle step (and a batch of them) launches
STEP_KINDS = ("reinit", "extend", "advect")


def tune_shape(sdf: SDF3, candidates=CANDIDATES, iters: int = 2, reps: int = 3, kinds=None) -> dict:
    """Pick pages per block for each stage kind on sdf's grid shape; returns
    {kind: {"pages": best, "ms": {candidate: time}}}.  sdf must be FP32 with its
    distances set (setDistance).  candidates="waves" takes wave_candidates(shape); `kinds`
    limits the tuning to those stage kinds (all of KINDS by default)."""
    if sdf.precision != "f32":
        raise ValueError("the tiled kernels are the FP32 form's")
    size = sdf.GD3.Size
    if isinstance(candidates, str):
        if candidates != "waves":
            raise ValueError("candidates: a sequence of page counts or 'waves'")
        candidates = wave_candidates(size)
    v = colmajor_full(size, 0.5, torch.float32)
    dt = 0.1 * min(sdf.GD3.Dx, sdf.GD3.Dy, sdf.GD3.Dz)
    ops = {
        "extend": lambda: sdf.WENO5RK3Extend(sdf.F, iters),
        "reinit": lambda: sdf.WENO5RK3Reinitialization(sdf.F, iters),
        "advect": lambda: sdf.WENO5RK3Advection(sdf.F, v, v, v, dt, iters),
        "enork2_extend": lambda: sdf.ENORK2Extend(sdf.F, iters),
        "enork2_reinit": lambda: sdf.ENORK2Reinitialization(sdf.F, iters),
    }
    report = {}
    for kind, fn in ops.items():
        if kinds is not None and kind not in kinds:
            continue
        times = {}
        for c in _candidates(size[2], candidates):
            set_pages(size, kind, c)
            times[c] = _elapsed_ms(fn, reps)
        best = min(times, key=times.get)
        set_pages(size, kind, best)
        report[kind] = {"pages": best, "ms": times}
    return report


def clear_shape(size) -> None:
    for kind in KINDS:
        set_pages(size, kind, 0)
