"""vsl_area_volume_noalloc_f64, the area/volume reduction that allocates nothing and keeps
its partial sums in a static device array, against vsl_area_volume_f64 (caller workspace).

Both run the same toolbox and fixed-order sum kernels, so the tolerance is zero: the two
results must be bitwise equal.  Two calls in a row on different grids (the larger first)
check that the second call is not affected by what the first left in the shared array.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import dev, ptr, stream

VSL_ERR_SCRATCH_LIMIT = 7
SCRATCH_BYTES = 1 << 20


def field(shape, axes, center, seed):
    rows, cols, pges = shape
    x = np.linspace(-1.5, 1.5, cols)
    y = np.linspace(-1.4, 1.4, rows)
    z = np.linspace(-1.3, 1.3, pges)
    Y, X, Z = np.meshgrid(y, x, z, indexing="ij")
    a, b, c = axes
    F = np.sqrt(((X - center[0]) / a) ** 2 + ((Y - center[1]) / b) ** 2 + ((Z - center[2]) / c) ** 2) - 1.0
    F += 0.01 * np.random.default_rng(seed).standard_normal(F.shape)
    return F, (x[1] - x[0], y[1] - y[0], z[1] - z[0])


def test_noalloc_rejects_grids_beyond_the_scratch(vsl):
    """ceil(rows/32) * ceil(cols/8) * pges partial pairs must fit in the 1 MiB array; the
    check comes before any CUDA call (no GPU needed)."""
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the call is rejected first
    blocks = lambda r, c, p: -(-r // 32) * -(-c // 8) * p
    assert blocks(264, 256, 256) * 16 > SCRATCH_BYTES
    st = vsl.raw("vsl_area_volume_noalloc_f64", fake, fake, 264, 256, 256, 0.01, 0.01, 0.01, None)
    assert st == VSL_ERR_SCRATCH_LIMIT
    assert "static scratch" in vsl.status_string(st)
    assert vsl.raw("vsl_area_volume_noalloc_f64", None, fake, 8, 8, 8, 0.1, 0.1, 0.1, None) == 1


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point(vsl):
    import torch

    cases = [
        ((200, 184, 120), (0.9, 0.7, 0.55), (0.1, -0.05, 0.02), 1),  # 7*23*120 = 19320 blocks
        ((48, 40, 56), (0.6, 0.8, 0.5), (-0.1, 0.05, 0.0), 2),  # 2*5*56 = 560 blocks
    ]
    fields, outs = [], []
    s = stream()
    # two no-allocation calls in a row, the larger grid first
    for shape, axes, center, seed in cases:
        F, (dx, dy, dz) = field(shape, axes, center, seed)
        Fd = dev(F)
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        vsl.call("vsl_area_volume_noalloc_f64", ptr(Fd), ptr(out), *shape, dx, dy, dz, s)
        fields.append((Fd, shape, (dx, dy, dz)))
        outs.append(out)
    torch.cuda.synchronize()
    for (Fd, shape, h), out in zip(fields, outs):
        ws_bytes = vsl.workspace_bytes("area_volume", *shape, 8)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        ref = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        vsl.call("vsl_area_volume_f64", ptr(Fd), ptr(ref), *shape, *h, ptr(ws), ws_bytes, s)
        torch.cuda.synchronize()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(want)) and want[0] > 0 and want[1] > 0
        assert np.array_equal(got, want), (shape, got, want)
