"""Helpers of the GPU parity tests: column-major device fields and comparisons."""
import numpy as np
import torch


def dev(a, dtype=torch.float64):
    """numpy (rows, cols, pges) array -> column-major CUDA tensor (the reference layout)."""
    a = np.asarray(a)
    r, c, p = a.shape
    if a.dtype == np.bool_:
        t = torch.from_numpy(a.ravel(order="F").copy()).view(p, c, r)
        return t.to("cuda").permute(2, 1, 0)
    t = torch.from_numpy(np.asarray(a, np.float64).ravel(order="F").copy()).view(p, c, r)
    return t.to(device="cuda", dtype=dtype).permute(2, 1, 0)


def empty(shape, dtype=torch.float64, fill=None):
    r, c, p = shape
    t = torch.empty((p, c, r), dtype=dtype, device="cuda").permute(2, 1, 0)
    if fill is not None:
        t.fill_(fill)
    return t


def host(t):
    torch.cuda.synchronize()
    return np.asfortranarray(t.detach().to("cpu", torch.float64).numpy())


def ptr(t):
    return t.data_ptr()


def stream():
    return torch.cuda.current_stream().cuda_stream


def max_rel(a, b, scale=None):
    """max |a - b| relative to max(|b|, 1) (or a given scale)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    s = scale if scale is not None else max(1.0, float(np.max(np.abs(b))))
    return float(np.max(np.abs(a - b))) / s if a.size else 0.0
