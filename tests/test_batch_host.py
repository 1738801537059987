"""Argument checks of the batch of vesicle steps (vsl_vesicle_step_batch_f32) and of the batch
of WENO5 RK3 reinitializations, extensions, advections and surface redistances
(vsl_weno5_rk3_{reinitialization,extend,advection}_batch_f32,
vsl_{weno5_rk3,wenork3}_surface_redistance_batch_f32) without a GPU:
every check runs on the host before any CUDA call, so bad descriptors and arguments are
rejected with their status codes and an empty batch is a no-op."""
import ctypes
import importlib

from conftest import ROOT  # noqa: F401  (puts the repository on sys.path)

L = importlib.import_module("2018_7_vesicle_gb300._lib")

VSL_OK, VSL_ERR_NULL, VSL_ERR_SHAPE, VSL_ERR_VALUE, VSL_ERR_WORKSPACE = 0, 1, 2, 3, 4
FAKE = 0x1000  # never dereferenced: every call below fails its checks first (or has no work)


def descriptor(rows=40, cols=36, pges=32, h=0.05, ws=FAKE * 16, nbytes=1 << 30, **over):
    d = L.VesicleF32()
    d.F = d.xpr = d.xpl = d.ypf = d.ypb = d.zpu = d.zpd = d.info = FAKE
    d.rows, d.cols, d.pges = rows, cols, pges
    d.dx = d.dy = d.dz = h
    d.workspace, d.workspace_bytes = ws, nbytes
    for k, v in over.items():
        setattr(d, k, v)
    return d


def call(vsl, arr, count, ext=30, re=20, cfl=0.5):
    ptr = ctypes.addressof(arr) if arr is not None else None
    return vsl.raw("vsl_vesicle_step_batch_f32", ptr, count, ext, re, cfl, None)


def test_batch_rejects_bad_arguments(vsl):
    arr = (L.VesicleF32 * 1)(descriptor())
    assert call(vsl, None, 1) == VSL_ERR_NULL
    assert call(vsl, arr, -1) == VSL_ERR_VALUE
    assert call(vsl, arr, 1, ext=-1) == VSL_ERR_VALUE
    assert call(vsl, arr, 1, re=-1) == VSL_ERR_VALUE
    assert call(vsl, arr, 1, cfl=0.0) == VSL_ERR_VALUE
    assert call(vsl, arr, 1, cfl=float("nan")) == VSL_ERR_VALUE


def test_batch_rejects_bad_descriptors(vsl):
    good = descriptor()
    for bad, status in ((descriptor(F=None), VSL_ERR_NULL), (descriptor(info=None), VSL_ERR_NULL),
                        (descriptor(rows=0), VSL_ERR_SHAPE), (descriptor(dx=0.0), VSL_ERR_VALUE),
                        (descriptor(ws=None), VSL_ERR_WORKSPACE), (descriptor(nbytes=16), VSL_ERR_WORKSPACE),
                        (descriptor(ws=FAKE + 1), VSL_ERR_WORKSPACE)):
        # the bad member is found wherever it sits, before any vesicle is stepped
        arr = (L.VesicleF32 * 3)(good, bad, good)
        assert call(vsl, arr, 3) == status


def test_empty_batch_is_a_no_op(vsl):
    assert call(vsl, None, 0) == VSL_OK


# ---- the batch of WENO5 RK3 reinitializations (vsl_weno5_rk3_reinitialization_batch_f32) ----


def reinit_member(rows=40, cols=36, pges=32, h=0.05, ws=FAKE * 16, nbytes=1 << 30, **over):
    d = L.ReinitF32()
    d.F = d.xpr = d.xpl = d.ypf = d.ypb = d.zpu = d.zpd = FAKE
    d.rows, d.cols, d.pges = rows, cols, pges
    d.dx = d.dy = d.dz = h
    d.workspace, d.workspace_bytes = ws, nbytes
    for k, v in over.items():
        setattr(d, k, v)
    return d


def reinit_call(vsl, arr, count, iteration=20):
    ptr = ctypes.addressof(arr) if arr is not None else None
    return vsl.raw("vsl_weno5_rk3_reinitialization_batch_f32", ptr, count, iteration, None)


def test_reinit_batch_rejects_bad_arguments(vsl):
    arr = (L.ReinitF32 * 1)(reinit_member())
    assert reinit_call(vsl, None, 1) == VSL_ERR_NULL
    assert reinit_call(vsl, arr, -1) == VSL_ERR_VALUE
    assert reinit_call(vsl, arr, 1, iteration=-1) == VSL_ERR_VALUE
    good = reinit_member()
    for bad, status in ((reinit_member(F=None), VSL_ERR_NULL), (reinit_member(zpd=None), VSL_ERR_NULL),
                        (reinit_member(pges=0), VSL_ERR_SHAPE), (reinit_member(dz=-1.0), VSL_ERR_VALUE),
                        (reinit_member(ws=None), VSL_ERR_WORKSPACE), (reinit_member(nbytes=16), VSL_ERR_WORKSPACE)):
        arr = (L.ReinitF32 * 3)(good, good, bad)
        assert reinit_call(vsl, arr, 3) == status
    assert reinit_call(vsl, None, 0) == VSL_OK


# ---- the batch of WENO5 RK3 extensions (vsl_weno5_rk3_extend_batch_f32) ----


def extend_member(rows=40, cols=36, pges=32, h=0.05, ws=FAKE * 16, nbytes=1 << 30, **over):
    d = L.ExtendF32()
    d.C = d.F = d.xpr = d.xpl = d.ypf = d.ypb = d.zpu = d.zpd = FAKE
    d.rows, d.cols, d.pges = rows, cols, pges
    d.dx = d.dy = d.dz = h
    d.workspace, d.workspace_bytes = ws, nbytes
    for k, v in over.items():
        setattr(d, k, v)
    return d


def extend_call(vsl, arr, count, iteration=30):
    ptr = ctypes.addressof(arr) if arr is not None else None
    return vsl.raw("vsl_weno5_rk3_extend_batch_f32", ptr, count, iteration, None)


def test_extend_batch_rejects_bad_arguments(vsl):
    arr = (L.ExtendF32 * 1)(extend_member())
    assert extend_call(vsl, None, 2) == VSL_ERR_NULL
    assert extend_call(vsl, arr, -1) == VSL_ERR_VALUE
    assert extend_call(vsl, arr, 1, iteration=-1) == VSL_ERR_VALUE
    good = extend_member()
    for bad, status in ((extend_member(C=None), VSL_ERR_NULL), (extend_member(F=None), VSL_ERR_NULL),
                        (extend_member(xpl=None), VSL_ERR_NULL), (extend_member(cols=-3), VSL_ERR_SHAPE),
                        (extend_member(dx=float("nan")), VSL_ERR_VALUE), (extend_member(nbytes=0), VSL_ERR_WORKSPACE)):
        arr = (L.ExtendF32 * 3)(bad, good, good)
        assert extend_call(vsl, arr, 3) == status
    assert extend_call(vsl, None, 0) == VSL_OK


# ---- the batch of WENO5 RK3 advections (vsl_weno5_rk3_advection_batch_f32) ----


def advect_member(rows=40, cols=36, pges=32, h=0.05, ws=FAKE * 16, nbytes=1 << 30, **over):
    d = L.AdvectF32()
    d.F = d.vx = d.vy = d.vz = d.dt = FAKE
    d.rows, d.cols, d.pges = rows, cols, pges
    d.dx = d.dy = d.dz = h
    d.workspace, d.workspace_bytes = ws, nbytes
    for k, v in over.items():
        setattr(d, k, v)
    return d


def advect_call(vsl, arr, count, steps=1):
    ptr = ctypes.addressof(arr) if arr is not None else None
    return vsl.raw("vsl_weno5_rk3_advection_batch_f32", ptr, count, steps, None)


def test_advect_batch_rejects_bad_arguments(vsl):
    arr = (L.AdvectF32 * 1)(advect_member())
    assert advect_call(vsl, None, 1) == VSL_ERR_NULL
    assert advect_call(vsl, arr, -2) == VSL_ERR_VALUE
    assert advect_call(vsl, arr, 1, steps=-1) == VSL_ERR_VALUE
    good = advect_member()
    for bad, status in ((advect_member(F=None), VSL_ERR_NULL), (advect_member(vy=None), VSL_ERR_NULL),
                        (advect_member(dt=None), VSL_ERR_NULL), (advect_member(rows=-1), VSL_ERR_SHAPE),
                        (advect_member(dy=0.0), VSL_ERR_VALUE), (advect_member(ws=None), VSL_ERR_WORKSPACE)):
        arr = (L.AdvectF32 * 2)(good, bad)
        assert advect_call(vsl, arr, 2) == status
    assert advect_call(vsl, None, 0) == VSL_OK


# ---- the batches of surface redistances (vsl_{weno5_rk3,wenork3}_surface_redistance_batch_f32) ----


def redistance_member(rows=40, cols=36, pges=32, h=0.05, ws=FAKE * 16, nbytes=1 << 30, **over):
    d = L.RedistanceF32()
    d.A = d.F = FAKE
    d.rows, d.cols, d.pges = rows, cols, pges
    d.dx = d.dy = d.dz = h
    d.workspace, d.workspace_bytes = ws, nbytes
    for k, v in over.items():
        setattr(d, k, v)
    return d


def test_redistance_batches_reject_bad_arguments(vsl):
    for fn in ("vsl_weno5_rk3_surface_redistance_batch_f32", "vsl_wenork3_surface_redistance_batch_f32"):
        def call(arr, count, it1=2, it2=3):
            ptr = ctypes.addressof(arr) if arr is not None else None
            return vsl.raw(fn, ptr, count, it1, it2, None)

        arr = (L.RedistanceF32 * 1)(redistance_member())
        assert call(None, 1) == VSL_ERR_NULL
        assert call(arr, -1) == VSL_ERR_VALUE
        assert call(arr, 1, it1=-1) == VSL_ERR_VALUE
        assert call(arr, 1, it2=-1) == VSL_ERR_VALUE
        good = redistance_member()
        for bad, status in ((redistance_member(A=None), VSL_ERR_NULL), (redistance_member(F=None), VSL_ERR_NULL),
                            (redistance_member(pges=0), VSL_ERR_SHAPE), (redistance_member(dx=0.0), VSL_ERR_VALUE),
                            (redistance_member(nbytes=64), VSL_ERR_WORKSPACE)):
            arr = (L.RedistanceF32 * 2)(good, bad)
            assert call(arr, 2) == status
        assert call(None, 0) == VSL_OK


def test_python_batch_wrappers_check_their_arguments():
    """batch.*_batched reject mismatched lists and FP64 objects before any device work."""
    import types

    import pytest

    Bm = importlib.import_module("2018_7_vesicle_gb300.batch")
    f32, f64 = types.SimpleNamespace(precision="f32"), types.SimpleNamespace(precision="f64")
    with pytest.raises(ValueError, match="one field"):
        Bm.reinitialize_batched([f32, f32], [None], 3)
    with pytest.raises(ValueError, match="FP32"):
        Bm.reinitialize_batched([f64], [None], 3)
    with pytest.raises(ValueError, match="one field"):
        Bm.extend_batched([f32], [None, None], 3)
    with pytest.raises(ValueError, match="FP32"):
        Bm.extend_batched([f32, f64], [None, None], 3)
    with pytest.raises(ValueError, match="one field, velocity and time step"):
        Bm.advect_batched([f32], [None], [], [0.1])
    with pytest.raises(ValueError, match="FP32"):
        Bm.advect_batched([f64], [None], [None], [0.1])
    with pytest.raises(ValueError, match="one field"):
        Bm.redistance_batched([f32], [], 2, 3)
    with pytest.raises(ValueError, match="FP32"):
        Bm.redistance_batched([f64], [None], 2, 3, eno3=True)
