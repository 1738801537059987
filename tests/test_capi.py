"""The C ABI library without a GPU: it loads, exports every entry point declared in
include/vsl_gb300.h with the declared arity, and rejects bad arguments with the documented
status before launching anything."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "vsl_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|size_t|const char \*)\s*(vsl_\w+)\s*\(([^;]*?)\);", text, flags=re.S):
        params = [p for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = len(params)
    return out


def test_header_declares_entry_points():
    d = declared()
    assert "vsl_re_step" in d and "vsl_vesicle_step_f32" in d
    assert len(d) >= 30


def test_header_is_plain_c(tmp_path):
    """The header serves C callers (a MEX gateway, cgo): it compiles as strict C99."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include "vsl_gb300.h"\nint main(void) { return VSL_OP_SURFACE_REDISTANCE_ENO3 == 20 ? 0 : 1; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I" + os.path.dirname(HEADER),
                        "-c", str(src), "-o", str(tmp_path / "use_header.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_library_exports_every_declared_symbol(vsl):
    lib = ctypes.CDLL(vsl.path)
    for name in declared():
        assert hasattr(lib, name), f"{name} not exported"


def test_bindings_match_header_arity(pkg):
    from importlib import import_module

    sigs = import_module(pkg.__name__ + "._lib").SIGNATURES
    d = declared()
    for name, sig in sigs.items():
        assert name in d, f"{name} bound but not declared"
        assert len(sig) == d[name], f"{name}: {len(sig)} bound vs {d[name]} declared"
    for name in d:
        if name not in ("vsl_status_string", "vsl_version", "vsl_workspace_bytes"):
            assert name in sigs, f"{name} declared but not bound"


def test_status_strings(vsl):
    assert vsl.status_string(0) == "ok"
    for st in range(1, 7):
        assert vsl.status_string(st) != "unknown status"
    assert vsl.lib.vsl_version() == 1


FAKE = 0x1000  # never dereferenced: every call below fails its checks first


def test_null_pointer_rejected(vsl):
    st = vsl.raw("vsl_re_step", 0, FAKE, FAKE, FAKE, *[FAKE] * 6, 8, 8, 8, 0.1, 0.1, 0.1, 512, None)
    assert st == 1
    st = vsl.raw("vsl_weno5_rk3_reinitialization_f32", 0, 3, *[FAKE] * 6, 8, 8, 8, 0.1, 0.1, 0.1, FAKE, 1 << 20, None)
    assert st == 1


def test_shape_checks(vsl):
    # num_ele inconsistent with rows*cols*pges
    st = vsl.raw("vsl_boundary_location", *[FAKE] * 7, 511, 8, 8, 8, 0.1, 0.1, 0.1, None)
    assert st == 2
    st = vsl.raw("vsl_boundary_location", *[FAKE] * 7, 0, 0, 8, 8, 0.1, 0.1, 0.1, None)
    assert st == 2
    st = vsl.raw("vsl_set_distance_f64", *[FAKE] * 7, 8, -1, 8, 0.1, 0.1, 0.1, FAKE, 1 << 20, None)
    assert st == 2
    # non-positive spacing
    st = vsl.raw("vsl_set_distance_f64", *[FAKE] * 7, 8, 8, 8, 0.1, 0.0, 0.1, FAKE, 1 << 20, None)
    assert st == 3
    # workspace too small for the edge lists
    st = vsl.raw("vsl_set_distance_f32", *[FAKE] * 7, 8, 8, 8, 0.1, 0.1, 0.1, FAKE, 64, None)
    assert st == 4


def test_value_and_workspace_checks(vsl):
    n = vsl.workspace_bytes("reinit_weno5", 8, 8, 8, 8)
    st = vsl.raw("vsl_weno5_rk3_reinitialization_f64", FAKE, -1, *[FAKE] * 6, 8, 8, 8, 0.1, 0.1, 0.1, FAKE, n, None)
    assert st == 3
    st = vsl.raw("vsl_weno5_rk3_reinitialization_f64", FAKE, 2, *[FAKE] * 6, 8, 8, 8, 0.1, 0.1, 0.1, 0, n, None)
    assert st == 4
    st = vsl.raw("vsl_weno5_rk3_reinitialization_f64", FAKE, 2, *[FAKE] * 6, 8, 8, 8, 0.1, 0.1, 0.1, FAKE, n - 1, None)
    assert st == 4
    st = vsl.raw("vsl_weno5_rk3_reinitialization_f64", FAKE, 2, *[FAKE] * 6, 8, 8, 8, 0.1, 0.1, 0.1, FAKE + 8, n, None)
    assert st == 4
    st = vsl.raw("vsl_vesicle_step_f32", *[FAKE] * 7, 3, 3, -0.5, FAKE, 8, 8, 8, 0.1, 0.1, 0.1, FAKE, 1 << 30, None)
    assert st == 3


def test_workspace_sizes(vsl):
    # FP64 per node; the FP32 extensions keep FP64 crossing values (6) and three FP64
    # shadow fields of the band beside their FP32 velocity (3) and stage fields (2)
    ext32 = 5 * 4 + 9 * 8 + 1
    for op, per_node_min, min32 in (("reinit_weno5", 2 * 8 + 1, None), ("reinit_eno3", 8 * 8 + 1, None),
                                    ("extend_weno5", 11 * 8 + 1, ext32), ("surface_redistance", 25 * 8 + 2, ext32),
                                    ("surface_redistance_eno3", 25 * 8 + 2, ext32),
                                    ("advection", 2 * 8, None), ("vesicle_step", 15 * 8 + 1, ext32),
                                    ("reinit_tol", 2 * 8 + 1, None)):
        n = vsl.workspace_bytes(op, 32, 24, 16, 8)
        assert n >= per_node_min * 32 * 24 * 16, op
        assert n % 256 == 0
        n32 = vsl.workspace_bytes(op, 32, 24, 16, 4)
        if min32 is None:
            assert n32 < n, op
        else:
            assert n32 >= min32 * 32 * 24 * 16, op
    assert vsl.workspace_bytes("area_volume", 64, 64, 64, 8) >= 16 * (64 // 32) * (64 // 8) * 64
    assert vsl.lib.vsl_workspace_bytes(99, 8, 8, 8, 8) == 0
    assert vsl.lib.vsl_workspace_bytes(1, 8, 8, 8, 2) == 0
    assert vsl.lib.vsl_workspace_bytes(1, 0, 8, 8, 8) == 0


def test_plane_loads_switch(vsl):
    """The process-wide plane-load mode of the tiled kernels (1 TMA, 0 registers) and the
    argument checks of its entry points (host only, no launch)."""
    call = vsl.raw
    assert call("vsl_plane_loads") == 0  # the default: registers
    assert call("vsl_set_plane_loads", 1) == 0 and call("vsl_plane_loads") == 1
    assert call("vsl_set_plane_loads", 2) == 3 and call("vsl_plane_loads") == 1  # VSL_ERR_VALUE, unchanged
    assert call("vsl_set_plane_loads", 0) == 0 and call("vsl_plane_loads") == 0
    assert call("vsl_tma_wait_timeouts", None) == 1  # VSL_ERR_NULL before any CUDA call


def test_tile_pages_table(vsl):
    """The pages-per-block table of the tiled kernels: default 20, set / replace / remove,
    argument checks (host only, no launch)."""
    call = vsl.raw
    assert call("vsl_tile_pages", 40, 36, 52, 1) == 20
    assert call("vsl_set_tile_pages", 40, 36, 52, 1, 8) == 0
    assert call("vsl_tile_pages", 40, 36, 52, 1) == 8
    assert call("vsl_tile_pages", 40, 36, 52, 0) == 20  # other kind untouched
    assert call("vsl_set_tile_pages", 40, 36, 52, 1, 4) == 0
    assert call("vsl_tile_pages", 40, 36, 52, 1) == 4
    assert call("vsl_set_tile_pages", 40, 36, 52, 1, 0) == 0  # back to the default
    assert call("vsl_tile_pages", 40, 36, 52, 1) == 20
    assert call("vsl_set_tile_pages", 0, 36, 52, 1, 8) == 2
    assert call("vsl_set_tile_pages", 40, 36, 52, 3, 8) == 0  # kind 3: the ENORK2 extension
    assert call("vsl_tile_pages", 40, 36, 52, 3) == 8
    assert call("vsl_set_tile_pages", 40, 36, 52, 3, 0) == 0
    assert call("vsl_set_tile_pages", 40, 36, 52, 4, 8) == 0  # kind 4: the ENORK2 reinitialization
    assert call("vsl_set_tile_pages", 40, 36, 52, 4, 0) == 0
    assert call("vsl_set_tile_pages", 40, 36, 52, 5, 8) == 3
    assert call("vsl_set_tile_pages", 40, 36, 52, 1, -1) == 3
    assert call("vsl_tile_pages", 40, 36, 52, 7) == 0
