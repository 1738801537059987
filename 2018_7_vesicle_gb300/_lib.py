"""ctypes binding of the C ABI declared in include/vsl_gb300.h.

The library is loaded from the package's ``lib/`` directory.  There is no fallback: if
the CUDA library is missing or fails to load, every operation raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libvsl_gb300.so")

# argument kinds: p pointer, i int, d double, z size_t, s stream
_K = {"p": ctypes.c_void_p, "i": ctypes.c_int, "d": ctypes.c_double, "z": ctypes.c_size_t, "s": ctypes.c_void_p}

_G = "iiiddd"  # rows, cols, pges, dx, dy, dz
SIGNATURES = {
    # drop-in kernels (FP64, reference argument order)
    "vsl_boundary_location": "ppppppp" + "i" + _G + "s",
    "vsl_cubic_boundary_correction": "ppppppp" + "i" + _G + "s",
    "vsl_re_step": "pppp" + "pppppp" + _G + "i" + "s",
    "vsl_re_step_eno3": "pppp" + "pppppp" + _G + "i" + "s",
    "vsl_upwind_normal": "pppp" + "pppppp" + _G + "i" + "s",
    "vsl_upwind_normal_eno3": "pppp" + "pppppp" + _G + "i" + "s",
    "vsl_boundary_interpolant": "pppppp" + "pppppp" + "p" + _G + "i" + "s",
    "vsl_boundary_interpolate_eno3": "pppppp" + "pppppp" + "p" + _G + "i" + "s",
    "vsl_extend_step": "pppppp" + "pppppp" + "pppppp" + _G + "i" + "s",
    "vsl_extend_step_eno3": "pppppp" + "pppppp" + "pppppp" + _G + "i" + "s",
    "vsl_set_calculus_toolbox": "p" * 18 + "pp" + _G + "d" + "i" + "s",
    "vsl_advection_step": "ppppp" + _G + "s",
    "vsl_weno_derivative": "ppppppp" + _G + "s",
    "vsl_auxi_set_calculus_toolbox": "p" * 27 + "pp" + "p" * 13 + _G + "d" + "i" + "s",
    # ENORK2 drop-ins (FP64, reference argument order)
    "vsl_enork2_boundary_correction": "ppppppp" + "i" + _G + "s",
    "vsl_enork2_re_step": "pppp" + "pppppp" + _G + "i" + "s",
    "vsl_enork2_upwind_normal": "pppp" + "pppppp" + _G + "i" + "s",
    "vsl_enork2_boundary_interpolate": "pppppp" + "pppppp" + "p" + _G + "i" + "s",
    "vsl_enork2_extend_step": "pppppp" + "pppppp" + "pppppp" + _G + "i" + "s",
    # tuning table of the tiled kernels (pages per block)
    "vsl_set_tile_pages": "iiiii",
    "vsl_tile_pages": "iiii",
    # plane loads of the tiled kernels (1 TMA, 0 registers) and the TMA wait-timeout count
    "vsl_set_plane_loads": "i",
    "vsl_plane_loads": "",
    "vsl_tma_wait_timeouts": "p",
    # no-allocation variant (static device scratch, no workspace argument)
    "vsl_area_volume_noalloc_f64": "pp" + _G + "s",
    # a batch of vesicle steps: host array of VesicleF32, count, ext/reinit pseudo-steps, CFL
    "vsl_vesicle_step_batch_f32": "piiid" + "s",
    # a batch of WENO5 RK3 reinitializations: host array of ReinitF32, count, pseudo-steps
    "vsl_weno5_rk3_reinitialization_batch_f32": "pii" + "s",
    # a batch of WENO5 RK3 extensions: host array of ExtendF32, count, pseudo-steps
    "vsl_weno5_rk3_extend_batch_f32": "pii" + "s",
    # a batch of WENO5 RK3 advections: host array of AdvectF32, count, steps
    "vsl_weno5_rk3_advection_batch_f32": "pii" + "s",
    # batches of closest-point surface redistances: host array of RedistanceF32, count, iter1, iter2
    "vsl_weno5_rk3_surface_redistance_batch_f32": "piii" + "s",
    "vsl_wenork3_surface_redistance_batch_f32": "piii" + "s",
}


class RedistanceF32(ctypes.Structure):
    """vsl_redistance_f32 of the C ABI: one member of vsl_*_surface_redistance_batch_f32."""

    _fields_ = [("A", ctypes.c_void_p), ("F", ctypes.c_void_p), ("rows", ctypes.c_int), ("cols", ctypes.c_int),
                ("pges", ctypes.c_int), ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]


class AdvectF32(ctypes.Structure):
    """vsl_advect_f32 of the C ABI: one member of vsl_weno5_rk3_advection_batch_f32."""

    _fields_ = [("F", ctypes.c_void_p), ("vx", ctypes.c_void_p), ("vy", ctypes.c_void_p), ("vz", ctypes.c_void_p),
                ("dt", ctypes.c_void_p), ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("pges", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]


class ExtendF32(ctypes.Structure):
    """vsl_extend_f32 of the C ABI: one member of vsl_weno5_rk3_extend_batch_f32."""

    _fields_ = [("C", ctypes.c_void_p), ("F", ctypes.c_void_p), ("xpr", ctypes.c_void_p), ("xpl", ctypes.c_void_p),
                ("ypf", ctypes.c_void_p), ("ypb", ctypes.c_void_p), ("zpu", ctypes.c_void_p), ("zpd", ctypes.c_void_p),
                ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("pges", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]


class ReinitF32(ctypes.Structure):
    """vsl_reinit_f32 of the C ABI: one member of vsl_weno5_rk3_reinitialization_batch_f32."""

    _fields_ = [("F", ctypes.c_void_p), ("xpr", ctypes.c_void_p), ("xpl", ctypes.c_void_p), ("ypf", ctypes.c_void_p),
                ("ypb", ctypes.c_void_p), ("zpu", ctypes.c_void_p), ("zpd", ctypes.c_void_p),
                ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("pges", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]


class VesicleF32(ctypes.Structure):
    """vsl_vesicle_f32 of the C ABI: one vesicle of vsl_vesicle_step_batch_f32."""

    _fields_ = [("F", ctypes.c_void_p), ("xpr", ctypes.c_void_p), ("xpl", ctypes.c_void_p), ("ypf", ctypes.c_void_p),
                ("ypb", ctypes.c_void_p), ("zpu", ctypes.c_void_p), ("zpd", ctypes.c_void_p),
                ("info", ctypes.c_void_p), ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("pges", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]
for _suf in ("f64", "f32"):
    SIGNATURES.update(
        {
            f"vsl_set_distance_{_suf}": "ppppppp" + _G + "pz" + "s",
            f"vsl_weno5_rk3_reinitialization_{_suf}": "pi" + "pppppp" + _G + "pz" + "s",
            f"vsl_weno5_rk3_reinitialization_tol_{_suf}": "pidd" + "pppppp" + _G + "pp" + "pz" + "s",
            f"vsl_wenork3_reinitialization_{_suf}": "pi" + _G + "pz" + "s",
            f"vsl_weno5_rk3_extend_{_suf}": "pip" + "pppppp" + _G + "pz" + "s",
            f"vsl_wenork3_extend_{_suf}": "pip" + _G + "pz" + "s",
            f"vsl_weno5_rk3_surface_redistance_{_suf}": "piip" + _G + "pz" + "s",
            f"vsl_wenork3_surface_redistance_{_suf}": "piip" + _G + "pz" + "s",
            f"vsl_area_volume_{_suf}": "pp" + _G + "pz" + "s",
            f"vsl_weno5_rk3_advection_{_suf}": "pppppi" + _G + "pz" + "s",
            f"vsl_vesicle_step_{_suf}": "p" + "pppppp" + "iid" + "p" + _G + "pz" + "s",
            f"vsl_enork2_reinitialization_{_suf}": "pi" + _G + "pz" + "s",
            f"vsl_enork2_extend_{_suf}": "pip" + _G + "pz" + "s",
            f"vsl_enork2_surface_redistance_{_suf}": "piip" + _G + "pz" + "s",
            f"vsl_laplacian_{_suf}": "pp" + _G + "s",
            f"vsl_gradient_{_suf}": "pppp" + _G + "s",
            f"vsl_smooth_bilaplacian_{_suf}": "pppdi" + _G + "pz" + "s",
            f"vsl_relax_step_{_suf}": "p" + "pppppp" + "dddddd" + "ii" + "p" + _G + "pz" + "s",
            f"vsl_weno5_rk3_advection_adjoint_{_suf}": "ppppp" + "pppp" + _G + "pz" + "s",
            f"vsl_weno5_rk3_reinitialization_adjoint_{_suf}": "pipp" + _G + "pz" + "s",
            f"vsl_a_set_calculus_toolbox_{_suf}": "ppp" + _G + "pz" + "s",
            f"vsl_masked_integral_{_suf}": "pppppp" + "p" + _G + "pz" + "s",
        }
    )

OP = {
    "reinit_weno5": 1,
    "reinit_eno3": 2,
    "extend_weno5": 3,
    "extend_eno3": 4,
    "surface_redistance": 5,
    "area_volume": 6,
    "advection": 7,
    "vesicle_step": 8,
    "set_distance": 9,
    "advection_adjoint": 10,
    "reinit_adjoint": 11,
    "reinit_enork2": 12,
    "extend_enork2": 13,
    "surface_redistance_enork2": 14,
    "smooth": 15,
    "relax_step": 16,
    "aux_toolbox": 17,
    "masked_integral": 18,
    "reinit_tol": 19,
    "surface_redistance_eno3": 20,
}


class VslError(RuntimeError):
    def __init__(self, fn: str, status: int, text: str):
        super().__init__(f"{fn} failed: status {status} ({text})")
        self.status = status


class Library:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            raise ImportError(
                f"CUDA library not built: {path} is missing; run the package build (build.build()) first"
            )
        self.path = path
        self.lib = ctypes.CDLL(path)
        self.lib.vsl_status_string.argtypes = [ctypes.c_int]
        self.lib.vsl_status_string.restype = ctypes.c_char_p
        self.lib.vsl_version.restype = ctypes.c_int
        self.lib.vsl_workspace_bytes.argtypes = [ctypes.c_int] * 5
        self.lib.vsl_workspace_bytes.restype = ctypes.c_size_t
        for name, sig in SIGNATURES.items():
            fn = getattr(self.lib, name)
            fn.argtypes = [_K[c] for c in sig]
            fn.restype = ctypes.c_int

    def status_string(self, st: int) -> str:
        return self.lib.vsl_status_string(st).decode()

    def workspace_bytes(self, op: str, rows: int, cols: int, pges: int, elem_bytes: int) -> int:
        return int(self.lib.vsl_workspace_bytes(OP[op], rows, cols, pges, elem_bytes))

    def call(self, name: str, *args) -> None:
        """Call an entry point; raise VslError on a nonzero status."""
        st = getattr(self.lib, name)(*args)
        if st != 0:
            raise VslError(name, st, self.status_string(st))

    def raw(self, name: str, *args) -> int:
        """Call an entry point and return its status (for tests of the error paths)."""
        return int(getattr(self.lib, name)(*args))


_LIB: Library | None = None


def lib() -> Library:
    global _LIB
    if _LIB is None:
        _LIB = Library()
    return _LIB
