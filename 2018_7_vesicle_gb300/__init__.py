"""GB300-native level-set hot path of the vesicle code (tiankuizhang/2018_7_Vesicle).

WENO5/ENO3 TVD-RK3 reinitialization with the sub-cell interface fix, PDE velocity
extension, closest-point surface redistance, WENO5 advection and the Heaviside/Dirac
area and volume reductions, as hand-written CUDA kernels for sm_103a behind the C ABI of
include/vsl_gb300.h.  ``sdf3`` mirrors the reference's SD.GD3 / SD.SDF3 classes on top
of that ABI; ``_lib`` is the ctypes binding.  There is no CPU fallback.
"""
from . import _lib
from ._lib import VslError, lib

__all__ = ["lib", "VslError", "GD3", "SDF3", "build"]


def build(force: bool = False) -> str:
    """Compile the CUDA library (csrc/*.cu, sm_103a) into lib/libvsl_gb300.so."""
    import importlib

    return importlib.import_module(__name__ + "._build").build(force=force)


def __getattr__(name):
    if name in ("GD3", "SDF3"):
        import importlib

        return getattr(importlib.import_module(__name__ + ".sdf3"), name)
    raise AttributeError(name)
