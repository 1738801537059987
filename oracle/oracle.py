"""CPU oracle for the level-set hot path -- TEST INFRASTRUCTURE ONLY.

Two interchangeable kernel sets with the reference kernels' names and argument order:

* ``kernels("port")``  -- ``vsl_oracle.c``, this repository's C restatement;
* ``kernels("port_crpow")`` -- the same with integer powers rounded once;
* ``kernels("ref")``   -- the reference's own ``.cu`` files compiled for the host by
  ``oracle/ref/Makefile`` into ``oracle/_ref/`` (only where the reference checkout exists).

On top of either set, the functions below restate the MATLAB glue of the reference's
``SD.SDF3`` class (setDistance, the TVD-RK3 loops, the extension normals, the closest-point
surface redistance, area/volume/surface integrals) with numpy float64 arithmetic.

Arrays are numpy float64 of shape (rows, cols, pges) in Fortran (column-major) order, the
reference's memory layout: element (i, j, k) = row (y), column (x), page (z).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
module.  The product (the CUDA library) never imports it.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "lib", "libvsl_oracle.so")
PORT_CRPOW_LIB = os.path.join(HERE, "lib", "libvsl_oracle_crpow.so")
REF_LIB = os.path.join(HERE, "_ref", "libvsl_ref.so")

_D = ctypes.c_double
_I = ctypes.c_int
_P = ctypes.c_void_p

# name -> argument kinds ('p' pointer, 'i' int, 'd' double), reference prototype order
SIGNATURES = {
    "boundary_location": "pppppppiiiiddd",
    "cubic_boundary_correction": "pppppppiiiiddd",
    "re_step": "ppppppppppiiidddi",
    "re_step_eno3": "ppppppppppiiidddi",
    "upwind_normal": "ppppppppppiiidddi",
    "upwind_normal_eno3": "ppppppppppiiidddi",
    "boundary_interpolant": "pppppppppppppiiidddi",
    "boundary_interpolate_eno3": "pppppppppppppiiidddi",
    "extend_step": "ppppppppppppppppppiiidddi",
    "extend_step_eno3": "ppppppppppppppppppiiidddi",
    "advection_step": "pppppiiiddd",
    "weno_derivative": "pppppppiiiddd",
    "set_calculus_toolbox": "ppppppppppppppppppppiiiddddi",
    "auxi_set_calculus_toolbox": "p" * 42 + "iiiddddi",
    "enork2_boundary_correction": "pppppppiiiiddd",
    "enork2_re_step": "ppppppppppiiidddi",
    "enork2_upwind_normal": "ppppppppppiiidddi",
    "enork2_boundary_interpolate": "pppppppppppppiiidddi",
    "enork2_extend_step": "ppppppppppppppppppiiidddi",
}
_KIND = {"p": _P, "i": _I, "d": _D}


class KernelSet:
    """ctypes front end of one kernel library; methods take numpy arrays for pointers."""

    def __init__(self, path: str, prefix: str):
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library not built: {path}")
        self.path = path
        self.lib = ctypes.CDLL(path)
        self._fns = {}
        for name, sig in SIGNATURES.items():
            fn = getattr(self.lib, prefix + name)
            fn.argtypes = [_KIND[c] for c in sig]
            fn.restype = None
            self._fns[name] = (fn, sig)

    def __getattr__(self, name):
        if name.startswith("_") or name not in SIGNATURES:
            raise AttributeError(name)
        fn, sig = self._fns[name]

        def call(*args):
            if len(args) != len(sig):
                raise TypeError(f"{name}: expected {len(sig)} arguments, got {len(args)}")
            conv = []
            for a, c in zip(args, sig):
                if c == "p":
                    if not (isinstance(a, np.ndarray) and a.flags.f_contiguous):
                        raise TypeError(f"{name}: array arguments must be Fortran-ordered numpy arrays")
                    conv.append(a.ctypes.data)
                elif c == "i":
                    conv.append(int(a))
                else:
                    conv.append(float(a))
            fn(*conv)

        return call


_CACHE: dict = {}


def kernels(which: str = "port") -> KernelSet:
    """The restatement ("port"), the restatement with integer powers rounded once
    ("port_crpow", the rounding of the CUDA plain form) or the reference host build ("ref")."""
    if which not in _CACHE:
        if which == "port":
            _CACHE[which] = KernelSet(PORT_LIB, "orc_")
        elif which == "port_crpow":
            _CACHE[which] = KernelSet(PORT_CRPOW_LIB, "orc_")
        elif which == "ref":
            _CACHE[which] = KernelSet(REF_LIB, "ref_")
        else:
            raise ValueError(which)
    return _CACHE[which]


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


# ---------------------------------------------------------------------------------------
# grid metadata: V/+SD/@GD3/GD3.m:86-106
# ---------------------------------------------------------------------------------------


@dataclass
class Grid:
    rows: int
    cols: int
    pges: int
    dx: float
    dy: float
    dz: float

    @property
    def ds(self) -> float:
        return (self.dx + self.dy + self.dz) / 3

    @property
    def size(self):
        return (self.rows, self.cols, self.pges)

    @property
    def num_ele(self) -> int:
        return self.rows * self.cols * self.pges

    def args(self):
        return (self.rows, self.cols, self.pges, self.dx, self.dy, self.dz)


def meshgrid(xv, yv, zv):
    """MATLAB meshgrid(xv, yv, zv): arrays of shape (len(yv), len(xv), len(zv)), F order."""
    x, y, z = np.meshgrid(np.asarray(xv, float), np.asarray(yv, float), np.asarray(zv, float))
    return np.asfortranarray(x), np.asfortranarray(y), np.asfortranarray(z)


def grid_from_mesh(x, y, z) -> Grid:
    """Dx = X(1,2,1)-X(1,1,1), Dy = Y(2,1,1)-Y(1,1,1), Dz = Z(1,1,2)-Z(1,1,1)."""
    r, c, p = x.shape
    return Grid(r, c, p, float(x[0, 1, 0] - x[0, 0, 0]), float(y[1, 0, 0] - y[0, 0, 0]), float(z[0, 0, 1] - z[0, 0, 0]))


def zeros(g: Grid):
    return np.zeros(g.size, order="F")


def full(g: Grid, v: float):
    return np.full(g.size, v, order="F")


def F64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


# ---------------------------------------------------------------------------------------
# setDistance: V/+SD/@SDF3/setDistance.m:5-21
# ---------------------------------------------------------------------------------------


@dataclass
class Distances:
    xpr: np.ndarray
    xpl: np.ndarray
    ypf: np.ndarray
    ypb: np.ndarray
    zpu: np.ndarray
    zpd: np.ndarray

    def six(self):
        return (self.xpr, self.xpl, self.ypf, self.ypb, self.zpu, self.zpd)

    @property
    def min_dist(self):
        return np.minimum(np.minimum(self.xpr, self.xpl), np.minimum(np.minimum(self.ypf, self.ypb), np.minimum(self.zpu, self.zpd)))


def set_distance(K: KernelSet, g: Grid, F, cubic: bool = False) -> Distances:
    """Distances to the interface along the six grid directions (Delta where none)."""
    F = F64(F)
    d = Distances(full(g, g.dx), full(g, g.dx), full(g, g.dy), full(g, g.dy), full(g, g.dz), full(g, g.dz))
    fn = K.cubic_boundary_correction if cubic else K.boundary_location
    fn(*d.six(), F, g.num_ele, *g.args())
    return d


# ---------------------------------------------------------------------------------------
# TVD-RK3 reinitialization: V/+SD/@SDF3/WENO5RK3Reinitialization.m:3-43 and
# V/+SD/@SDF3/WENORK3Reinitialization.m:3-61
# ---------------------------------------------------------------------------------------


def _rk3(F, stage):
    """Shu-Osher TVD-RK3 exactly as the MATLAB loops combine the stages."""
    step = stage(F)
    t1 = F - step
    step = stage(t1)
    t2 = t1 - step
    t05 = 3.0 / 4.0 * F + 1.0 / 4.0 * t2
    step = stage(t05)
    t15 = t05 - step
    return 1.0 / 3.0 * F + 2.0 / 3.0 * t15


def reinit_weno5(K, g: Grid, F, iteration: int, dist: Distances):
    """WENO5RK3Reinitialization(F, iteration) with the object's cached distances."""
    F = F64(F).copy(order="F")
    mask = np.asfortranarray(F < 0)
    deltat = F64(0.3 * dist.min_dist)
    step = zeros(g)

    def stage(Fs):
        K.re_step(step, F64(Fs), mask, deltat, *dist.six(), *g.args(), g.num_ele)
        return step.copy(order="F")

    for _ in range(iteration):
        F = F64(_rk3(F, stage))
    return F


def reinit_residual(K, g: Grid, F, mask, dist: Distances, band: float) -> float:
    """Residual of the reinitialization at F: the maximum over the nodes with |F| < band of
    | |grad F|_G - 1 |, the Godunov norm of re_step (re_step.cu:382-392) with the call's
    mask, recovered as |step| / deltat (deltat = 0.3 min_dist); fixed nodes (step 0) count 0.
    No counterpart in the reference, whose loop runs a fixed count."""
    F = F64(F)
    deltat = F64(0.3 * dist.min_dist)
    step = zeros(g)
    K.re_step(step, F, mask, deltat, *dist.six(), *g.args(), g.num_ele)
    sel = (np.abs(F) < band) & (deltat > 0)
    if not np.any(sel):
        return 0.0
    r = np.abs(step[sel]) / deltat[sel]
    return float(np.inf) if np.any(np.isnan(r)) else float(np.max(r))


def reinit_weno5_tol(K, g: Grid, F, max_iters: int, tol: float, band: float, dist: Distances):
    """WENO5RK3Reinitialization run while the residual exceeds tol, at most max_iters
    pseudo-steps (mask = F < 0 on entry, the cached distances).  Returns (F, steps taken,
    converged, residual history [0..steps])."""
    F = F64(F).copy(order="F")
    mask = np.asfortranarray(F < 0)
    deltat = F64(0.3 * dist.min_dist)
    step = zeros(g)

    def stage(Fs):
        K.re_step(step, F64(Fs), mask, deltat, *dist.six(), *g.args(), g.num_ele)
        return step.copy(order="F")

    hist = [reinit_residual(K, g, F, mask, dist, band)]
    n = 0
    while hist[-1] > tol and n < max_iters:
        F = F64(_rk3(F, stage))
        n += 1
        hist.append(reinit_residual(K, g, F, mask, dist, band))
    return F, n, hist[-1] <= tol, hist


def reinit_eno3(K, g: Grid, F, iteration: int):
    """WENORK3Reinitialization(F, iteration): cubic distances recomputed from F."""
    F = F64(F).copy(order="F")
    mask = np.asfortranarray(F < 0)
    dist = set_distance(K, g, F, cubic=True)
    deltat = F64(0.3 * dist.min_dist)
    step = zeros(g)

    def stage(Fs):
        K.re_step_eno3(step, F64(Fs), mask, deltat, *dist.six(), *g.args(), g.num_ele)
        return step.copy(order="F")

    for _ in range(iteration):
        F = F64(_rk3(F, stage))
    return F


# ---------------------------------------------------------------------------------------
# ENORK2 reinitialization: V/+SD/@SDF3/ENORK2Reinitialization.m:3-45
# ---------------------------------------------------------------------------------------


def _rk2(F, stage):
    """Heun RK2 as the ENORK2 MATLAB loops combine the stages: (F + Ftmp - step) / 2."""
    step = stage(F)
    Ftmp = F - step
    step = stage(Ftmp)
    return (F + Ftmp - step) / 2


def set_distance_enork2(K: KernelSet, g: Grid, F) -> Distances:
    """Quadratic-ENO distances (ENORK2_boundary_correction on spacing-filled arrays)."""
    F = F64(F)
    d = Distances(full(g, g.dx), full(g, g.dx), full(g, g.dy), full(g, g.dy), full(g, g.dz), full(g, g.dz))
    K.enork2_boundary_correction(*d.six(), F, g.num_ele, *g.args())
    return d


def reinit_enork2(K, g: Grid, F, iteration: int):
    """ENORK2Reinitialization(F, iteration): distances recomputed from F, Heun RK2."""
    F = F64(F).copy(order="F")
    mask = np.asfortranarray(F < 0)
    dist = set_distance_enork2(K, g, F)
    deltat = F64(0.3 * dist.min_dist)
    step = zeros(g)

    def stage(Fs):
        K.enork2_re_step(step, F64(Fs), mask, deltat, *dist.six(), *g.args(), g.num_ele)
        return step.copy(order="F")

    for _ in range(iteration):
        F = F64(_rk2(F, stage))
    return F


# ---------------------------------------------------------------------------------------
# extension: V/+SD/@SDF3/WENO5RK3Extend.m:9-76 and V/+SD/@SDF3/WENORK3Extend.m:9-98
# ---------------------------------------------------------------------------------------


def extension_velocity(K, g: Grid, F, dist: Distances, eno3: bool = False, floor: float = 1e-6, enork2: bool = False):
    """v = sign(F) * n, n = upwind gradient / max(|gradient|, floor)."""
    fx, fy, fz = zeros(g), zeros(g), zeros(g)
    fn = K.enork2_upwind_normal if enork2 else (K.upwind_normal_eno3 if eno3 else K.upwind_normal)
    fn(fx, fy, fz, F64(F), *dist.six(), *g.args(), g.num_ele)
    grad = np.maximum(np.sqrt(fx ** 2 + fy ** 2 + fz ** 2), floor)
    s = np.sign(F)
    return F64(s * (fx / grad)), F64(s * (fy / grad)), F64(s * (fz / grad))


def crossing_values(K, g: Grid, C, dist: Distances, eno3: bool = False):
    cp = [zeros(g) for _ in range(6)]
    fn = K.boundary_interpolate_eno3 if eno3 else K.boundary_interpolant
    fn(*cp, *dist.six(), F64(C), *g.args(), g.num_ele)
    return cp


def extend_loop(K, g: Grid, C, iteration, dist: Distances, v, deltat, cp, eno3: bool = False):
    step = zeros(g)
    fn = K.extend_step_eno3 if eno3 else K.extend_step

    def stage(Cs):
        fn(step, deltat, F64(Cs), *v, *dist.six(), *cp, *g.args(), g.num_ele)
        return step.copy(order="F")

    C = F64(C).copy(order="F")
    for _ in range(iteration):
        C = F64(_rk3(C, stage))
    return C


def extend_enork2(K, g: Grid, F, C, iteration: int):
    """ENORK2Extend(C, iteration) (V/+SD/@SDF3/ENORK2Extend.m:9-81): quadratic-ENO
    distances of F, ENO upwind normals, quadratic crossing values of C, Heun RK2."""
    dist = set_distance_enork2(K, g, F)
    v = extension_velocity(K, g, F, dist, enork2=True)
    cp = [zeros(g) for _ in range(6)]
    K.enork2_boundary_interpolate(*cp, *dist.six(), F64(C), *g.args(), g.num_ele)
    deltat = F64(0.3 * dist.min_dist)
    step = zeros(g)

    def stage(Cs):
        K.enork2_extend_step(step, deltat, F64(Cs), *v, *dist.six(), *cp, *g.args(), g.num_ele)
        return step.copy(order="F")

    C = F64(C).copy(order="F")
    for _ in range(iteration):
        C = F64(_rk2(C, stage))
    return C


def extend_weno5(K, g: Grid, F, dist: Distances, C, iteration: int):
    """WENO5RK3Extend(C, iteration) with the object's cached distances of F."""
    v = extension_velocity(K, g, F, dist)
    cp = crossing_values(K, g, C, dist)
    deltat = F64(0.3 * dist.min_dist)
    return extend_loop(K, g, C, iteration, dist, v, deltat, cp)


def extend_eno3(K, g: Grid, F, C, iteration: int):
    """WENORK3Extend(C, iteration): cubic distances of F recomputed inside."""
    dist = set_distance(K, g, F, cubic=True)
    v = extension_velocity(K, g, F, dist, eno3=True)
    cp = crossing_values(K, g, C, dist, eno3=True)
    deltat = F64(0.3 * dist.min_dist)
    return extend_loop(K, g, C, iteration, dist, v, deltat, cp, eno3=True)


# ---------------------------------------------------------------------------------------
# closest-point surface redistance: V/+SD/@SDF3/WENO5RK3ClosetPointSurfaceRedistance.m:4-157
# ---------------------------------------------------------------------------------------


def surface_redistance(K, g: Grid, F, A, iter1: int, iter2: int, eno3: bool = False):
    """WENO5RK3ClosetPointSurfaceRedistance(A, iter1, iter2); eno3=True gives
    WENORK3ClosetPointSurfaceRedistance (V/+SD/@SDF3/WENORK3ClosetPointSurfaceRedistance.m:4-152),
    the same composition with cubic_boundary_correction for both distance sets (:16, :39),
    WENORK3_upwind_normal (:55), WENORK3_reinitialization_step (:85-101),
    WENORK3_boundary_interpolate (:118) and WENORK3_extend_step (:126-141)."""
    A = F64(A).copy(order="F")
    dA = set_distance(K, g, A, cubic=eno3)
    deltat = F64(0.3 * dA.min_dist)
    mask = np.asfortranarray(A < 0)
    dF = set_distance(K, g, F, cubic=eno3)
    fdeltat = F64(0.3 * dF.min_dist)
    v = extension_velocity(K, g, F, dF, eno3=eno3, floor=1e-14)
    step = zeros(g)
    re_step = K.re_step_eno3 if eno3 else K.re_step

    def ext(C):
        cp = crossing_values(K, g, C, dF, eno3=eno3)
        return extend_loop(K, g, C, iter2, dF, v, fdeltat, cp, eno3=eno3)

    def re(Cs):
        re_step(step, F64(Cs), mask, deltat, *dA.six(), *g.args(), g.num_ele)
        return step.copy(order="F")

    new = A
    for _ in range(iter1):
        new = ext(new)
        t1 = new - re(new)
        t1 = ext(t1)
        t2 = t1 - re(t1)
        t05 = 3.0 / 4.0 * new + 1.0 / 4.0 * t2
        t05 = ext(t05)
        t15 = t05 - re(t05)
        new = F64(1.0 / 3.0 * new + 2.0 / 3.0 * t15)
    return ext(new)


def surface_redistance_enork2(K, g: Grid, F, A, iter1: int, iter2: int):
    """ENORK2ClosetPointSurfaceRedistance(A, iter1, iter2)
    (V/+SD/@SDF3/ENORK2ClosetPointSurfaceRedistance.m:4-128): A's quadratic-ENO distances,
    mask and dt for the reinitialization; F's distances, ENO upwind normals (floor 1e-14)
    and dt for the extensions, whose crossing values are taken from each input."""
    A = F64(A).copy(order="F")
    dA = set_distance_enork2(K, g, A)
    deltat = F64(0.3 * dA.min_dist)
    mask = np.asfortranarray(A < 0)
    dF = set_distance_enork2(K, g, F)
    fdeltat = F64(0.3 * dF.min_dist)
    v = extension_velocity(K, g, F, dF, floor=1e-14, enork2=True)
    step = zeros(g)

    def ext(C):
        cp = [zeros(g) for _ in range(6)]
        K.enork2_boundary_interpolate(*cp, *dF.six(), F64(C), *g.args(), g.num_ele)
        st = zeros(g)

        def stage(Cs):
            K.enork2_extend_step(st, fdeltat, F64(Cs), *v, *dF.six(), *cp, *g.args(), g.num_ele)
            return st.copy(order="F")

        C = F64(C).copy(order="F")
        for _ in range(iter2):
            C = F64(_rk2(C, stage))
        return C

    def re(Cs):
        K.enork2_re_step(step, F64(Cs), mask, deltat, *dA.six(), *g.args(), g.num_ele)
        return step.copy(order="F")

    new = A
    for _ in range(iter1):
        new = ext(new)
        t = new - re(new)
        t = ext(t)
        t2 = t - re(t)
        new = F64((new + t2) / 2)
    return ext(new)


# ---------------------------------------------------------------------------------------
# calculus toolbox and reductions: V/+SD/@SDF3/GPUsetCalculusToolBox.m:2-42, SDF3.m:73-85
# ---------------------------------------------------------------------------------------

TOOLBOX_FIELDS = ("Fx", "Fy", "Fz", "FGradMag", "Nx", "Ny", "Nz", "Fxx", "Fyy", "Fzz", "Fxy", "Fyz", "Fzx",
                  "FLaplacian", "MeanCurvature", "GaussianCurvature", "Heaviside", "DiracDelta")


def calculus_toolbox(K, g: Grid, F):
    F = F64(F)
    hp = F64(np.maximum(F, 0))
    out = {n: zeros(g) for n in TOOLBOX_FIELDS}
    K.set_calculus_toolbox(*[out[n] for n in TOOLBOX_FIELDS], F, hp, *g.args(), g.ds, g.num_ele)
    return out


AUX_FIELDS = ("Ax", "Ay", "Az", "AGradMag", "Cx", "Cy", "Cz", "NormCrossAF", "tx", "ty", "tz", "nx", "ny", "nz",
              "Axx", "Ayy", "Azz", "Axy", "Ayz", "Azx", "ALaplacian", "GeodesicCurvature", "NormalCurvature",
              "GeodesicTorsion", "BPerpendicular", "AHeaviside", "ADiracDelta")
AUX_INPUTS = ("Fx", "Fy", "Fz", "FGradMag", "Nx", "Ny", "Nz", "Fxx", "Fyy", "Fzz", "Fxy", "Fyz", "Fzx")


def periodic_gradient(g: Grid, f):
    """GD3.Gradient (GD3.m:314-318): central differences with circshift neighbours,
    (f(x + h) - f(x - h)) / (2 h) per axis; arrays are (rows = y, cols = x, pges = z)."""
    f = F64(f)
    fx = (np.roll(f, -1, axis=1) - np.roll(f, 1, axis=1)) / (2 * g.dx)
    fy = (np.roll(f, -1, axis=0) - np.roll(f, 1, axis=0)) / (2 * g.dy)
    fz = (np.roll(f, -1, axis=2) - np.roll(f, 1, axis=2)) / (2 * g.dz)
    return F64(fx), F64(fy), F64(fz)


def auxiliary_toolbox(K, g: Grid, F, A, tb=None):
    """GPUAsetCalculusToolBox.m:2-63: the toolbox of the auxiliary level set A with F's
    toolbox fields (`tb`, computed when not given): the 27 kernel fields, then
    AFDiracDelta = (C . (grad H_F x grad H_A)) / |C|^2 and
    ADiracDeltaDn = (Laplacian(H_A) - ADiracDelta Laplacian(A)) / |grad A| with the
    periodic GD3 operators."""
    F, A = F64(F), F64(A)
    tb = calculus_toolbox(K, g, F) if tb is None else tb
    out = {n: zeros(g) for n in AUX_FIELDS}
    K.auxi_set_calculus_toolbox(*[out[n] for n in AUX_FIELDS], A, F64(np.maximum(A, 0)),
                                *[F64(tb[n]) for n in AUX_INPUTS], *g.args(), g.ds, g.num_ele)
    h1x, h1y, h1z = periodic_gradient(g, out["AHeaviside"])
    h2x, h2y, h2z = periodic_gradient(g, tb["Heaviside"])
    chx, chy, chz = h2y * h1z - h2z * h1y, h2z * h1x - h2x * h1z, h2x * h1y - h2y * h1x
    dot = out["Cx"] * chx + out["Cy"] * chy + out["Cz"] * chz
    out["AFDiracDelta"] = F64(dot / (out["NormCrossAF"] * out["NormCrossAF"]))
    out["ADiracDeltaDn"] = F64((laplacian(g, out["AHeaviside"]) - out["ADiracDelta"] * laplacian(g, A))
                               / out["AGradMag"])
    return out, tb


def line_mask(g: Grid, F, A):
    return (np.abs(F64(F)) < 2 * g.ds) & (np.abs(F64(A)) < 2 * g.ds)


def cal_length(g: Grid, F, A, aux) -> float:
    """SDF3.calLength (SDF3.m:212-215): sum(AFDiracDelta .* NormCrossAF) over |F|, |A| < 2 Ds."""
    m = line_mask(g, F, A)
    return exact_sum(aux["AFDiracDelta"][m] * aux["NormCrossAF"][m]) * g.ds ** 3


def line_integral(g: Grid, F, A, field, aux) -> float:
    """SDF3.LineIntegral (SDF3.m:216-219): sum((f .* AFDiracDelta) .* NormCrossAF)."""
    m = line_mask(g, F, A)
    return exact_sum((F64(field)[m] * aux["AFDiracDelta"][m]) * aux["NormCrossAF"][m]) * g.ds ** 3


def a_cal_area(g: Grid, F, tb, aux) -> float:
    """SDF3.AcalArea (SDF3.m:220-223): sum(DiracDelta .* (1 - AHeaviside)) over |F| < 2 Ds."""
    m = np.abs(F64(F)) < 2 * g.ds
    return exact_sum(F64(tb["DiracDelta"])[m] * (1 - aux["AHeaviside"][m])) * g.ds ** 3


def a_surface_integral(g: Grid, F, field, tb, aux) -> float:
    """SDF3.AsurfaceIntegral (SDF3.m:224-227):
    sum(((f .* DiracDelta) .* FGradMag) .* (1 - AHeaviside)) over |F| < 2 Ds."""
    m = np.abs(F64(F)) < 2 * g.ds
    return exact_sum(((F64(field)[m] * F64(tb["DiracDelta"])[m]) * F64(tb["FGradMag"])[m])
                     * (1 - aux["AHeaviside"][m])) * g.ds ** 3


def exact_sum(a) -> float:
    """Correctly rounded sum (the oracle's reduction; any summation order approximates it)."""
    return math.fsum(np.asarray(a, dtype=np.float64).ravel(order="F").tolist())


def cal_area(g: Grid, F, delta) -> float:
    mask = np.abs(F) < 2 * g.ds
    return exact_sum(delta[mask]) * g.ds ** 3


def cal_volume(g: Grid, F, heaviside) -> float:
    mask = F < 2 * g.ds
    return exact_sum(1 - heaviside[mask]) * g.ds ** 3


def surface_integral(g: Grid, F, field, delta, gradmag) -> float:
    mask = np.abs(F) < 2 * g.ds
    return exact_sum(field[mask] * delta[mask] * gradmag[mask]) * g.ds ** 3


# ---------------------------------------------------------------------------------------
# WENO5 advection (GD3.WENODotGrad, V/+SD/@GD3/GD3.m:393-398) in a TVD-RK3 wrapper
# ---------------------------------------------------------------------------------------


def weno_dot_grad(K, g: Grid, vx, vy, vz, field):
    out = zeros(g)
    K.advection_step(out, F64(vx), F64(vy), F64(vz), F64(field), *g.args())
    return out


def advect_rk3(K, g: Grid, F, vx, vy, vz, dt: float, steps: int = 1):
    """phi_t + v.grad(phi) = 0, each stage F_s - dt*(v.grad F_s), Shu-Osher combination."""
    def stage(Fs):
        return dt * weno_dot_grad(K, g, vx, vy, vz, Fs)

    F = F64(F).copy(order="F")
    for _ in range(steps):
        F = F64(_rk3(F, stage))
    return F


# ---------------------------------------------------------------------------------------
# composite vesicle step (order of V/p00_test_singlephase_relax.m:60-196)
# ---------------------------------------------------------------------------------------


def vesicle_step(K, g: Grid, F, dist: Distances, ext_iters=30, reinit_iters=20, cfl=0.5):
    """One step: toolbox -> area/volume -> extend mean curvature -> dt -> WENO5 RK3 advection
    along v = Vn*N -> setDistance -> WENO5 reinitialization.  Returns (F, dist, info)."""
    tb = calculus_toolbox(K, g, F)
    area = cal_area(g, F, tb["DiracDelta"])
    volume = cal_volume(g, F, tb["Heaviside"])
    vn = extend_weno5(K, g, F, dist, tb["MeanCurvature"], ext_iters)
    band = np.abs(F) < 2 * g.ds
    vmax = float(np.max(np.abs(vn[band])))
    dt = cfl * g.ds / vmax
    F = advect_rk3(K, g, F, vn * tb["Nx"], vn * tb["Ny"], vn * tb["Nz"], dt)
    dist = set_distance(K, g, F)
    F = reinit_weno5(K, g, F, reinit_iters, dist)
    return F, dist, {"area": area, "volume": volume, "dt": dt, "vmax": vmax}


# ---------------------------------------------------------------------------------------
# SD.GD3 operators with periodic neighbours (V/+SD/@GD3/GD3.m:110-207, 344-346, 434-485)
# and one pass of the relaxation driver's time loop (V/p00_test_singlephase_relax.m:60-196)
# ---------------------------------------------------------------------------------------


def laplacian(g: Grid, f):
    """GD3.Laplacian: (Fxx + Fyy) + Fzz, Fxx = (F(oXo) - 2F + F(oxo)) / Dx^2 with circshift
    neighbours; arrays are (rows = y, cols = x, pges = z)."""
    f = F64(f)
    fxx = (np.roll(f, -1, axis=1) - 2 * f + np.roll(f, 1, axis=1)) / (g.dx * g.dx)
    fyy = (np.roll(f, -1, axis=0) - 2 * f + np.roll(f, 1, axis=0)) / (g.dy * g.dy)
    fzz = (np.roll(f, -1, axis=2) - 2 * f + np.roll(f, 1, axis=2)) / (g.dz * g.dz)
    return F64(fxx + fyy + fzz)


def gradient(g: Grid, f):
    """GD3.Gradient (GD3.m:314-318): Fx = (F(oXo) - F(oxo)) / (2 Dx) (GD3.m:218-220), Fy and
    Fz alike, circshift neighbours; arrays are (rows = y, cols = x, pges = z)."""
    f = F64(f)
    fx = (np.roll(f, -1, axis=1) - np.roll(f, 1, axis=1)) / (2 * g.dx)
    fy = (np.roll(f, -1, axis=0) - np.roll(f, 1, axis=0)) / (2 * g.dy)
    fz = (np.roll(f, -1, axis=2) - np.roll(f, 1, axis=2)) / (2 * g.dz)
    return F64(fx), F64(fy), F64(fz)


def wave_numbers(g: Grid):
    """GD3.m:195-207: kx, ky, kz from fftshift(2 pi (-n/2 : n/2-1) / (n h)) on meshgrid."""
    def axis(n, h):
        v = 2 * np.pi * (-n / 2 + np.arange(n)) / (n * h)
        return np.roll(v, n // 2)  # MATLAB fftshift = circshift by floor(n/2)
    kx, ky, kz = np.meshgrid(axis(g.cols, g.dx), axis(g.rows, g.dy), axis(g.pges, g.dz))
    return kx, ky, kz


def smooth_fft(g: Grid, rhs, dt: float, alpha: float):
    """GD3.smoothFFT: real(ifftn(fftn(rhs) ./ (1 + alpha dt (kx^2 + ky^2 + kz^2)^2)))."""
    kx, ky, kz = wave_numbers(g)
    s = np.fft.fftn(F64(rhs)) / (1 + alpha * dt * (kx ** 2 + ky ** 2 + kz ** 2) ** 2)
    return F64(np.real(np.fft.ifftn(s)))


def smooth_gmres(g: Grid, rhs, dt: float, alpha: float, tol: float = 1e-12, maxit: int = 300):
    """GD3.smoothGMRES: (I + alpha dt L^2) x = rhs by GMRES (no restart, at most 300
    iterations, relative tolerance 1e-12) preconditioned by smoothFFT's inverse symbol."""
    from scipy.sparse.linalg import LinearOperator, gmres

    n = g.num_ele
    shape = g.size

    def op(x):
        u = x.reshape(shape, order="F")
        return (u + alpha * dt * laplacian(g, laplacian(g, u))).ravel(order="F")

    kx, ky, kz = wave_numbers(g)
    denom = 1 + alpha * dt * (kx ** 2 + ky ** 2 + kz ** 2) ** 2

    def pre(x):
        u = x.reshape(shape, order="F")
        return np.real(np.fft.ifftn(np.fft.fftn(u) / denom)).ravel(order="F")

    A = LinearOperator((n, n), matvec=op, dtype=np.float64)
    M = LinearOperator((n, n), matvec=pre, dtype=np.float64)
    x, info = gmres(A, F64(rhs).ravel(order="F"), rtol=tol, atol=0.0, restart=maxit, maxiter=maxit, M=M)
    return F64(x.reshape(shape, order="F"))


def surface_integral_mask(g: Grid, F, field, delta, gradmag) -> float:
    """SDF3.surfaceIntegral (SDF3.m:82-85): sum((f .* DiracDelta) .* FGradMag) over
    |F| < 2 Ds, times Ds^3 (exactly rounded sum)."""
    mask = np.abs(F64(F)) < 2 * g.ds
    return exact_sum((F64(field)[mask] * F64(delta)[mask]) * F64(gradmag)[mask]) * g.ds ** 3


def relax_step(K, g: Grid, F, A0: float, V0: float, kappa: float = 1.0, spon_c: float = 0.0, cfl: float = 0.5,
               alpha: float = 0.5, ext_iters: int = 100, reinit_iters: int = 0):
    """One pass of the driver's time loop without plotting: returns (F, dist, info) with
    info the 11 values of the C ABI's relax step."""
    F = F64(F).copy(order="F")
    tb = calculus_toolbox(K, g, F)
    area = cal_area(g, F, tb["DiracDelta"])
    volume = cal_volume(g, F, tb["Heaviside"])
    H = extend_eno3(K, g, F, tb["MeanCurvature"], ext_iters)
    Kg = tb["GaussianCurvature"]
    nsb = kappa * (laplacian(g, H) + 0.5 * H * (H * H - 4 * Kg) + 2. * spon_c * Kg - 0.5 * (spon_c * spon_c) * H)
    nsb = extend_enork2(K, g, F, F64(nsb), ext_iters)
    band = np.abs(F) < 2 * g.ds
    vmax = float(np.max(np.abs(nsb[band])))
    dt = cfl * g.ds / vmax
    d, G = tb["DiracDelta"], tb["FGradMag"]
    c11 = surface_integral_mask(g, F, H * H, d, G)
    c12 = surface_integral_mask(g, F, H, d, G)
    i_hn = surface_integral_mask(g, F, H * nsb, d, G)
    i_n = surface_integral_mask(g, F, nsb, d, G)
    s1 = i_hn - (A0 - area) / dt
    s2 = i_n + (V0 - volume) / dt
    tension, pressure = np.linalg.solve(np.array([[c11, c12], [c12, A0]]), np.array([s1, s2]))
    vn = F64((tension * H - nsb + pressure) * G)
    vs = smooth_gmres(g, vn, dt, alpha)
    vs = extend_enork2(K, g, F, vs, ext_iters)
    F = F64(F - dt * vs)
    dist = set_distance(K, g, F)
    ene = surface_integral_mask(g, F, (H - spon_c) ** 2, d, G)
    if reinit_iters > 0:
        F = reinit_weno5(K, g, F, reinit_iters, dist)
    info = np.array([area, volume, dt, vmax, c11, c12, i_hn, i_n, tension, pressure, ene])
    return F, dist, info

