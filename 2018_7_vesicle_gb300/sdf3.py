"""Host-side mirror of the reference's level-set classes SD.GD3 and SD.SDF3.

Same method names, argument meaning and order as the MATLAB classes
(src/7_0_paper/2_0_Vesicle/+SD/@GD3/GD3.m, +SD/@SDF3/*.m); the arithmetic runs in the
CUDA library through the C ABI (``_lib``).  Fields are torch tensors on the current CUDA
device with the MATLAB layout: shape (rows, cols, pges) = (y, x, z), column-major
storage (strides 1, rows, rows*cols).

``precision="f64"`` is the plain form (FP64 everywhere); ``precision="f32"`` is the
mixed-precision form (FP32 fields and stencils, FP64 interface roots and reductions).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from ._lib import lib

_DTYPES = {"f64": torch.float64, "f32": torch.float32}


# ---------------------------------------------------------------------------------------
# column-major field helpers
# ---------------------------------------------------------------------------------------


def is_colmajor(t: torch.Tensor) -> bool:
    return t.dim() == 3 and t.permute(2, 1, 0).is_contiguous()


def colmajor_empty(size, dtype, device=None) -> torch.Tensor:
    r, c, p = size
    return torch.empty((p, c, r), dtype=dtype, device=device or "cuda").permute(2, 1, 0)


def colmajor_full(size, value, dtype, device=None) -> torch.Tensor:
    t = colmajor_empty(size, dtype, device)
    t.fill_(value)
    return t


def as_field(a, dtype, device=None) -> torch.Tensor:
    """A (rows, cols, pges) column-major CUDA tensor of `dtype` holding `a` (numpy array in
    any order, or tensor)."""
    device = device or "cuda"
    if isinstance(a, np.ndarray):
        r, c, p = a.shape
        flat = np.asarray(a, dtype=np.float64).ravel(order="F")
        t = torch.from_numpy(flat.copy()).view(p, c, r).permute(2, 1, 0)
    else:
        t = a
    t = t.to(device=device, dtype=dtype)
    if not is_colmajor(t):
        t = t.permute(2, 1, 0).contiguous().permute(2, 1, 0)
    return t


def to_numpy(t: torch.Tensor) -> np.ndarray:
    """Fortran-ordered float64 numpy copy of a column-major field."""
    return np.asfortranarray(t.detach().to("cpu", torch.float64).numpy())


def _ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


# ---------------------------------------------------------------------------------------
# SD.GD3: grid metadata (GD3.m:86-106)
# ---------------------------------------------------------------------------------------


class GD3:
    """Meshgrid metadata: X, Y, Z of shape (rows, cols, pges) as MATLAB meshgrid(xv,yv,zv)."""

    def __init__(self, Xm, Ym, Zm, spacing=None, device=None):
        self.X = as_field(Xm, torch.float64, device)
        self.Y = as_field(Ym, torch.float64, device)
        self.Z = as_field(Zm, torch.float64, device)
        self.Size = tuple(self.X.shape)
        self.mrows, self.ncols, self.lshts = self.Size
        self.NumElt = self.mrows * self.ncols * self.lshts
        if spacing is None:
            X, Y, Z = (to_numpy(v) for v in (self.X, self.Y, self.Z))
            spacing = (float(X[0, 1, 0] - X[0, 0, 0]), float(Y[1, 0, 0] - Y[0, 0, 0]), float(Z[0, 0, 1] - Z[0, 0, 0]))
        self.Dx, self.Dy, self.Dz = (float(s) for s in spacing)
        self.Ds = (self.Dx + self.Dy + self.Dz) / 3

    @staticmethod
    def meshgrid(xv, yv, zv, device=None):
        """MATLAB [x,y,z] = meshgrid(xv,yv,zv) as column-major CUDA tensors."""
        x, y, z = np.meshgrid(np.asarray(xv, float), np.asarray(yv, float), np.asarray(zv, float))
        return as_field(x, torch.float64, device), as_field(y, torch.float64, device), as_field(z, torch.float64, device)

    def args(self):
        return (self.mrows, self.ncols, self.lshts, self.Dx, self.Dy, self.Dz)

    def WENODotGrad(self, vx, vy, vz, field):
        """Upwind WENO5 v.grad(field) (GD3.m:393-398), FP64."""
        f = as_field(field, torch.float64)
        v = [as_field(a, torch.float64) for a in (vx, vy, vz)]
        out = colmajor_empty(self.Size, torch.float64)
        lib().call("vsl_advection_step", _ptr(out), *map(_ptr, v), _ptr(f), *self.args(), _stream())
        return out

    def Laplacian(self, field, precision: str = "f64"):
        """GD3.Laplacian (GD3.m:344-346): 7-point Laplacian with periodic neighbours."""
        dtype = _DTYPES[precision]
        f = as_field(field, dtype)
        out = colmajor_empty(self.Size, dtype)
        lib().call(f"vsl_laplacian_{precision}", _ptr(f), _ptr(out), *self.args(), _stream())
        return out

    def Gradient(self, field, precision: str = "f64"):
        """GD3.Gradient (GD3.m:314-318): central differences with periodic neighbours;
        returns (fx, fy, fz)."""
        dtype = _DTYPES[precision]
        f = as_field(field, dtype)
        out = [colmajor_empty(self.Size, dtype) for _ in range(3)]
        lib().call(f"vsl_gradient_{precision}", _ptr(f), *[_ptr(o) for o in out], *self.args(), _stream())
        return tuple(out)

    def _smooth(self, rhs, Dt, Alpha, exact: int, precision: str):
        dtype = _DTYPES[precision]
        f = as_field(rhs, dtype)
        out = colmajor_empty(self.Size, dtype)
        dt = Dt if isinstance(Dt, torch.Tensor) else torch.tensor([float(Dt)], dtype=torch.float64, device="cuda")
        n = lib().workspace_bytes("smooth", *self.Size, 8 if precision == "f64" else 4)
        ws = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
        lib().call(f"vsl_smooth_bilaplacian_{precision}", _ptr(f), _ptr(out), _ptr(dt), float(Alpha), int(exact),
                   *self.args(), _ptr(ws), ws.numel(), _stream())
        return out

    def smoothGMRES(self, rhs, Dt, Alpha, precision: str = "f64"):
        """GD3.smoothGMRES (GD3.m:436-452): the solution of (I + Alpha Dt L^2) x = rhs, L the
        periodic 7-point Laplacian, by the exact spectral solve the GMRES iteration approaches."""
        return self._smooth(rhs, Dt, Alpha, 1, precision)

    def smoothFFT(self, rhs, Dt, Alpha, precision: str = "f64"):
        """GD3.smoothFFT (GD3.m:455-460): rhs filtered by 1 / (1 + Alpha Dt |k|^4)."""
        return self._smooth(rhs, Dt, Alpha, 0, precision)

    def GPUWENODerivative(self, field):
        """Six one-sided WENO5 derivatives [back_x, fore_x, back_y, fore_y, back_z, fore_z]."""
        f = as_field(field, torch.float64)
        outs = [colmajor_empty(self.Size, torch.float64) for _ in range(6)]
        lib().call("vsl_weno_derivative", *map(_ptr, outs), _ptr(f), *self.args(), _stream())
        return outs


# ---------------------------------------------------------------------------------------
# SD.SDF3: the level-set object
# ---------------------------------------------------------------------------------------

TOOLBOX_FIELDS = ("Fx", "Fy", "Fz", "FGradMag", "Nx", "Ny", "Nz", "Fxx", "Fyy", "Fzz", "Fxy", "Fyz", "Fzx",
                  "FLaplacian", "MeanCurvature", "GaussianCurvature", "Heaviside", "DiracDelta")
# GPUAsetCalculusToolBox.m's fields: the 27 of auxi_set_calculus_toolbox in its argument
# order, then AFDiracDelta and ADiracDeltaDn
AUX_FIELDS = ("Ax", "Ay", "Az", "AGradMag", "Cx", "Cy", "Cz", "NormCrossAF", "tx", "ty", "tz", "nx", "ny", "nz",
              "Axx", "Ayy", "Azz", "Axy", "Ayz", "Azx", "ALaplacian", "GeodesicCurvature", "NormalCurvature",
              "GeodesicTorsion", "BPerpendicular", "AHeaviside", "ADiracDelta", "AFDiracDelta", "ADiracDeltaDn")


class SDF3:
    """Signed distance function on a GD3 grid (SDF3.m)."""

    def __init__(self, grid: GD3, Xm=None, Ym=None, Zm=None, Val=None, precision: str = "f64"):
        if precision not in _DTYPES:
            raise ValueError(f"precision must be one of {sorted(_DTYPES)}")
        self.GD3 = grid
        self.precision = precision
        self.dtype = _DTYPES[precision]
        self.elem = 8 if precision == "f64" else 4
        self.F = None if Val is None else as_field(Val, self.dtype)
        self.A = None  # the auxiliary level set of a multiphase vesicle (SDF3.m's A)
        self.xpr = self.xpl = self.ypf = self.ypb = self.zpu = self.zpd = None
        self._ws = {}

    # -- plumbing ----------------------------------------------------------------------
    def _fn(self, base: str) -> str:
        return f"{base}_{self.precision}"

    def _field(self, a) -> torch.Tensor:
        return as_field(a, self.dtype)

    def workspace(self, op: str) -> torch.Tensor:
        n = lib().workspace_bytes(op, *self.GD3.Size, self.elem)
        ws = self._ws.get(op)
        if ws is None or ws.numel() < n:
            ws = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
            self._ws[op] = ws
        return ws

    def _dist(self):
        if self.xpr is None:
            raise RuntimeError("setDistance must be called before any use of the distances")
        return (self.xpr, self.xpl, self.ypf, self.ypb, self.zpu, self.zpd)

    @property
    def min_dist(self):
        xpr, xpl, ypf, ypb, zpu, zpd = self._dist()
        return torch.minimum(torch.minimum(xpr, xpl), torch.minimum(torch.minimum(ypf, ypb), torch.minimum(zpu, zpd)))

    # -- setDistance.m:3-33 -----------------------------------------------------------------
    def setDistance(self):
        size = self.GD3.Size
        if self.xpr is not None and tuple(self.xpr.shape) == size and self.xpr.dtype == self.dtype:
            d = list(self._dist())  # rewritten in place (keeps recorded graphs valid)
        else:
            d = [colmajor_empty(size, self.dtype) for _ in range(6)]
        ws = self.workspace("set_distance")
        lib().call(self._fn("vsl_set_distance"), _ptr(self.F), *map(_ptr, d), *self.GD3.args(), _ptr(ws), ws.numel(),
                   _stream())
        self.xpr, self.xpl, self.ypf, self.ypb, self.zpu, self.zpd = d

    # -- reinitialization ------------------------------------------------------------------
    def WENO5RK3Reinitialization(self, F, iteration: int):
        """WENO5RK3Reinitialization.m:3-43 (cached distances of setDistance)."""
        out = self._field(F).clone()
        ws = self.workspace("reinit_weno5")
        lib().call(self._fn("vsl_weno5_rk3_reinitialization"), _ptr(out), int(iteration), *map(_ptr, self._dist()),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return out

    def WENO5RK3ReinitializationTol(self, F, max_iters: int, tol: float, band: float | None = None,
                                    history: bool = True):
        """WENO5RK3Reinitialization run until its residual is at most `tol` (no counterpart in
        the reference, whose loop runs a fixed count): the FP64 maximum over |F| < band
        (default 3 Ds) of | |grad F|_G - 1 |, tested on the device after every pseudo-step,
        at most `max_iters` pseudo-steps.  Returns (F, status, residual) as device tensors:
        status = [pseudo-steps taken, 1 if converged], residual[n] after n pseudo-steps
        (entries past the stop stay NaN), or None with history=False."""
        out = self._field(F).clone()
        ws = self.workspace("reinit_tol")
        band = 3 * self.GD3.Ds if band is None else float(band)
        status = torch.zeros(2, dtype=torch.int32, device="cuda")
        res = torch.full((int(max_iters) + 1,), float("nan"), dtype=torch.float64, device="cuda") if history else None
        lib().call(self._fn("vsl_weno5_rk3_reinitialization_tol"), _ptr(out), int(max_iters), float(tol), band,
                   *map(_ptr, self._dist()), *self.GD3.args(), _ptr(status), _ptr(res), _ptr(ws), ws.numel(),
                   _stream())
        return out, status, res

    def WENORK3Reinitialization(self, F, iteration: int):
        """WENORK3Reinitialization.m:3-61 (cubic distances recomputed from F)."""
        out = self._field(F).clone()
        ws = self.workspace("reinit_eno3")
        lib().call(self._fn("vsl_wenork3_reinitialization"), _ptr(out), int(iteration), *self.GD3.args(), _ptr(ws),
                   ws.numel(), _stream())
        return out

    def ENORK2Reinitialization(self, F, iteration: int):
        """ENORK2Reinitialization.m:3-45: quadratic-ENO distances recomputed from F, Heun RK2
        pseudo-steps with the second-order ENO Godunov Hamiltonian."""
        out = self._field(F).clone()
        ws = self.workspace("reinit_enork2")
        lib().call(self._fn("vsl_enork2_reinitialization"), _ptr(out), int(iteration), *self.GD3.args(), _ptr(ws),
                   ws.numel(), _stream())
        return out

    # -- extension ---------------------------------------------------------------------------
    def WENO5RK3Extend(self, C, iteration: int):
        """WENO5RK3Extend.m:9-76."""
        out = self._field(C).clone()
        ws = self.workspace("extend_weno5")
        lib().call(self._fn("vsl_weno5_rk3_extend"), _ptr(out), int(iteration), _ptr(self.F), *map(_ptr, self._dist()),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return out

    def WENORK3Extend(self, C, iteration: int):
        """WENORK3Extend.m:9-98."""
        out = self._field(C).clone()
        ws = self.workspace("extend_eno3")
        lib().call(self._fn("vsl_wenork3_extend"), _ptr(out), int(iteration), _ptr(self.F), *self.GD3.args(), _ptr(ws),
                   ws.numel(), _stream())
        return out

    def ENORK2Extend(self, C, iteration: int):
        """ENORK2Extend.m:9-81: C extended off the zero set of self.F (quadratic-ENO distances
        and ENO upwind normals of F, quadratic crossing values of C, Heun RK2)."""
        out = self._field(C).clone()
        ws = self.workspace("extend_enork2")
        lib().call(self._fn("vsl_enork2_extend"), _ptr(out), int(iteration), _ptr(self.F), *self.GD3.args(),
                   _ptr(ws), ws.numel(), _stream())
        return out

    # -- surface redistance -------------------------------------------------------------------
    def WENO5RK3ClosetPointSurfaceRedistance(self, A, iter1: int, iter2: int):
        """WENO5RK3ClosetPointSurfaceRedistance.m:4-157."""
        out = self._field(A).clone()
        ws = self.workspace("surface_redistance")
        lib().call(self._fn("vsl_weno5_rk3_surface_redistance"), _ptr(out), int(iter1), int(iter2), _ptr(self.F),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return out

    def WENORK3ClosetPointSurfaceRedistance(self, A, iter1: int, iter2: int):
        """WENORK3ClosetPointSurfaceRedistance.m:4-152: the WENO5 method's composition with
        the cubic distances, the WENORK3 normals, crossing values and extension step and the
        ENO3 interface scheme of the reinitialization."""
        out = self._field(A).clone()
        ws = self.workspace("surface_redistance_eno3")
        lib().call(self._fn("vsl_wenork3_surface_redistance"), _ptr(out), int(iter1), int(iter2), _ptr(self.F),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return out

    def ENORK2ClosetPointSurfaceRedistance(self, A, iter1: int, iter2: int):
        """ENORK2ClosetPointSurfaceRedistance.m:4-128 (second-order ENO, Heun RK2)."""
        out = self._field(A).clone()
        ws = self.workspace("surface_redistance_enork2")
        lib().call(self._fn("vsl_enork2_surface_redistance"), _ptr(out), int(iter1), int(iter2), _ptr(self.F),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return out

    # -- calculus toolbox and integrals ----------------------------------------------------
    def GPUsetCalculusToolBox(self):
        """GPUsetCalculusToolBox.m:2-42: the 18 toolbox fields (computed in FP64)."""
        f64 = as_field(self.F, torch.float64)
        hp = torch.clamp(f64, min=0)  # HPrimal = max(F, 0)
        outs = [colmajor_empty(self.GD3.Size, torch.float64) for _ in TOOLBOX_FIELDS]
        lib().call("vsl_set_calculus_toolbox", *map(_ptr, outs), _ptr(f64), _ptr(hp), *self.GD3.args(), self.GD3.Ds,
                   self.GD3.NumElt, _stream())
        for name, t in zip(TOOLBOX_FIELDS, outs):
            setattr(self, name, t if self.dtype == torch.float64 else t.to(self.dtype))
        self.HPrimal = hp

    def area_volume(self) -> torch.Tensor:
        """Device tensor [area, volume] (SDF3.m:73-80), FP64 fixed-order sums."""
        out = torch.empty(2, dtype=torch.float64, device="cuda")
        ws = self.workspace("area_volume")
        lib().call(self._fn("vsl_area_volume"), _ptr(self.F), _ptr(out), *self.GD3.args(), _ptr(ws), ws.numel(),
                   _stream())
        return out

    def calArea(self) -> float:
        return float(self.area_volume()[0])

    def calVolume(self) -> float:
        return float(self.area_volume()[1])

    def _masked_integral(self, A, f0, f1, f2, one_minus) -> float:
        out = torch.empty(1, dtype=torch.float64, device="cuda")
        ws = self.workspace("masked_integral")
        fs = [None if t is None else self._field(t) for t in (A, f0, f1, f2, one_minus)]
        lib().call(self._fn("vsl_masked_integral"), _ptr(self.F), *map(_ptr, fs), _ptr(out), *self.GD3.args(),
                   _ptr(ws), ws.numel(), _stream())
        return float(out)

    def surfaceIntegral(self, field) -> float:
        """SDF3.m:82-85: sum of (field DiracDelta) FGradMag over |F| < 2Ds, times Ds^3 (FP64);
        the toolbox fields of the last GPUsetCalculusToolBox."""
        return self._masked_integral(None, field, self.DiracDelta, self.FGradMag, None)

    # -- the auxiliary level set of multiphase vesicles ----------------------------------
    def GPUAsetCalculusToolBox(self, fields=None):
        """GPUAsetCalculusToolBox.m:2-63: the toolbox of the auxiliary level set self.A on
        self.F, stored as attributes (AUX_FIELDS; `fields` limits it to a subset), from A and F
        alone.  AHPrimal = max(A, 0) as the MATLAB method sets it."""
        if self.A is None:
            raise ValueError("set the auxiliary level set (obj.A) first")
        import ctypes

        self.A = self._field(self.A)
        names = AUX_FIELDS if fields is None else tuple(fields)
        unknown = set(names) - set(AUX_FIELDS)
        if unknown:
            raise ValueError(f"unknown auxiliary toolbox fields: {sorted(unknown)}")
        outs = {n: colmajor_empty(self.GD3.Size, self.dtype) for n in names}
        ptrs = (ctypes.c_void_p * len(AUX_FIELDS))(*[_ptr(outs.get(n)) or None for n in AUX_FIELDS])
        ws = self.workspace("aux_toolbox")
        lib().call(self._fn("vsl_a_set_calculus_toolbox"), _ptr(self.A), _ptr(self.F), ctypes.addressof(ptrs),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        for n, t in outs.items():
            setattr(self, n, t)
        self.AHPrimal = torch.clamp(self.A, min=0)

    def calLength(self) -> float:
        """SDF3.m:212-215: length of the curve A = 0 on F = 0, sum of AFDiracDelta NormCrossAF
        over |F|, |A| < 2Ds, times Ds^3 (FP64)."""
        return self._masked_integral(self.A, self.AFDiracDelta, self.NormCrossAF, None, None)

    def LineIntegral(self, field) -> float:
        """SDF3.m:216-219: the integral of field along the curve A = 0 on F = 0."""
        return self._masked_integral(self.A, field, self.AFDiracDelta, self.NormCrossAF, None)

    def AcalArea(self) -> float:
        """SDF3.m:220-223: area of the part of the surface where A < 0."""
        return self._masked_integral(None, self.DiracDelta, None, None, self.AHeaviside)

    def AsurfaceIntegral(self, field) -> float:
        """SDF3.m:224-227: the surface integral of field over the part where A < 0."""
        return self._masked_integral(None, field, self.DiracDelta, self.FGradMag, self.AHeaviside)

    def BivalueField(self, valNeg, valPos):
        """SDF3.m:228-232: valPos where A > 0 and valNeg where A < 0, blended by AHeaviside."""
        return valPos * self.AHeaviside + valNeg * (1 - self.AHeaviside)

    # -- advection and the composite step ----------------------------------------------------
    def WENO5RK3Advection(self, F, vx, vy, vz, dt, steps: int = 1):
        """F advanced `steps` WENO5 TVD-RK3 steps of phi_t + v.grad(phi) = 0 with time step dt."""
        out = self._field(F).clone()
        v = [self._field(a) for a in (vx, vy, vz)]
        dtt = dt if isinstance(dt, torch.Tensor) else torch.tensor([float(dt)], dtype=torch.float64, device="cuda")
        ws = self.workspace("advection")
        lib().call(self._fn("vsl_weno5_rk3_advection"), _ptr(out), *map(_ptr, v), _ptr(dtt), int(steps),
                   *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return out

    def vesicle_step(self, ext_iters: int = 30, reinit_iters: int = 20, cfl: float = 0.5, info=None,
                     graph: bool = False) -> torch.Tensor:
        """One vesicle step in place on self.F and its cached distances; returns the device
        tensor [area, volume, dt, max|Vn|].

        graph=True records the step's whole launch sequence (about 300 kernels and memsets
        for 30 + 20 pseudo-steps) once as a CUDA graph and replays it; the graph is
        re-recorded when the arguments or the field/distance buffers change."""
        if graph:
            return self._vesicle_step_graph(int(ext_iters), int(reinit_iters), float(cfl))
        info = torch.empty(4, dtype=torch.float64, device="cuda") if info is None else info
        ws = self.workspace("vesicle_step")
        lib().call(self._fn("vsl_vesicle_step"), _ptr(self.F), *map(_ptr, self._dist()), int(ext_iters),
                   int(reinit_iters), float(cfl), _ptr(info), *self.GD3.args(), _ptr(ws), ws.numel(), _stream())
        return info

    def relax_step(self, A0: float, V0: float, kappa: float = 1.0, spon_c: float = 0.0, cfl: float = 0.5,
                   alpha: float = 0.5, ext_iters: int = 100, reinit_iters: int = 0, info=None,
                   graph: bool = False) -> torch.Tensor:
        """One pass of the single-phase relaxation driver's time loop
        (p00_test_singlephase_relax.m:60-196, without plotting) in place on self.F and its
        cached distances: bending speed from the extended mean curvature, tension and
        pressure enforcing the area A0 and volume V0, the smoothed normal speed, the
        explicit update, setDistance, and `reinit_iters` reinitialization pseudo-steps
        (0: none).  Returns the device tensor of 11 values {area, volume, Dt, max|NSB|,
        int H^2, int H, int H NSB, int NSB, tension, pressure, energy}.  graph=True records
        the step's launches (toolbox, extensions, reductions, FFTs, update, setDistance,
        reinitialization) as one CUDA graph on first use and replays it; the returned tensor
        is then the graph's own, overwritten by the next replay."""
        if self.xpr is None:
            self.setDistance()
        ws = self.workspace("relax_step")
        args = (float(A0), float(V0), float(kappa), float(spon_c), float(cfl), float(alpha), int(ext_iters),
                int(reinit_iters))

        def launch(out):
            lib().call(self._fn("vsl_relax_step"), _ptr(self.F), *map(_ptr, self._dist()), *args, _ptr(out),
                       *self.GD3.args(), _ptr(ws), ws.numel(), _stream())

        if not graph:
            info = torch.empty(11, dtype=torch.float64, device="cuda") if info is None else info
            launch(info)
            return info
        # one graph per argument set (a driver alternating steps with and without the
        # reinitialization keeps two); a new field or workspace drops the recorded ones
        bufs = (_ptr(self.F), tuple(map(_ptr, self._dist())), _ptr(ws))
        if getattr(self, "_relax_graph_bufs", None) != bufs:
            self._relax_graphs, self._relax_graph_bufs = {}, bufs
        entry = self._relax_graphs.get(args)
        if entry is None:
            out = torch.empty(11, dtype=torch.float64, device="cuda")
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                launch(out)
            entry = self._relax_graphs[args] = (g, out)
        entry[0].replay()
        if info is not None:
            info.copy_(entry[1])
            return info
        return entry[1]

    def _vesicle_step_graph(self, ext_iters: int, reinit_iters: int, cfl: float) -> torch.Tensor:
        key = (ext_iters, reinit_iters, cfl, _ptr(self.F), tuple(map(_ptr, self._dist())))
        if getattr(self, "_graph_key", None) != key:
            ws = self.workspace("vesicle_step")
            self._graph_info = torch.empty(4, dtype=torch.float64, device="cuda")
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                lib().call(self._fn("vsl_vesicle_step"), _ptr(self.F), *map(_ptr, self._dist()), ext_iters,
                           reinit_iters, cfl, _ptr(self._graph_info), *self.GD3.args(), _ptr(ws), ws.numel(),
                           _stream())
            self._graph, self._graph_key = g, key
        self._graph.replay()
        return self._graph_info


def ellipsoid_phi(x, y, z, a: float, b: float, c: float):
    """sqrt(x^2/a^2 + y^2/b^2 + z^2/c^2) - 1 (Ellipsoid.m:45)."""
    return torch.sqrt(x**2 / a**2 + y**2 / b**2 + z**2 / c**2) - 1


def reduced_volume(area: float, volume: float) -> float:
    """(3V/4pi) (4pi/A)^(3/2) (p00_test_singlephase_relax.m:32)."""
    return (3 * volume / 4 / math.pi) * (4 * math.pi / area) ** 1.5
