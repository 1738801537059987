"""The plain FP64 reference GPU form (TEST AND MEASUREMENT INFRASTRUCTURE ONLY): the
reference's own CUDA kernels, compiled for sm_103a from the reference checkout by
oracle/ref/Makefile into PTX (oracle/_ref/ptx/, see gpu_shim.cuh), loaded through the CUDA
driver and launched with the reference's geometry, ThreadBlockSize = [mrows,
floor(256/mrows), 1] and GridSize = ceil([mrows ncols lshts] ./ ThreadBlockSize)
(V/+SD/@SDF3/GPUInitialize.m:7-10).  The MATLAB glue around them (elementwise gpuArray
arithmetic, min, sum) is restated with torch FP64 tensor operations on the GPU, in the
order of the same MATLAB methods the CPU oracle (oracle.py) restates:

* setDistance.m:5-21 -> set_distance
* WENO5RK3Reinitialization.m:7-39 / WENORK3Reinitialization.m:7-57 -> reinit_weno5 / reinit_eno3
* WENO5RK3Extend.m:11-74 -> extend_weno5
* GPUsetCalculusToolBox.m:2-42, SDF3.m:73-80 -> calculus_toolbox, cal_area, cal_volume
* GD3.WENODotGrad (GD3.m:393-398) in the TVD-RK3 combination -> advect_rk3
* the composite vesicle step of oracle.vesicle_step -> vesicle_step

Fields are torch FP64 tensors of shape (rows, cols, pges) in the reference's column-major
storage (strides 1, rows, rows*cols).  Nothing of this is part of the product: tests check
it against the CPU oracle and the bench times it as the reference's GPU path.
"""
from __future__ import annotations

import ctypes
import math
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
PTX_DIR = os.path.join(HERE, "_ref", "ptx")
MODULES = {
    "gpu_boundary_location.ptx": ("boundary_location",),
    "gpu_re_step_weno5.ptx": ("re_step",),
    "gpu_reinit_eno3.ptx": ("cubic_boundary_correction", "re_step_eno3"),
    "gpu_upwind_normal_weno5.ptx": ("upwind_normal",),
    "gpu_interpolant_weno5.ptx": ("boundary_interpolant",),
    "gpu_extend_step_weno5.ptx": ("extend_step",),
    "gpu_toolbox.ptx": ("set_calculus_toolbox",),
    "gpu_advection.ptx": ("advection_step",),
}
# argument kinds per kernel (p pointer, i int, d double), the reference prototypes
_G = "iiiddd"
SIGS = {
    "boundary_location": "ppppppp" + "i" + _G,
    "re_step": "pppp" + "pppppp" + _G + "i",
    "cubic_boundary_correction": "ppppppp" + "i" + _G,
    "re_step_eno3": "pppp" + "pppppp" + _G + "i",
    "upwind_normal": "pppp" + "pppppp" + _G + "i",
    "boundary_interpolant": "pppppp" + "pppppp" + "p" + _G + "i",
    "extend_step": "pppppp" + "pppppp" + "pppppp" + _G + "i",
    "set_calculus_toolbox": "p" * 18 + "pp" + _G + "d" + "i",
    "advection_step": "ppppp" + _G,
}


def available() -> bool:
    return all(os.path.exists(os.path.join(PTX_DIR, m)) for m in MODULES)


class RefKernels:
    """The reference's kernels on the current CUDA device (modules JIT-loaded from PTX)."""

    def __init__(self):
        if not available():
            raise RuntimeError(f"reference PTX not built ({PTX_DIR}); oracle/ref/Makefile builds it where the "
                               "reference checkout is")
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the runtime's primary context is current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.fn = {}
        self._mods = []
        for name, kernels in MODULES.items():
            with open(os.path.join(PTX_DIR, name), "rb") as f:
                image = f.read() + b"\0"
            mod = ctypes.c_void_p()
            self._check(self.cu.cuModuleLoadData(ctypes.byref(mod), ctypes.c_char_p(image)), f"load {name}")
            self._mods.append(mod)
            for k in kernels:
                fn = ctypes.c_void_p()
                self._check(self.cu.cuModuleGetFunction(ctypes.byref(fn), mod, f"vslref_{k}".encode()), k)
                self.fn[k] = fn

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"CUDA driver error {rc} in {what}")

    def launch(self, name, rows, cols, pges, *args):
        """One launch with the reference geometry of a rows x cols x pges grid, on torch's
        current stream."""
        bx, by = rows, 256 // rows
        if by < 1:
            raise ValueError("the reference launch geometry needs rows <= 256")
        grid = (math.ceil(rows / bx), math.ceil(cols / by), pges)
        sig = SIGS[name]
        vals = []
        for kind, a in zip(sig, args):
            if kind == "p":
                vals.append(ctypes.c_void_p(a.data_ptr() if isinstance(a, torch.Tensor) else a))
            elif kind == "i":
                vals.append(ctypes.c_int(int(a)))
            else:
                vals.append(ctypes.c_double(float(a)))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._check(self.cu.cuLaunchKernel(self.fn[name], *grid, bx, by, 1, 0, stream, params, None), name)


# ---------------------------------------------------------------------------------------
# the MATLAB glue on torch FP64 tensors (column-major fields)
# ---------------------------------------------------------------------------------------


def field(a) -> torch.Tensor:
    """A (rows, cols, pges) FP64 CUDA tensor with column-major storage."""
    if not isinstance(a, torch.Tensor):
        import numpy as np

        a = np.asarray(a, dtype=np.float64)
        r, c, p = a.shape
        a = torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).view(p, c, r).permute(2, 1, 0)
    a = a.to(device="cuda", dtype=torch.float64)
    if not a.permute(2, 1, 0).is_contiguous():
        a = a.permute(2, 1, 0).contiguous().permute(2, 1, 0)
    return a


def empty_like(f: torch.Tensor, fill=None) -> torch.Tensor:
    r, c, p = f.shape
    t = torch.empty((p, c, r), dtype=torch.float64, device="cuda").permute(2, 1, 0)
    if fill is not None:
        t.fill_(fill)
    return t


class Grid:
    def __init__(self, rows, cols, pges, dx, dy, dz):
        self.rows, self.cols, self.pges = rows, cols, pges
        self.dx, self.dy, self.dz = dx, dy, dz
        self.ds = (dx + dy + dz) / 3
        self.num = rows * cols * pges

    def args(self):
        return (self.rows, self.cols, self.pges, self.dx, self.dy, self.dz)


class RefGpu:
    """The reference's GPU path: its kernels and the MATLAB methods' glue on one grid."""

    def __init__(self, g: Grid, kernels: RefKernels | None = None):
        self.g = g
        self.K = kernels or RefKernels()

    def launch(self, name, *args):
        self.K.launch(name, self.g.rows, self.g.cols, self.g.pges, *args)

    # setDistance.m:5-21
    def set_distance(self, F, cubic=False):
        g = self.g
        d = [empty_like(F, g.dx), empty_like(F, g.dx), empty_like(F, g.dy), empty_like(F, g.dy),
             empty_like(F, g.dz), empty_like(F, g.dz)]
        self.launch("cubic_boundary_correction" if cubic else "boundary_location", *d, F, g.num, *g.args())
        return d

    @staticmethod
    def min_dist(d):
        return torch.minimum(torch.minimum(torch.minimum(d[0], d[1]), torch.minimum(d[2], d[3])),
                             torch.minimum(d[4], d[5]))

    @staticmethod
    def rk3(F, stage):
        step = stage(F)
        t1 = F - step
        step = stage(t1)
        t2 = t1 - step
        t05 = 3.0 / 4.0 * F + 1.0 / 4.0 * t2
        step = stage(t05)
        t15 = t05 - step
        return 1.0 / 3.0 * F + 2.0 / 3.0 * t15

    def _reinit(self, F, iteration, d, kernel):
        g = self.g
        mask = F < 0
        deltat = 0.3 * self.min_dist(d)
        step = empty_like(F)

        def stage(Fs):
            Fs = field(Fs)
            self.launch(kernel, step, Fs, mask, deltat, *d, *g.args(), g.num)
            return step.clone()

        for _ in range(iteration):
            F = self.rk3(F, stage)
        return field(F)

    # WENO5RK3Reinitialization.m:7-39 (the object's cached distances d)
    def reinit_weno5(self, F, iteration, d):
        return self._reinit(field(F), iteration, d, "re_step")

    # WENORK3Reinitialization.m:7-57 (cubic distances of the input)
    def reinit_eno3(self, F, iteration):
        F = field(F)
        return self._reinit(F, iteration, self.set_distance(F, cubic=True), "re_step_eno3")

    # WENO5RK3Extend.m:11-74
    def extend_weno5(self, F, d, C, iteration):
        g = self.g
        F, C = field(F), field(C)
        n = [empty_like(F) for _ in range(3)]
        self.launch("upwind_normal", *n, F, *d, *g.args(), g.num)
        mag = torch.sqrt(n[0] ** 2 + n[1] ** 2 + n[2] ** 2).clamp(min=1e-6)
        s = torch.sign(F)
        v = [field(s * (a / mag)) for a in n]
        deltat = 0.3 * self.min_dist(d)
        cp = [empty_like(F) for _ in range(6)]
        self.launch("boundary_interpolant", *cp, *d, C, *g.args(), g.num)
        step = empty_like(F)

        def stage(Cs):
            Cs = field(Cs)
            self.launch("extend_step", step, deltat, Cs, *v, *d, *cp, *g.args(), g.num)
            return step.clone()

        for _ in range(iteration):
            C = self.rk3(C, stage)
        return field(C)

    # GPUsetCalculusToolBox.m:2-42
    def calculus_toolbox(self, F):
        g = self.g
        F = field(F)
        hp = field(torch.clamp(F, min=0))
        names = ("Fx", "Fy", "Fz", "FGradMag", "Nx", "Ny", "Nz", "Fxx", "Fyy", "Fzz", "Fxy", "Fyz", "Fzx",
                 "FLaplacian", "MeanCurvature", "GaussianCurvature", "Heaviside", "DiracDelta")
        out = [empty_like(F) for _ in names]
        self.launch("set_calculus_toolbox", *out, F, hp, *g.args(), g.ds, g.num)
        return dict(zip(names, out))

    # SDF3.m:73-80
    def cal_area(self, F, delta):
        mask = F.abs() < 2 * self.g.ds
        return float(delta[mask].sum()) * self.g.ds**3

    def cal_volume(self, F, heaviside):
        mask = F < 2 * self.g.ds
        return float((1 - heaviside[mask]).sum()) * self.g.ds**3

    def advect_rk3(self, F, vx, vy, vz, dt, steps=1):
        g = self.g
        vx, vy, vz = field(vx), field(vy), field(vz)
        out = empty_like(vx)

        def stage(Fs):
            Fs = field(Fs)
            self.launch("advection_step", out, vx, vy, vz, Fs, *g.args())
            return dt * out

        F = field(F)
        for _ in range(steps):
            F = self.rk3(F, stage)
        return field(F)

    def vesicle_step(self, F, d, ext_iters=30, reinit_iters=20, cfl=0.5):
        """The composite step of oracle.vesicle_step (toolbox -> area/volume -> extension of
        the mean curvature -> dt -> advection along Vn*N -> setDistance -> reinitialization)."""
        g = self.g
        F = field(F)
        tb = self.calculus_toolbox(F)
        area = self.cal_area(F, tb["DiracDelta"])
        volume = self.cal_volume(F, tb["Heaviside"])
        vn = self.extend_weno5(F, d, tb["MeanCurvature"], ext_iters)
        band = F.abs() < 2 * g.ds
        vmax = float(vn[band].abs().max())
        dt = cfl * g.ds / vmax
        F = self.advect_rk3(F, vn * tb["Nx"], vn * tb["Ny"], vn * tb["Nz"], dt)
        d = self.set_distance(F)
        F = self.reinit_weno5(F, reinit_iters, d)
        return F, d, {"area": area, "volume": volume, "dt": dt, "vmax": vmax}
