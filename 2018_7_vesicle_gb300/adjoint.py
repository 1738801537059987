"""Differentiable level-set transport.

A field is advanced `steps` WENO5 TVD-RK3 advection steps with a fixed time step under a
velocity field (vx, vy, vz); after every `reinit_every` steps it is reinitialized
(setDistance with degree-5 roots, then `reinit_iters` WENO5 TVD-RK3 pseudo-steps), the
composition of GD3.WENODotGrad / SDF3.WENO5RK3Reinitialization the vesicle code uses.
`transport(...)` is a torch.autograd.Function: its backward pass runs the hand-written
adjoint kernels of the C ABI (vsl_weno5_rk3_advection_adjoint_*,
vsl_weno5_rk3_reinitialization_adjoint_*) and returns dL/dphi0 and dL/dv.

Memory: the forward pass keeps one checkpoint field every `checkpoint_every` steps; the
backward pass recomputes one segment at a time from its checkpoint (storing that
segment's step inputs) and sweeps it in reverse.  The recomputation uses the forward
kernels, so it reproduces the forward states bit for bit.

The time step is a constant of the map (CFL * dx / max|v| evaluated once by the caller);
the max in that rule is not differentiated.

The module also holds the pieces of the differentiation workload: divergence-free
Fourier velocity modes, the smoothed Heaviside and the Heaviside-mismatch loss.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import lib
from .sdf3 import GD3, _DTYPES, _ptr, _stream, as_field, colmajor_empty


@dataclass(frozen=True)
class TransportPlan:
    steps: int = 40
    reinit_every: int = 10
    reinit_iters: int = 10
    checkpoint_every: int = 10

    def segments(self):
        """[(first step, end step)) of each checkpoint segment."""
        c = max(1, int(self.checkpoint_every))
        return [(s, min(s + c, self.steps)) for s in range(0, self.steps, c)]

    def reinit_after(self, s: int) -> bool:
        return self.reinit_every > 0 and self.reinit_iters > 0 and (s + 1) % self.reinit_every == 0


class Transport:
    """Forward and adjoint sweeps of the transport map on one grid and precision."""

    def __init__(self, grid: GD3, dt: float, plan: TransportPlan = TransportPlan(), precision: str = "f32"):
        if precision not in _DTYPES:
            raise ValueError(f"precision must be one of {sorted(_DTYPES)}")
        self.grid = grid
        self.plan = plan
        self.precision = precision
        self.dtype = _DTYPES[precision]
        self.elem = 8 if precision == "f64" else 4
        self.dt = torch.tensor([float(dt)], dtype=torch.float64, device="cuda")
        self._ws = {}
        self._dist = None
        self._tape = None

    # -- plumbing ------------------------------------------------------------------------
    def _fn(self, base: str) -> str:
        return f"{base}_{self.precision}"

    def _args(self):
        return self.grid.args()

    def _workspace(self, op: str) -> torch.Tensor:
        n = lib().workspace_bytes(op, *self.grid.Size, self.elem)
        ws = self._ws.get(op)
        if ws is None or ws.numel() < n:
            ws = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
            self._ws[op] = ws
        return ws

    def field(self, a) -> torch.Tensor:
        return as_field(a, self.dtype)

    # -- forward pieces (in place) ---------------------------------------------------------
    def advect(self, phi: torch.Tensor, v) -> None:
        ws = self._workspace("advection")
        lib().call(self._fn("vsl_weno5_rk3_advection"), _ptr(phi), *map(_ptr, v), _ptr(self.dt), 1, *self._args(),
                   _ptr(ws), ws.numel(), _stream())

    def reinitialize(self, phi: torch.Tensor) -> None:
        if self._dist is None:
            self._dist = [colmajor_empty(self.grid.Size, self.dtype) for _ in range(6)]
        ws = self._workspace("set_distance")
        lib().call(self._fn("vsl_set_distance"), _ptr(phi), *map(_ptr, self._dist), *self._args(), _ptr(ws),
                   ws.numel(), _stream())
        ws = self._workspace("reinit_weno5")
        lib().call(self._fn("vsl_weno5_rk3_reinitialization"), _ptr(phi), int(self.plan.reinit_iters),
                   *map(_ptr, self._dist), *self._args(), _ptr(ws), ws.numel(), _stream())

    def run(self, phi: torch.Tensor, v, first: int = 0, end: int | None = None, record=None) -> None:
        """Steps [first, end) in place; with `record` a list, append ('adv', input) and
        ('re', input) for every advection step and reinitialization."""
        end = self.plan.steps if end is None else end
        for s in range(first, end):
            if record is not None:
                record.append(("adv", phi.clone()))
            self.advect(phi, v)
            if self.plan.reinit_after(s):
                if record is not None:
                    record.append(("re", phi.clone()))
                self.reinitialize(phi)

    # -- adjoint pieces ----------------------------------------------------------------------
    def advect_adjoint(self, phi_in: torch.Tensor, v, lam: torch.Tensor, gv) -> None:
        ws = self._workspace("advection_adjoint")
        lib().call(self._fn("vsl_weno5_rk3_advection_adjoint"), _ptr(phi_in), *map(_ptr, v), _ptr(self.dt),
                   _ptr(lam), *map(_ptr, gv), *self._args(), _ptr(ws), ws.numel(), _stream())

    def reinit_adjoint(self, phi_in: torch.Tensor, lam: torch.Tensor) -> None:
        k = int(self.plan.reinit_iters)
        n = self.grid.NumElt * k
        if self._tape is None or self._tape.numel() < n:
            self._tape = torch.empty(n, dtype=self.dtype, device="cuda")
        ws = self._workspace("reinit_adjoint")
        lib().call(self._fn("vsl_weno5_rk3_reinitialization_adjoint"), _ptr(phi_in), k, _ptr(lam),
                   _ptr(self._tape), *self._args(), _ptr(ws), ws.numel(), _stream())

    def __call__(self, phi0: torch.Tensor, vx: torch.Tensor, vy: torch.Tensor, vz: torch.Tensor) -> torch.Tensor:
        return _TransportFn.apply(phi0, vx, vy, vz, self)


class _TransportFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phi0, vx, vy, vz, tr: Transport):
        v = [tr.field(a) for a in (vx, vy, vz)]
        phi = tr.field(phi0).clone()
        checkpoints = []
        for first, end in tr.plan.segments():
            checkpoints.append(phi.clone())
            tr.run(phi, v, first, end)
        ctx.tr = tr
        ctx.v = v
        ctx.checkpoints = checkpoints
        return phi

    @staticmethod
    def backward(ctx, grad_out):
        tr: Transport = ctx.tr
        v, checkpoints = ctx.v, ctx.checkpoints
        lam = tr.field(grad_out).clone()
        gv = [torch.zeros_like(a) for a in v]
        for (first, end), ck in reversed(list(zip(tr.plan.segments(), checkpoints))):
            record = []
            tr.run(ck.clone(), v, first, end, record=record)
            for kind, x in reversed(record):
                if kind == "adv":
                    tr.advect_adjoint(x, v, lam, gv)
                else:
                    tr.reinit_adjoint(x, lam)
            del record
        return lam, gv[0], gv[1], gv[2], None


def transport(phi0, vx, vy, vz, grid: GD3, dt: float, plan: TransportPlan = TransportPlan(), precision: str = "f32"):
    """phi_T of the transport map (differentiable in phi0, vx, vy, vz)."""
    return Transport(grid, dt, plan, precision)(phi0, vx, vy, vz)


# ---------------------------------------------------------------------------------------
# the differentiation workload
# ---------------------------------------------------------------------------------------


def fourier_modes(grid: GD3, count: int = 8, kmax: float = 3.0, seed: int = 0, dtype=torch.float64):
    """`count` divergence-free velocity modes u_m(x) = p_m sin(2 pi k_m . x / L + theta_m):
    integer wave vectors with 1 <= |k_m| <= kmax drawn without repetition, unit
    polarisations p_m orthogonal to k_m (so div u_m = 0), phases uniform in [0, 2 pi), L
    the box length along each axis.  Returns a tensor (count, 3, rows, cols, pges) of
    column-major fields (x, y, z components)."""
    rng = np.random.default_rng(seed)
    r = int(math.floor(kmax))
    ks = [(a, b, c) for a in range(-r, r + 1) for b in range(-r, r + 1) for c in range(-r, r + 1)
          if 1 <= math.sqrt(a * a + b * b + c * c) <= kmax]
    pick = rng.choice(len(ks), size=count, replace=False)
    X, Y, Z = grid.X, grid.Y, grid.Z
    L = [float(t.max() - t.min()) + s for t, s in ((X, grid.Dx), (Y, grid.Dy), (Z, grid.Dz))]
    out = torch.empty((count, 3) + tuple(grid.Size), dtype=dtype, device=X.device)
    for m, idx in enumerate(pick):
        k = np.array(ks[idx], dtype=float)
        p = rng.standard_normal(3)
        p -= k * (p @ k) / (k @ k)
        p /= np.linalg.norm(p)
        theta = rng.uniform(0.0, 2 * math.pi)
        arg = 2 * math.pi * (k[0] * X / L[0] + k[1] * Y / L[1] + k[2] * Z / L[2]) + theta
        s = torch.sin(arg)
        for a in range(3):
            out[m, a] = (p[a] * s).to(dtype)
    return out


def velocity(amplitudes: torch.Tensor, modes: torch.Tensor):
    """(vx, vy, vz) = sum_m a_m u_m as column-major fields (differentiable in a)."""
    v = torch.einsum("m,mapqr->apqr", amplitudes.to(modes.dtype), modes)
    return [v[a].permute(2, 1, 0).contiguous().permute(2, 1, 0) for a in range(3)]


def smoothed_heaviside(phi: torch.Tensor, eps: float) -> torch.Tensor:
    """H_eps(phi) = 0 below -eps, 1 above eps, 1/2 (1 + phi/eps + sin(pi phi/eps)/pi) between."""
    t = torch.clamp(phi / eps, -1.0, 1.0)
    mid = 0.5 * (1.0 + t + torch.sin(math.pi * t) / math.pi)
    return torch.where(t <= -1.0, torch.zeros_like(t), torch.where(t >= 1.0, torch.ones_like(t), mid))


def heaviside_mismatch(phi: torch.Tensor, target: torch.Tensor, eps: float, cell_volume: float) -> torch.Tensor:
    """sum over cells of (H_eps(phi) - H_eps(target))^2 dx^3, in FP64."""
    d = smoothed_heaviside(phi.double(), eps) - smoothed_heaviside(target.double(), eps)
    return (d * d).sum() * cell_volume


def time_step(amplitudes, modes, grid: GD3, cfl: float = 0.5) -> float:
    """CFL * min spacing / max |v| of the velocity of `amplitudes` (a constant of the map)."""
    with torch.no_grad():
        v = torch.einsum("m,mapqr->apqr", torch.as_tensor(amplitudes, dtype=modes.dtype, device=modes.device), modes)
        vmax = float(v.abs().amax())
    return cfl * min(grid.Dx, grid.Dy, grid.Dz) / max(vmax, 1e-12)
