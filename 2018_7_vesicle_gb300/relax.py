"""The single-phase relaxation driver (p00_test_singlephase_relax.m) without its plotting:
set-up, the time loop over SDF3.relax_step, and the history it records, read and written
as MATLAB v5 files in the reference's own variable naming (``save('CFL0_5', 't0_5',
'ene0_5', 'da0_5', 'dv0_5', 'P0_5', 'ten0_5')``, p00_test_singlephase_relax.m:198-300).

    x, y, z, F = shapes.oblate_ellipsoid((96, 96, 96), 0.6, 0.35, device="cuda")
    m, A0, V0 = relax_setup(GD3(x, y, z), F, "f64")
    hist = relax_run(m, A0, V0, total_time=1.6e-3, cfl=0.5)
    save_history("CFL0_5.mat", hist, "0_5")
"""
from __future__ import annotations

import numpy as np

from .sdf3 import GD3, SDF3

FIELDS = ("t", "ene", "da", "dv", "P", "ten")


def relax_setup(grid: GD3, F, precision: str = "f64", reinit_iters: int = 500):
    """The driver's set-up (p00_test_singlephase_relax.m:24-35): the level-set object,
    setDistance, `reinit_iters` WENO5 RK3 reinitialization pseudo-steps, and its area and
    volume, the targets of the loop.  Returns (object, A0, V0)."""
    m = SDF3(grid, Val=F, precision=precision)
    m.setDistance()
    if reinit_iters > 0:
        m.F = m.WENO5RK3Reinitialization(m.F, reinit_iters)
    A0, V0 = (float(v) for v in m.area_volume().cpu())
    return m, A0, V0


def relax_run(m: SDF3, A0: float, V0: float, steps: int | None = None, total_time: float | None = None,
              cfl: float = 0.5, reinit_rate: int = 1, reinit_iters: int = 100, kappa: float = 1.0,
              spon_c: float = 0.0, alpha: float = 0.5, ext_iters: int = 100, graph: bool = False) -> dict:
    """The time loop (p00_test_singlephase_relax.m:60-196): steps until `steps` steps are
    taken or the time reaches `total_time` (at least one of them is given).  The iteration
    counter starts at 1 and is advanced at the top of the loop, so the reinitialization at
    the end of a step runs when the advanced counter is a multiple of `reinit_rate`.
    Returns the history {"t", "ene", "da", "dv", "P", "ten"} as numpy arrays: the time
    after each step, the energy int (H - c0)^2, the relative area and volume changes at
    the start of the step, the pressure and the tension."""
    if steps is None and total_time is None:
        raise ValueError("give steps, total_time or both")
    if reinit_rate < 1:
        raise ValueError("reinit_rate must be >= 1")
    rows = {f: [] for f in FIELDS}
    time, i, n = 0.0, 1, 0
    while (steps is None or n < steps) and (total_time is None or time < total_time):
        i += 1
        re = reinit_iters if i % reinit_rate == 0 else 0
        info = m.relax_step(A0, V0, kappa=kappa, spon_c=spon_c, cfl=cfl, alpha=alpha, ext_iters=ext_iters,
                            reinit_iters=re, graph=graph).cpu().numpy()
        time += float(info[2])
        rows["t"].append(time)
        rows["ene"].append(info[10])
        rows["da"].append((info[0] - A0) / A0)
        rows["dv"].append((info[1] - V0) / V0)
        rows["P"].append(info[9])
        rows["ten"].append(info[8])
        n += 1
    return {f: np.asarray(v, dtype=np.float64) for f, v in rows.items()}


def save_history(path: str, hist: dict, suffix: str) -> None:
    """Write the history as the driver's MATLAB file: variables t<suffix>, ene<suffix>,
    ... with ene a column and the others rows, as the driver's arrays are."""
    import scipy.io as sio

    out = {}
    for f in FIELDS:
        v = np.asarray(hist[f], dtype=np.float64)
        out[f + suffix] = v.reshape(-1, 1) if f == "ene" else v.reshape(1, -1)
    sio.savemat(path, out)


def load_history(path: str, suffix: str | None = None) -> dict:
    """Read a history written by the driver (or save_history): {"t", "ene", ...} as flat
    arrays.  The suffix is found from the file's variables when not given."""
    import scipy.io as sio

    d = {k: v for k, v in sio.loadmat(path).items() if not k.startswith("__")}
    if suffix is None:
        ts = [k for k in d if k.startswith("t") and not k.startswith("ten")]
        if len(ts) != 1:
            raise ValueError(f"{path}: cannot tell the history's suffix from {sorted(d)}")
        suffix = ts[0][1:]
    return {f: np.ravel(d[f + suffix]).astype(np.float64) for f in FIELDS}
