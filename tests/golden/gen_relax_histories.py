"""Extract the relaxation histories the reference recorded with its own runs into a small
fixture, ``relax_histories.npz`` beside this script.

The reference ships MATLAB v5 files written by ``p00_test_singlephase_relax.m:198-300``
(``save('CFL0_5', 't0_5', 'ene0_5', ...)``): per time step the accumulated time t, the
energy int (H - c0)^2, the relative area and volume changes at the start of the step
(DiffArea / 100, DiffVolume / 100), the pressure P and the tension.  Each run starts from
``SD.Shape.Ellipsoid(GridSize, 0.6, 'O', 0.35)``, setDistance and 500 reinitialization
pseudo-steps, with kappa 1 and SponC 0.  The first FIRST entries of every history are kept
(key ``<file>/<field>``); the grid and CFL number of each run are in ``<file>/grid`` and
``<file>/cfl`` where the file's name or its first time step gives them (the CFL runs are
at 96^3: their first time steps are CFL / 0.1 times that of the CFL 0.1 run).

It reads the reference checkout, so it runs in the development container only; the
fixture is committed.

    python tests/golden/gen_relax_histories.py
"""
from __future__ import annotations

import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build_oracle  # noqa: E402

SRC = build_oracle.reference_vesicle()
FIRST = 8
FIELDS = ("t", "ene", "da", "dv", "P", "ten")
# file -> (variable suffix, grid edge, CFL number)
RUNS = {
    "CFL0_05": ("0_05", None, 0.05),
    "CFL0_1": ("0_1", 96, 0.1),
    "CFL0_25": ("0_25", 96, 0.25),
    "CFL0_5": ("0_5", 96, 0.5),
    "CFL1": ("1", 96, 1.0),
    "oblate48": ("48", 48, None),
    "oblate64": ("64", 64, None),
    "oblate80": ("80", 80, None),
    "oblate96": ("96", 96, None),
    "oblate128": ("128", 128, None),
}


def main():
    out = {}
    for name, (suf, grid, cfl) in RUNS.items():
        d = sio.loadmat(os.path.join(SRC, name + ".mat"))
        for f in FIELDS:
            out[f"{name}/{f}"] = np.ravel(d[f + suf])[:FIRST].astype(np.float64)
        out[f"{name}/length"] = np.array(np.ravel(d["t" + suf]).size)
        out[f"{name}/grid"] = np.array(-1 if grid is None else grid)
        out[f"{name}/cfl"] = np.array(np.nan if cfl is None else cfl)
    path = os.path.join(HERE, "relax_histories.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays")


if __name__ == "__main__":
    main()
