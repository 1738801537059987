"""Host side of the relaxation driver (no GPU): the history files in the reference's
MATLAB naming, and the committed first entries of the reference's own records."""
import importlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_history_mat_roundtrip(tmp_path):
    pytest.importorskip("scipy")
    import scipy.io as sio

    R = importlib.import_module("2018_7_vesicle_gb300.relax")
    rng = np.random.default_rng(0)
    hist = {f: rng.standard_normal(7) for f in R.FIELDS}
    path = str(tmp_path / "CFL0_5.mat")
    R.save_history(path, hist, "0_5")
    raw = sio.loadmat(path)
    # the driver's variable names and shapes: ene a column, the others rows
    assert raw["ene0_5"].shape == (7, 1) and raw["t0_5"].shape == (1, 7) and raw["ten0_5"].shape == (1, 7)
    back = R.load_history(path)
    for f in R.FIELDS:
        assert np.array_equal(back[f], hist[f])
    assert np.array_equal(R.load_history(path, "0_5")["P"], hist["P"])


def test_reference_records_fixture():
    G = np.load(os.path.join(HERE, "golden", "relax_histories.npz"))
    runs = {k.split("/")[0] for k in G.files}
    assert {"CFL0_5", "CFL0_05", "oblate64", "oblate80", "oblate96", "oblate128"} <= runs
    for r in runs:
        t = G[f"{r}/t"]
        assert np.all(np.diff(t) > 0) and t[0] > 0  # accumulated time
        assert G[f"{r}/da"][0] == 0 and G[f"{r}/dv"][0] == 0  # changes at the first step's start
        assert int(G[f"{r}/length"]) >= t.size
    # the CFL study at 96^3: the first time step scales with the CFL number
    t0 = {c: float(G[f"CFL{c}/t"][0]) for c in ("0_1", "0_25", "0_5", "1")}
    for c, v in (("0_25", 2.5), ("0_5", 5.0), ("1", 10.0)):
        assert abs(t0[c] / t0["0_1"] - v) < 1e-9 * v
