"""The oracle's auxiliary level set toolbox against the reference's own kernel
(golden_auxi.npz, written by tests/golden/gen_golden_auxi.py from the host build of
auxi_set_calculus_toolbox.cu): the 27 kernel fields bit for bit, and the integrals of
SDF3.m:82-85, 212-227.  No GPU."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("plane", "cap")


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "golden_auxi.npz"))


def case(O, G, name):
    x, y, z = np.meshgrid(G[f"{name}/xv"], G[f"{name}/yv"], G[f"{name}/zv"])
    return O.grid_from_mesh(x, y, z), x, y, z, G[f"{name}/F"], G[f"{name}/A"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_auxiliary_toolbox_matches_reference(oracle_mod, golden, name):
    O = oracle_mod
    g, x, y, z, F, A = case(O, golden, name)
    aux, tb = O.auxiliary_toolbox(O.kernels("port"), g, F, A)
    for n in O.AUX_FIELDS:
        assert np.array_equal(aux[n], golden[f"{name}/{n}"]), n
    fld = O.F64(np.sin(2 * x) * np.cos(y) + z)
    got = {
        "calLength": O.cal_length(g, F, A, aux),
        "LineIntegral": O.line_integral(g, F, A, fld, aux),
        "AcalArea": O.a_cal_area(g, F, tb, aux),
        "AsurfaceIntegral": O.a_surface_integral(g, F, fld, tb, aux),
        "surfaceIntegral": O.surface_integral_mask(g, F, fld, tb["DiracDelta"], tb["FGradMag"]),
    }
    for k, v in got.items():
        assert v == float(golden[f"{name}/{k}"]), k
    assert got["calLength"] > 0 and got["AcalArea"] > 0


def test_crpow_oracle_within_ulps(oracle_mod, golden):
    """The oracle built with correctly rounded integer powers (the GPU's FP64 form) differs
    from the libm-pow build only in the last bits of the power-dependent fields."""
    O = oracle_mod
    g, x, y, z, F, A = case(O, golden, "cap")
    aux, _ = O.auxiliary_toolbox(O.kernels("port_crpow"), g, F, A)
    for n in O.AUX_FIELDS:
        ref = golden[f"cap/{n}"]
        assert np.abs(aux[n] - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1e-300), n
