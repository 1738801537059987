import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "2018_7_vesicle_gb300"
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ("sphere14", "aniso", "merge15", "tiny", "slab", "pear14")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build_oracle
    from oracle import oracle as O

    build_oracle.build_port()
    return O


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module(PKG_NAME)


@pytest.fixture(scope="session")
def vsl(pkg):
    """The loaded CUDA library (built on demand)."""
    pkg.build()
    return pkg.lib()


def load_golden(name):
    import numpy as np

    d = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    return {k: d[k] for k in d.files}
