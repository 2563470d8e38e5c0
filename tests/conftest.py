import importlib
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "clbm_ibm-moving-airfoil_gb300"
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def pytest_collection_modifyitems(config, items):
    # tests marked gpu that also carry "slow" run after the quick ones of the same file
    pass


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module(PKG_NAME)


@pytest.fixture(scope="session")
def built_pkg(pkg):
    """The package with its CUDA library compiled (nvcc cross-compiles without a GPU)."""
    pkg.build()
    return pkg


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build as ob
    ob.build()
    from oracle import oracle
    return oracle


def load_golden(name):
    return np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))


def golden_inflow(d):
    a = math.radians(float(d["AoA0_deg"]))
    u = float(d["U_inf"])
    return float(u * math.cos(a)), float(-u * math.sin(a))


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
