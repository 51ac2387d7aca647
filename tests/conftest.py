import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "sph-particle-simulator_gb300"
sys.path.insert(0, str(PKG / "python"))
sys.path.insert(0, str(REPO / "oracle"))
sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden" / "sph_ref_golden.npz"
GOLDEN_CASES = ("lattice", "exact", "edge", "collapse")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    import sphx_build

    sphx_build.build_sphx()
    sphx_build.build_oracle()
    return True


@pytest.fixture(scope="session")
def port(built):
    import sph_oracle as O

    return O.Port()


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def golden_case(golden, name):
    g = {k.split("/", 1)[1]: golden[k] for k in golden.files if k.startswith(name + "/")}
    return g
