import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "reference_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and librealcaustics.so")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture
def in_tmpdir(tmp_path, monkeypatch):
    # the reference writes D:\*.obj files into the working directory
    monkeypatch.chdir(tmp_path)
    return tmp_path


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle
    lib = oracle.reference()
    if lib is None:
        pytest.skip("reference sources not available on this host (golden fixtures cover it)")
    return lib
