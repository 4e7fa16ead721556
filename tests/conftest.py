import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the liblvn kernels")


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all"], check=True)
    yield


@pytest.fixture(scope="session")
def lvn_gpu():
    """liblvn initialised on cuda:0 (noise seed 1, default material 0)."""
    import leven_gb300 as lvn

    lvn.initialise(1, 0, 2)
    yield lvn
