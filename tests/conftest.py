import os
import sys
from pathlib import Path

import pytest

# Under pytest-xdist every worker would start an OpenMP team as wide as the
# machine for the oracle; one thread per worker keeps them from starving
# each other (a team's threads spin while they wait)
if os.environ.get("PYTEST_XDIST_WORKER"):
    os.environ.setdefault("OMP_NUM_THREADS", "1")

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_lib():
    from dgcom_gb300 import _build, abi

    _build.build()
    return abi.cuda_library()


@pytest.fixture(scope="session")
def reference_data():
    """A data file of the reference repository (read-only, CPU tests only),
    found under the directory the DGCOM_REFERENCE environment variable
    names, or a skip where it is unset or the file is absent."""
    root = os.environ.get("DGCOM_REFERENCE")

    def get(relative: str) -> Path:
        if not root:
            pytest.skip("DGCOM_REFERENCE (the reference repository's root) is not set")
        path = Path(root) / relative
        if not path.is_file():
            pytest.skip(f"reference data {relative} not present")
        return path

    return get
