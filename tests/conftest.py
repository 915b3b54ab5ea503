import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

REF_FIXTURE_DIR = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def mesh_lib():
    from solver_gb300 import build
    return build.build_mesh()


@pytest.fixture(scope="session")
def cuda_lib():
    from solver_gb300 import build
    return build.build_cuda()
