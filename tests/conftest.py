import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_built():
    """Build the CUDA library (no-op when up to date) for GPU tests."""
    from flow_structure_interaction_fem_ibm_gb300.build import build_all
    build_all()
    from flow_structure_interaction_fem_ibm_gb300 import _native
    return _native.solver()
