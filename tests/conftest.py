import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU and libstart_gpu.so")


@pytest.fixture(scope="session")
def built():
    """Builds libstart_gpu.so and the oracle once per session."""
    from start_gb300.build import build_library
    from oracle.build import build_oracle

    return build_library(), build_oracle()
