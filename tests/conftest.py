import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for path in (ROOT, ROOT / "ratpoints-gpu_gb300", ROOT / "oracle"):
    if str(path) not in sys.path:
        sys.path.insert(0, str(path))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())


@pytest.fixture(scope="session")
def rpg():
    """The built library binding (builds in-tree on first use)."""
    import ratpoints_gb300

    ratpoints_gb300.build()
    ratpoints_gb300.load()
    return ratpoints_gb300


@pytest.fixture(scope="session")
def oracle():
    import ratpoints_oracle

    ratpoints_oracle.build()
    return ratpoints_oracle
