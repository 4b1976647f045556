import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    g = ROOT / "tests" / "golden"
    arrays = np.load(g / "golden.npz")
    index = json.loads((g / "index.json").read_text())
    return arrays, index


@pytest.fixture(scope="session")
def native():
    """The native library, built in tree when missing; GPU tests fail loudly without it."""
    from redblackgraph_gb300 import build, _lib
    build.build()
    return _lib.load()
