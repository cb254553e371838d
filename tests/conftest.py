import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libapbf_gb300.so")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "reference_known_answers.json").read_text())["tests"]


@pytest.fixture(scope="session")
def orc():
    """The oracle (test infrastructure), built on demand."""
    from oracle import oracle as o

    o.build()
    return o


@pytest.fixture(scope="session")
def native_lib():
    """The CUDA library; on a machine with a GPU it must exist (built by __graft_entry__.build())."""
    from apbf_gb300 import build as b

    b.build()
    from apbf_gb300 import _native

    return _native.load()


@pytest.fixture(scope="session")
def cuda(native_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return torch.device("cuda:0")
