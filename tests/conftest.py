import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def _ensure_library():
    """Several test modules import the package, whose ctypes binding needs libtnx.so at import
    time: build it (nvcc cross-compiles without a GPU) before collection when it is missing."""
    if os.environ.get("TNX_LIB") or (ROOT / "tnpy_gb300" / "libtnx.so").exists():
        return
    import __graft_entry__

    __graft_entry__.build()


_ensure_library()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libtnx")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def pytest_collection_modifyitems(config, items):
    # keep the CPU suite single-threaded-BLAS friendly and deterministic
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    np.set_printoptions(precision=12)
