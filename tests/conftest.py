import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if p.stem != "search")


def load_golden(name):
    import numpy as np
    d = np.load(GOLDEN / f"{name}.npz")
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def sblas_lib():
    """The CUDA library, built in-tree if needed (never a fallback)."""
    from hpda_sblas_pnnl_gb300 import _lib
    return _lib.load(build_if_missing=True)


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda:0")
