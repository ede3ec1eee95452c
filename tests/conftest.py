import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden():
    """The reference afft library's own outputs (tests/golden/make_golden.py)."""
    import json
    import numpy as np
    here = os.path.join(ROOT, "tests", "golden")
    z = np.load(os.path.join(here, "afft_golden.npz"))
    idx = json.load(open(os.path.join(here, "afft_golden.json")))
    return z, idx["cases"]


@pytest.fixture(scope="session")
def golden64():
    """The reference afft library's own double outputs (afft_64_*, scalar
    backend; tests/golden/make_golden.py --f64).  Inputs are float32 values
    to be widened to double."""
    import json
    import numpy as np
    here = os.path.join(ROOT, "tests", "golden")
    z = np.load(os.path.join(here, "afft_golden64.npz"))
    idx = json.load(open(os.path.join(here, "afft_golden64.json")))
    return z, idx["cases"]
