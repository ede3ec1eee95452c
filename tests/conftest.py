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


@pytest.fixture(scope="session")
def golden_configs():
    """afft's own float outputs at the benchmark configurations' full sizes,
    sampled at stored indices (tests/golden/make_golden.py --configs); the
    inputs are regenerated from each case's mt19937 seed."""
    import json
    import numpy as np
    here = os.path.join(ROOT, "tests", "golden")
    z = np.load(os.path.join(here, "afft_golden_configs.npz"))
    idx = json.load(open(os.path.join(here, "afft_golden_configs.json")))
    return z, idx["cases"]


def config_case_inputs(case):
    """The inputs of a config-size golden case (tests/golden/make_golden.py)."""
    import numpy as np
    from oracle import oracle as O
    kind, dims, seed = case["kind"], case["dims"], case["seed"]
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    if kind in ("c", "ci"):
        v = O.mt19937_uniform(2 * n, seed)
        return v[:n], v[n:]
    if kind == "r":
        return O.mt19937_uniform(n, seed), None
    v = O.mt19937_uniform(2 * h, seed)
    return v[:h], v[h:]
