import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        d = {k: z[k] for k in z.files}
    d["n"] = int(d["n"])
    d["posdef"] = bool(d["posdef"])
    d["flag"] = int(d["flag"])
    d["inertia"] = tuple(int(v) for v in d["inertia"])
    if "closed_inertia" in d:
        d["closed_inertia"] = tuple(int(v) for v in d["closed_inertia"])
    d["name"] = name
    return d


@pytest.fixture(scope="session")
def sylver():
    import sylver_gb300
    sylver_gb300.build()
    return sylver_gb300.load() and sylver_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gpu(sylver):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return True
