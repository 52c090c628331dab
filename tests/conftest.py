import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_small.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs libcontract.so kernels")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def c_oracle():
    from oracle import lib as L
    L.build()
    c = L.c_oracle()
    assert c is not None, "oracle/_ref/liboracle.so failed to build"
    return c


def rel_err(got, ref):
    got = np.asarray(got)
    ref = np.asarray(ref)
    scale = np.abs(ref).max()
    if scale == 0:
        return float(np.abs(got).max())
    return float(np.abs(got - ref).max() / scale)
