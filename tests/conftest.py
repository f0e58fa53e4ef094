import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def hgb_lib():
    """The built libhipacc_gb300.so (compiled in-tree if missing)."""
    from hipacc_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(hgb_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hipacc_gb300 import api

    api.init(0)
    return api


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "hipacc_ref_golden.npz"))
