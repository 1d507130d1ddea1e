import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, 'tests', 'golden')

# element triplet values must match to this norm-wise relative tolerance:
# max |v - v_ref| <= REL_TOL * max |v_ref| over each element's block
REL_TOL = 1e-12


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built library')


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if cuda_available():
        return
    skip = pytest.mark.skip(reason='no CUDA device in this environment')
    for item in items:
        if 'gpu' in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope='session')
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name + '.npz'))
    return load


@pytest.fixture(scope='session')
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope='session')
def gpulib():
    """Build (if needed) and load the CUDA library; the tests call through it."""
    from pyfe3d_gb300 import build, _lib
    build.build()
    return _lib.load()


def blockwise_rel_err(v, ref, block):
    v = np.asarray(v).reshape(-1, block)
    ref = np.asarray(ref).reshape(-1, block)
    scale = np.abs(ref).max(axis=1)
    scale[scale == 0] = 1.
    return (np.abs(v - ref).max(axis=1) / scale).max()
