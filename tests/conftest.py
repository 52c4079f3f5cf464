import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / 'tests' / 'golden'
sys.path.insert(0, str(ROOT))
import __graft_entry__  # noqa: E402

__graft_entry__.reference_source()


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GB300 device (run with -m gpu)')


def load_golden(name):
    with np.load(GOLDEN / f'golden_{name}.npz', allow_pickle=False) as d:
        return {k: d[k] for k in d.files}


@pytest.fixture(scope='session')
def tiny8():
    return load_golden('tiny8')


@pytest.fixture(scope='session')
def device_library():
    """The built C-ABI library on a GPU machine (built on demand); the GPU tests call through it."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pcbqs_gb300 import build
    build.build()
    from pcbqs_gb300 import _lib
    return _lib.load()
