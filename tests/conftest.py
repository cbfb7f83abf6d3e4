import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden', 'golden_ref.npz')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a GB300 GPU (runs on the GPU host)')


@pytest.fixture(scope='session')
def golden():
    with np.load(GOLDEN) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope='session')
def gpu():
    """The GPU tests' entry fixture: builds the library if needed and fails loudly when
    no GB300 is visible (a GPU test must never pass on a CPU path)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail('GPU test selected but no CUDA device is visible')
    from gravitation_gb300 import build as gbuild
    gbuild.build()
    from gravitation_gb300.engine import device_info
    return device_info(0)
