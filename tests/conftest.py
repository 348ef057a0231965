import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libfastipc.so')
    config.addinivalue_line('markers', 'slow: long-running parity case')


@pytest.fixture(scope='session')
def unit_golden():
    import numpy as np
    return np.load(os.path.join(GOLDEN, 'unit_kernels.npz'))


@pytest.fixture(scope='session')
def newton_golden():
    import numpy as np
    return np.load(os.path.join(GOLDEN, 'newton_two_cubes_n3.npz'))


@pytest.fixture(scope='session')
def newton2d_golden():
    import numpy as np
    return np.load(os.path.join(GOLDEN, 'newton2d_two_squares_n3.npz'))
