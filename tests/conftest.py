import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension')


@pytest.fixture
def golden():
    import numpy as np

    def load(name):
        with np.load(os.path.join(GOLDEN, name + '.npz')) as f:
            return {k: f[k] for k in f.files}
    return load


# Rays of the 2048^2 grid over [-10, 10] M at a = 0.94, theta_o = 17 deg (ngeo = 256), as (row,
# column) of the grid, whose radial Pi passes within rho ~ 1.0e-3 of its pole late in a
# 64-sample recurrence chunk: with a flat 1e-3 re-seed zone phi missed the 1e-10 bar there
# (1.21x at row 837, column 683, sample 63).
PI_ZONE_RAYS = ((837, 683), (837, 682), (837, 684), (836, 683), (838, 683))
