"""Host-side argument handling of the elliptic-Pi drop-in (no GPU needed): the reference's
shape rule and exception text (kgeo/scipy_ellip_binding.py:95-106), checked before any launch."""
import numpy as np
import pytest


def test_last_dimension_mismatch_raises_reference_message():
    from kgeo_gb300 import scipy_ellip_binding as b
    with pytest.raises(Exception, match='inputs to ellip_pi_arr do not have same last dimension!'):
        b.ellip_pi_arr(np.zeros(3), np.zeros(4), np.zeros(3))


def test_no_cpu_path():
    torch = pytest.importorskip('torch')
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from kgeo_gb300 import scipy_ellip_binding as b
    with pytest.raises(RuntimeError, match='needs a CUDA device'):
        b.ellip_pi_arr(np.array([0.3]), np.array([0.7]), np.array([0.2]))
