"""The elliptic-Pi adapter on the GPU (kgeo_ellip_pi, through the drop-in
kgeo_gb300.scipy_ellip_binding.ellip_pi_arr) against the reference's ellip_pi_arr
(kgeo/scipy_ellip_binding.py:87-237) on 608 points: random in-domain values, n > 1, and one
point for each special case (phi ~ 0 of both signs, n = 1 beyond a quarter period, n = inf,
m sin^2 > 1, m < -1e14, the pole 1 - n sin^2 = 0). Every compiled copy of the kernels'
arithmetic is checked: the per-ray setup's (FMA contraction off), the direct sample
evaluators' and the standalone adapter."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def binding():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kgeo_gb300 import scipy_ellip_binding
    return scipy_ellip_binding


@pytest.mark.parametrize('form', ['setup', 'samples', 'adapter'])
def test_ellip_pi_vs_reference_fixture(binding, golden, form):
    g = golden('ellip_pi')
    got = binding.ellip_pi_arr(g['n'], g['phi'], g['m'], form=form)
    ref = g['pi']
    assert np.array_equal(np.isfinite(got), np.isfinite(ref))
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(got[np.isinf(ref)], ref[np.isinf(ref)])
    fin = np.isfinite(ref)
    # beyond |phi| > pi/2 Pi is a sum of O(1) periodic and incomplete parts: absolute scale 1;
    # next to the pole 1 - n sin^2 phi = 0 (one fixture point sits on it up to rounding) Pi
    # carries rounding ~eps / rho, the parity rule of tests/parity.py
    rho = np.abs(1 - g['n'] * np.sin(g['phi']) ** 2)
    bar = np.where(g['n'] > 0, np.maximum(1e-13, 10 * 2.220446049250313e-16 / np.maximum(rho, 1e-300)), 1e-13)
    err = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)
    assert np.all(err <= bar[fin]), (err / bar[fin]).max()
    if form == 'setup':
        # the setup's arithmetic rounds one operation at a time, as numpy does
        assert np.max(err) < 1e-13
    # the special-case points come out exactly as the reference's
    special = slice(600, 608)
    fs = np.isfinite(ref[special])
    assert np.array_equal(got[special][~fs], ref[special][~fs], equal_nan=True)


def test_ellip_pi_broadcasting_like_reference(binding, golden):
    """1-d n, m against a 2-d phi are repeated along phi's first axis; scalars work."""
    g = golden('ellip_pi')
    n, m = g['n'][:50], g['m'][:50]
    phi = np.stack([g['phi'][:50], 0.5 * g['phi'][:50]])
    got = binding.ellip_pi_arr(n, phi, m)
    assert got.shape == (2, 50)
    np.testing.assert_array_equal(got[0], binding.ellip_pi_arr(n, phi[0], m))
    np.testing.assert_array_equal(got[1], binding.ellip_pi_arr(n, phi[1], m))
    v = binding.ellip_pi_arr(0.3, 0.7, 0.2)
    assert v.shape == (1,) and abs(v[0] - 0.745431064313508) < 1e-14  # mpmath.ellippi(0.3, 0.7, 0.2)
