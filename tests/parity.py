"""Parity metric between the CUDA path and the reference / oracle: the bars of
oracle/parity.py (their statement and the conditioning allowances are documented there),
applied with the non-finite pattern checks of the tests."""
import numpy as np

from oracle.parity import (EPS, SENS_FACTOR, TOL, lambda_eta_sensitivity, parity_ratios,  # noqa: F401
                           rel_err)


def _mask_pattern(x, y, name):
    fx, fy = np.isfinite(x), np.isfinite(y)
    assert np.array_equal(fx, fy), '%s: finite pattern differs at %d entries' % (name, int((fx != fy).sum()))
    assert np.array_equal(np.isnan(x), np.isnan(y)), '%s: NaN pattern differs' % name
    ix = np.isinf(x)
    assert np.array_equal(x[ix], y[ix]), '%s: inf signs differ' % name
    return fx


def check_trace(got, ref, r_o, rclass, name='', tol=TOL, exclude=None, rho=None, sens=None):
    """got / ref: dicts with t, r, th, ph, sig arrays (nsamp, npix); rho: optional (nsamp, npix)
    pole distances (oracle.kgeo_oracle.pole_distance); sens: optional lambda_eta_sensitivity
    callable, consulted for the rays that exceed the other bars. rclass is kept for the
    callers' signature. Returns the largest error relative to each sample's bar, per output."""
    keep = np.ones(np.asarray(ref['r']).shape[1], dtype=bool)
    if exclude is not None:
        keep[exclude] = False
    for k in ('r', 'th', 'ph', 't', 'sig'):
        x, y = np.asarray(got[k], dtype=float), np.asarray(ref[k], dtype=float)
        _mask_pattern(x[:, keep], y[:, keep], name + ':' + k)
    sub_got = {k: np.asarray(got[k], dtype=float)[:, keep] for k in ('r', 'th', 'ph', 't', 'sig')}
    sub_ref = {k: np.asarray(ref[k], dtype=float)[:, keep] for k in ('r', 'th', 'ph', 't', 'sig')}
    sub_rho = None if rho is None else np.asarray(rho, dtype=float)[:, keep]
    kept = np.nonzero(keep)[0]
    sub_sens = None if sens is None else (lambda cols: sens(kept[cols]))
    ratio = parity_ratios(sub_got, sub_ref, r_o, tol, sub_rho, sub_sens)
    out = {}
    for k in ('r', 'th', 'ph', 't', 'sig'):
        m = ratio[k].max() if ratio[k].size else 0.0
        assert m <= tol, '%s:%s max err %.3g > %.1g (relative to the bar)' % (name, k, m, tol)
        out[k] = m
    return out
