"""Parity metric between the CUDA path and the reference / oracle.

Bars (FP64 path):
  * rclass, thclass, crossing counts, masks: bit-exact;
  * r: |dr| <= 1e-10 |r|;
  * theta, phi: |dx| <= 1e-10 max(|x|, 1)  (angles, radians);
  * t, sigma: |dx| <= 1e-10 max(|x|, r_o)  (their natural scale is the light travel
    time r_o: at tau = 0 both are sums of O(r_o) terms that cancel to 0, so the
    reference itself carries ~1e-11 r_o of rounding there);
  * non-finite patterns (NaN / inf) identical.
Two conditioning exceptions, both measured against an mpmath evaluation:
  * the last Mino sample of a ray that ends on the horizon (rclass 2, 3, 4) lies
    (1 - maxtaufrac) tau_tot = 1e-10 tau_tot before the horizon, where t and phi diverge
    logarithmically and an elliptic-Pi characteristic sits on its pole (rho ~ 1e-14 when
    the characteristic is within 1e-6 of 1); one ulp of sn moves the value by up to 1e-3
    relative, so t, phi and sigma at that sample are held to 1e-2;
  * a sample whose amplitude lies within rho = |1 - n sin^2| of a Pi pole (n > 1, or n just
    below 1 at a turning point near the polar axis): there the reference's Pi and the R1/S1
    combinations that cancel its pole carry rounding ~eps / rho, so the bar for that sample
    is max(1e-10, 10 eps / rho) (rho from oracle.kgeo_oracle.pole_distance when given).
"""
import numpy as np

TOL = 1e-10
TOL_HORIZON = 1e-2
EPS = 2.220446049250313e-16


def _mask_pattern(x, y, name):
    fx, fy = np.isfinite(x), np.isfinite(y)
    assert np.array_equal(fx, fy), '%s: finite pattern differs at %d entries' % (name, int((fx != fy).sum()))
    assert np.array_equal(np.isnan(x), np.isnan(y)), '%s: NaN pattern differs' % name
    ix = np.isinf(x)
    assert np.array_equal(x[ix], y[ix]), '%s: inf signs differ' % name
    return fx


def rel_err(x, y, scale):
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    fin = np.isfinite(x) & np.isfinite(y)
    e = np.zeros(x.shape)
    e[fin] = np.abs(x[fin] - y[fin]) / np.maximum(np.abs(y[fin]), scale if np.isscalar(scale) else scale[fin])
    return e


def check_trace(got, ref, r_o, rclass, name='', tol=TOL, tol_horizon=TOL_HORIZON, exclude=None, rho=None):
    """got / ref: dicts with t, r, th, ph, sig arrays (ngeo, npix); rho: optional (ngeo, npix)
    pole distances (oracle.kgeo_oracle.pole_distance). Returns max errors relative to each
    sample's bar."""
    ngeo = ref['r'].shape[0]
    horizon = np.isin(rclass, (2, 3, 4))
    last = np.zeros(ref['r'].shape, dtype=bool)
    if ngeo > 1:
        last[-1, :] = horizon
    keep = np.ones(ref['r'].shape, dtype=bool)
    if exclude is not None:
        keep[:, exclude] = False
    out = {}
    bar = np.full(ref['r'].shape, float(tol))
    if rho is not None:
        bar = np.maximum(bar, 10 * EPS / np.maximum(np.asarray(rho, dtype=float), 1e-300))
    tscale = r_o if np.isfinite(r_o) else 1.0
    for k, scale in (('r', 0.0), ('th', 1.0), ('ph', 1.0), ('t', tscale), ('sig', tscale)):
        x, y = np.asarray(got[k])[:, keep[0]], np.asarray(ref[k])[:, keep[0]]
        _mask_pattern(x, y, name + ':' + k)
        e = rel_err(x, y, scale if scale > 0 else 1e-300) / bar[:, keep[0]] * tol
        l = last[:, keep[0]]
        if k in ('t', 'ph', 'sig'):
            body = e[~l].max() if (~l).any() else 0.0
            edge = e[l].max() if l.any() else 0.0
            assert body <= tol, '%s:%s max err %.3g > %.1g' % (name, k, body, tol)
            assert edge <= tol_horizon, '%s:%s horizon-sample err %.3g > %.1g' % (name, k, edge, tol_horizon)
            out[k] = (body, edge)
        else:
            m = e.max() if e.size else 0.0
            assert m <= tol, '%s:%s max err %.3g > %.1g' % (name, k, m, tol)
            out[k] = m
    return out
