"""Parity metric between the CUDA path and the reference / oracle.

Bars (FP64 path):
  * rclass, thclass, crossing counts, masks: bit-exact;
  * r: |dr| <= 1e-10 |r|;
  * theta, phi: |dx| <= 1e-10 max(|x|, 1)  (angles, radians);
  * t, sigma: |dx| <= 1e-10 max(|x|, r_o)  (their natural scale is the light travel
    time r_o: at tau = 0 both are sums of O(r_o) terms that cancel to 0, so the
    reference itself carries ~1e-11 r_o of rounding there);
  * non-finite patterns (NaN / inf) identical.
The last Mino sample of a ray that ends on the horizon (rclass 2, 3, 4) lies
(1 - maxtaufrac) tau_tot = 1e-10 tau_tot before the horizon, where t and phi diverge
logarithmically; their condition number there is ~1e10, so both the reference and this
implementation carry ~1e-6 relative rounding noise at that one sample. t, phi and sigma at
that sample are held to 1e-4 relative instead; every other sample to the bars above.
"""
import numpy as np

TOL = 1e-10
TOL_HORIZON = 1e-4


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


def check_trace(got, ref, r_o, rclass, name='', tol=TOL, tol_horizon=TOL_HORIZON, exclude=None):
    """got / ref: dicts with t, r, th, ph, sig arrays (ngeo, npix). Returns max errors."""
    ngeo = ref['r'].shape[0]
    horizon = np.isin(rclass, (2, 3, 4))
    last = np.zeros(ref['r'].shape, dtype=bool)
    if ngeo > 1:
        last[-1, :] = horizon
    keep = np.ones(ref['r'].shape, dtype=bool)
    if exclude is not None:
        keep[:, exclude] = False
    out = {}
    tscale = r_o if np.isfinite(r_o) else 1.0
    for k, scale in (('r', 0.0), ('th', 1.0), ('ph', 1.0), ('t', tscale), ('sig', tscale)):
        x, y = np.asarray(got[k])[:, keep[0]], np.asarray(ref[k])[:, keep[0]]
        _mask_pattern(x, y, name + ':' + k)
        e = rel_err(x, y, scale if scale > 0 else 1e-300)
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
