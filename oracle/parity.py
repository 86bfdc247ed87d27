"""Parity bars between the CUDA path and the reference / oracle.

TEST INFRASTRUCTURE ONLY (the checker, like oracle.kgeo_oracle): used by ``tests/`` and by the
checker legs of ``bench.py`` (after the GPU timings). The product package never imports it.

Bars (FP64 path), per sample:
  * rclass, thclass, crossing counts, masks: bit-exact;
  * r: |dr| <= 1e-10 |r|;
  * theta, phi: |dx| <= 1e-10 max(|x|, 1)  (angles, radians);
  * t, sigma: |dx| <= 1e-10 max(|x|, r_o)  (at tau = 0 both are exactly 0, and the
    reference returns sums of O(r_o) terms that cancel to up to 1e-10 r_o there);
  * non-finite patterns (NaN / inf) identical.
Two conditioning allowances widen a sample's bar, each an estimate of how far the
reference's own FP64 value can lie from the exact one; tests/test_conditioning_cpu.py
measures the reference and the kernel arithmetic against 30-digit integrations of the
equations of motion at such samples:
  * pole rule: a sample whose elliptic amplitude lies within rho = |1 - n sin^2| of an
    elliptic-Pi pole (oracle.kgeo_oracle.pole_distance) carries rounding amplified by
    ~1/rho (the Pi, the R1/S1 combinations that cancel its pole, and the radial formula
    r ~ 1/(1 - n0 sn^2)); the bar is max(1e-10, 10 eps / rho). This covers the last sample
    of a horizon-bound ray, 1e-10 tau_tot before the horizon, where a Pi characteristic
    sits within rho ~ 1e-12 of its pole and the reference's phi is off by up to 1e-5;
  * input conditioning (rays next to the critical curve): where a ray's output moves by S
    when lambda or eta moves by one ulp (lambda_eta_sensitivity), the bar is at least 10 S.
    Evaluated only for the rays that exceed the other bars.
"""
import contextlib

import numpy as np

TOL = 1e-10
EPS = 2.220446049250313e-16
SENS_FACTOR = 10.0


def rel_err(x, y, scale):
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    fin = np.isfinite(x) & np.isfinite(y)
    e = np.zeros(x.shape)
    e[fin] = np.abs(x[fin] - y[fin]) / np.maximum(np.abs(y[fin]), scale if np.isscalar(scale) else scale[fin])
    return e


@contextlib.contextmanager
def _perturbed_conserved(ko, dlam, deta):
    """The oracle with lambda and eta moved by dlam, deta ulps (in every function that
    derives them from alpha, beta)."""
    orig = ko.conserved

    def conserved(a, th_o, alpha, beta, clamp=True):
        lam, eta = orig(a, th_o, alpha, beta, clamp)
        if dlam:
            lam = np.nextafter(lam, np.copysign(np.inf, dlam))
        if deta:
            eta = np.nextafter(eta, np.copysign(np.inf, deta))
        return lam, eta
    ko.conserved = conserved
    try:
        yield
    finally:
        ko.conserved = orig


def lambda_eta_sensitivity(a, r_o, th_o, alpha, beta, ngeo=None, tau=None):
    """Callable cols -> {t, r, th, ph, sig: (nsamp, ncols)}: the largest change of the
    oracle's output when lambda or eta of those rays moves by one ulp either way (the
    rounding every FP64 evaluation of lambda = -alpha sin(theta_o) and eta makes). With
    ngeo the Mino grid is re-derived from each perturbed tau_tot, as a trace does; with tau
    the Mino times are held. Perturbations that change a ray's radial class are skipped."""
    from oracle import kgeo_oracle as ko
    alpha = np.asarray(alpha, dtype=float)
    beta = np.asarray(beta, dtype=float)

    def run(cols):
        A, B = alpha[cols], beta[cols]
        if tau is None:
            o = ko.raytrace(a, r_o, th_o, A, B, ngeo)
            return dict(t=o['t'], r=o['r'], th=o['th'], ph=o['ph'], sig=o['affine_times']), o['rclass']
        sig, (t, r, th, ph) = ko.coords_at_tau(a, r_o, th_o, A, B, np.asarray(tau)[:, cols])
        rc = ko.quartic_roots(a, *ko.conserved(a, th_o, A, B))[4]
        return dict(t=t, r=r, th=th, ph=ph, sig=sig), rc

    def sens(cols):
        base, rc0 = run(cols)
        S = {k: np.zeros(v.shape) for k, v in base.items()}
        for dl, de in ((1, 0), (-1, 0), (0, 1), (0, -1)):
            with _perturbed_conserved(ko, dl, de):
                o, rc = run(cols)
            same = rc == rc0
            for k in S:
                d = np.abs(o[k] - base[k])
                d[~np.isfinite(d)] = 0.0
                d[:, ~same] = 0.0
                S[k] = np.maximum(S[k], d)
        return S
    return sens


def parity_ratios(got, ref, r_o, tol=TOL, rho=None, sens=None):
    """got / ref: dicts with t, r, th, ph, sig arrays (nsamp, npix); rho: optional (nsamp, npix)
    pole distances; sens: optional lambda_eta_sensitivity callable, consulted for the rays
    that exceed the other bars. Returns {output: (nsamp, npix) error / bar * tol}: a sample
    meets its bar where the value is <= tol. Non-finite samples count as 0."""
    bar = np.full(np.asarray(ref['r']).shape, float(tol))
    if rho is not None:
        bar = np.maximum(bar, 10 * EPS / np.maximum(np.asarray(rho, dtype=float), 1e-300))
    tscale = r_o if np.isfinite(r_o) else 1.0
    scales = (('r', 0.0), ('th', 1.0), ('ph', 1.0), ('t', tscale), ('sig', tscale))
    errs = {}
    for k, scale in scales:
        x, y = np.asarray(got[k], dtype=float), np.asarray(ref[k], dtype=float)
        sc = np.maximum(np.abs(np.where(np.isfinite(y), y, 0.0)), scale if scale > 0 else 1e-300)
        fin = np.isfinite(x) & np.isfinite(y)
        errs[k] = (np.where(fin, np.abs(x - y), 0.0), sc)
    ratio = {k: e / (bar * sc) * tol for k, (e, sc) in errs.items()}
    bad = np.zeros(bar.shape[1], dtype=bool)
    for k in ratio:
        bad |= (ratio[k] > tol).any(axis=0)
    if sens is not None and bad.any():
        cols = np.nonzero(bad)[0]
        S = sens(cols)
        for k, (e, sc) in errs.items():
            allow = np.maximum(bar[:, cols] * sc[:, cols], SENS_FACTOR * S[k])
            ratio[k][:, cols] = e[:, cols] / allow * tol
    return ratio
