"""The oracle's getstokes of the monopole field-line model against the reference's own outputs
(tests/golden/jet_stokes.npz, made by tests/golden/make_golden.py from kgeo/off_eq.py:124-233).

Bars: I, Q, U within 1e-10 of the image maximum; the EVPA within 1e-7 rad (mod pi) where the
polarised flux is above 1e-6 of the maximum (the angle of a vanishing Q + iU is undefined);
the crossing radii and angles within 1e-12.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import kgeo_oracle as ko  # noqa: E402

GOLD = np.load(os.path.join(HERE, 'golden', 'jet_stokes.npz'), allow_pickle=False)
CASES = range(int(GOLD['ncase']))
DEG = np.pi / 180


def stokes_bars(I, Q, U, ev, ref):
    Ir, Qr, Ur, er = ref
    scale = np.max(np.abs(Ir))
    assert scale > 0
    for x, y in ((I, Ir), (Q, Qr), (U, Ur)):
        assert np.max(np.abs(x - y)) <= 1e-10 * scale
    pol = np.hypot(Qr, Ur) > 1e-6 * scale
    d = np.abs(((ev - er) + np.pi / 2) % np.pi - np.pi / 2)
    assert np.max(d[pol], initial=0.0) <= 1e-7


@pytest.mark.parametrize('i', CASES)
def test_oracle_getstokes_vs_reference(i):
    model, psit, a, inc, pval, nu, neqmax, sigma = eval(str(GOLD['case%d' % i]))
    x = np.linspace(-8, 8, 16)
    A, B = np.meshgrid(x, x)
    with np.errstate(all='ignore'):
        I, Q, U, ev, r, th = ko.getstokes_mono(psit, A, B, 1.e4, inc * DEG, a, 200, neqmax=neqmax, model=model,
                                               pval=pval, nu_parallel=nu, sigma=sigma, table=True)
    g = lambda k: GOLD['%s%d' % (k, i)]  # noqa: E731
    assert I.shape == g('I').shape
    stokes_bars(I, Q, U, ev, (g('I'), g('Q'), g('U'), g('evpa')))
    assert np.max(np.abs(r - g('r'))) <= 1e-12
    assert np.max(np.abs(th - g('th'))) <= 1e-12


def test_stagnation_radius_is_largest_real_root():
    """r0min_mono keeps numpy's sorted root 4 of the quintic (kgeo/ff_boost.py:7-18): the
    largest real part, which the CUDA path finds by Aberth iteration."""
    for th, a in ((0.3, 0.5), (1.1, 0.9), (0.05, 0.2)):
        om = ko.omega_field(a, 10., th, 'bz_monopole', {})
        r0 = ko.r0min_mono(th, om, a)
        c = np.cos(th)
        s = np.sin(th)
        k = 2 - a * om + a * om * np.cos(2 * th)
        coef = [-a ** 2 / 2 * c ** 2 * k ** 2, -2 * a ** 4 * om ** 2 * c ** 4 * s ** 2, k ** 2 / 2,
                -a ** 2 * om ** 2 * np.sin(2 * th) ** 2, 0.0, -2 * om ** 2 * s ** 2]
        roots = np.roots(coef[::-1])
        assert abs(r0 - np.max(roots.real)) <= 1e-9 * abs(r0)


def test_host_stagnation_matches_numpy_roots():
    """The kernel's Aberth solve of the stagnation quintic (host build) against the oracle's
    numpy root 4, and its refusal of a = 0 (the reference's root 4 does not exist there)."""
    import hmlib
    for th in (0.05, 0.3, 0.7, 1.2, 1.5, 2.0, 3.0):
        for a in (0.1, 0.5, 0.94, -0.6):
            st, r0, om = hmlib.jet_stagnation(a, th)
            thn = np.arccos(np.abs(np.cos(th)))
            om_ref = ko.omega_field(a, 10., thn, 'bz_monopole', {})
            assert st == 0
            assert abs(om - om_ref) <= 1e-15
            assert abs(r0 - ko.r0min_mono(th, om_ref, a)) <= 1e-11 * abs(r0)
    assert hmlib.jet_stagnation(0.0, 0.5)[0] == 2


@pytest.mark.parametrize('i', CASES)
def test_host_emission_matches_oracle(i):
    """Per-crossing (I, Q, U) of the emission kernel (host build, same source as the CUDA
    kernel) against the oracle's Iobs_off at the reference's crossings."""
    import hmlib
    model, psit, a, inc, pval, nu, neqmax, sigma = eval(str(GOLD['case%d' % i]))
    x = np.linspace(-8, 8, 16)
    A, B = np.meshgrid(x, x)
    A, B = A.flatten(), B.flatten()
    th_o = inc * DEG
    geo = ko.raytrace(a, 1.e4, th_o, A, B, 200)
    tau, rv, tv, spr, spt, neq, shape = ko.findroot(geo, psit, A, B, 1.e4, th_o, a, 200, model=model, neqmax=neqmax,
                                                    pval=pval)
    At, Bt = np.tile(A, shape[0]), np.tile(B, shape[0])
    r0, _ = ko.jet_stagnation(rv, tv, shape, a)
    with np.errstate(all='ignore'):
        dv = ko.density_mono_all(rv, tv, shape, a, nu, sigma, table=True)
        field = ('bz_monopole', {'C': 1, 'table': True}) if model == 'mono' else ('power', {'p': pval})
        Io, Qo, Uo = ko.iobs_off(a, 1.e4, rv, th_o, At, Bt, spr, spt, field, nu, tv, dv)
    Io, Qo, Uo = (np.nan_to_num(np.where(rv == 0, 0, v)) for v in (Io, Qo, Uo))
    Ih, Qh, Uh = hmlib.jet_stokes(a, 1.e4, th_o, 0 if model == 'mono' else 1, nu, sigma, r0, 1.0, At, Bt, rv, tv,
                                  spr, spt)
    scale = np.max(np.abs(Io))
    for h, o in ((Ih, Io), (Qh, Qo), (Uh, Uo)):
        assert np.max(np.abs(h - o)) <= 1e-10 * scale


def test_dropin_argument_handling_before_any_launch():
    """off_eq.getstokes refuses what the GPU path does not cover, and raises the reference's
    errors, before touching the GPU."""
    from kgeo_gb300 import off_eq
    x = np.linspace(-8, 8, 4)
    A, B = np.meshgrid(x, x)
    for kw in (dict(model='para'), dict(model='power', pval=0.5), dict(model='mono', gammamax=3.0),
               dict(model='mono', retsin=True), dict(model='mono', nu_parallel='FF')):
        with pytest.raises(NotImplementedError):
            off_eq.getstokes(0.4, A, B, 1.e4, 1.0, 0.5, 50, **kw)
    with pytest.raises(Exception, match=r"nu_parallel should be in the range \(-1,1\)"):
        off_eq.getstokes(0.4, A, B, 1.e4, 1.0, 0.5, 50, model='mono', nu_parallel=1.5)
    with pytest.raises(IndexError):
        off_eq._stagnation_error(1)
    with pytest.raises(np.linalg.LinAlgError):
        off_eq._stagnation_error(2)
    off_eq._stagnation_error(0)


@pytest.mark.parametrize('model,a,nu,sigma', [('mono', 0.5, 0.0, 2.0), ('mono', 0.9, -0.4, 0.5), ('mono', 0.2, 0.7, 0.0),
                                              ('power', 0.6, 0.3, 1.0)])
def test_host_emission_random_crossings(model, a, nu, sigma):
    """The emission kernel (host build) against the oracle's Iobs_off on seeded random crossings
    over both hemispheres, from just outside the horizon to r = 300, near the axis included.
    Bar: 1e-10 of the sample's largest |I|. Per crossing the two agree to ~1e-12 at small r but
    not at large r: there f'(r) is the difference of neighbouring table nodes 1e-3 apart, whose
    values carry the rounding of a closed form that cancels terms of size r^3 down to 1/(4r)
    (the reference's table does the same), so B^theta and the emission of a crossing at
    r ~ 100 hold only a few digits; their share of the image is small."""
    import hmlib
    rng = np.random.default_rng(7)
    n = 3000
    rh = 1 + np.sqrt(1 - a * a)
    r = np.exp(rng.uniform(np.log(rh * 1.001), np.log(300.), n))
    th = rng.uniform(0.005, np.pi - 0.005, n)
    th[:50] = rng.uniform(1e-4, 1e-2, 50)
    alpha, beta = rng.uniform(-12, 12, (2, n))
    kr, kth = rng.choice([-1.0, 1.0], (2, n))
    th_o = 1.1
    shape = (1, n)
    r0, _ = ko.jet_stagnation(r, th, shape, a)
    with np.errstate(all='ignore'):
        dv = ko.density_mono_all(r, th, shape, a, nu, sigma, table=True)
        field = ('bz_monopole', {'C': 1, 'table': True}) if model == 'mono' else ('power', {'p': 0})
        Io, Qo, Uo = ko.iobs_off(a, 1.e4, r, th_o, alpha, beta, kr, kth, field, nu, th, dv)
    Io, Qo, Uo = (np.real(np.nan_to_num(v)) for v in (Io, Qo, Uo))
    Ih, Qh, Uh = hmlib.jet_stokes(a, 1.e4, th_o, 0 if model == 'mono' else 1, nu, sigma, r0, 1.0, alpha, beta, r, th,
                                  kr, kth)
    scale = np.max(np.abs(Io))
    assert scale > 0
    for h, o in ((Ih, Io), (Qh, Qo), (Uh, Uo)):
        assert np.max(np.abs(h - o)) <= 1e-10 * scale, np.max(np.abs(h - o)) / scale
        assert np.all(h[Io == 0] == 0)
