"""CPU checks of the lensed-curve library (rho_of_req) and the critical curve: the oracle
against the reference's fixtures (bit-equal), and the curve kernel's Brent solve (the device
headers built for the host) against the same fixtures.

Bar for the roots: |rho - rho_ref| <= 1e-8 rho, and rho a root of the oracle's objective to
1e-8 (the objective takes both signs on [rho (1 - 1e-8), rho (1 + 1e-8)]). The curves of
r_eq = r_h are the edges of the m-th image where the crossing count Nmax steps: there the
objective jumps between r_s - r_h ~ +1e-8 and 1 - r_h, and inside a band of a few 1e-9 in
rho the floor() that decides Nmax flips back and forth with the rounding of its argument
(measured for a = 0.6, 130 deg, m = 1), so every point of the band is a root of the
reference's own objective and the reference's brentq returns one of them; elsewhere the roots
agree to ~1e-11."""
import warnings

import numpy as np

import hmlib
from oracle import kgeo_oracle as ko

DEG = np.pi / 180


def curve_cases(g):
    for i in range(int(g['ncase'])):
        a, inc, req, m = g['case%d' % i]
        yield i, float(a), float(inc) * DEG, float(req), int(m)


def is_root(a, th0, req, m, varphi, rho, rel=1e-8, n=21):
    """The oracle's objective takes both signs (or vanishes) on [rho (1 - rel), rho (1 + rel)]:
    the two ends first, then n points across (the Nmax band of the r_h curves)."""
    d = rel * max(abs(rho), 1.0)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        f = lambda x: ko.r_equatorial2(x, varphi, a, th0, mbar=m) - req  # noqa: E731
        f0, f1 = f(rho - d), f(rho + d)
        if f0 * f1 <= 0:
            return True
        vals = [f(x) for x in np.linspace(rho - d, rho + d, n)]
    return min(vals) <= 0 <= max(vals)


def check_roots(rho, g, i, a, th0, req, m, vp):
    ref = g['rho%d' % i]
    assert np.all(np.abs(rho - ref) <= 1e-8 * np.abs(ref)), (i, np.max(np.abs(rho - ref) / np.abs(ref)))
    for j in range(len(vp)):
        assert is_root(a, th0, req, m, vp[j], rho[j]), (i, j)


def test_oracle_rho_of_req(golden):
    g = golden('curves')
    vp = g['varphi']
    for i, a, th0, req, m in curve_cases(g):
        if 'error%d' % i in g:
            try:
                ko.rho_of_req(a, th0, req, mbar=m, varphis=vp)
                raise AssertionError('no error for case %d' % i)
            except ValueError as e:
                assert str(e) == str(g['error%d' % i])
            continue
        rho = ko.rho_of_req(a, th0, req, mbar=m, varphis=vp)[1]
        assert np.array_equal(rho, g['rho%d' % i]), i


def test_host_curve_solver(golden):
    """The curve kernel's Brent solve and objective (host build) against rho_of_req of the reference."""
    g = golden('curves')
    vp = g['varphi']
    for i, a, th0, req, m in curve_cases(g):
        rho, st = hmlib.curve_rho(a, th0, req, m, vp, ko.rho_bracket(m, req))
        if 'error%d' % i in g:
            assert np.all(st == 1) and np.all(np.isnan(rho)), i
            continue
        assert np.all(st == 0), i
        check_roots(rho, g, i, a, th0, req, m, vp)


def test_host_curve_solver_library_file(golden):
    """A make_curves2 table (360 angles, orders 0..2, r_eq = 10, a = 0.5, 30 deg)."""
    g = golden('curves')
    tab = g['library_a50_i30_r10']
    vp = tab[:, 0]
    for m in range(3):
        rho, st = hmlib.curve_rho(0.5, 30 * DEG, 10.0, m, vp, ko.rho_bracket(m, 10.0))
        assert np.all(st == 0)
        assert np.all(np.abs(rho - tab[:, m + 1]) <= 1e-8 * np.abs(tab[:, m + 1])), m


def test_oracle_critical_curve(golden):
    g = golden('curves')
    for i in range(4):
        a, th0, n = g['crit%d' % i]
        al, be = ko.critical_curve(a, th0, int(n))
        assert np.array_equal(al, g['crit_alpha%d' % i]) and np.array_equal(be, g['crit_beta%d' % i]), i
