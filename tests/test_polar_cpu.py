"""CPU checks of the polarised equatorial image: the oracle and the image kernel's
arithmetic (the device headers built for the host) against the reference's lab-frame
B-fields and polarised make_image fixtures, the oracle against the ipole EVPA profiles of
the reference's tests/test_images.py (same masks and tolerances), and the kernel's
Lambert W and dilogarithm against scipy.

Tolerances: I, Q and U are compared relative to I (|Q|, |U| <= I). I carries
sin(theta_B)^(1 + specind), whose relative error grows as 1/sin(theta_B) where the photon runs
along the field, so the kernel's bar is 1e-9 (elementwise) rather than the unpolarised 1e-10.
'bz_monopole' differs from the reference by its f(r): closed form here, a linearly
interpolated table there (Br to ~1e-8, Bth = O(cos(pi/2)) ~ 1e-17 Br), bar 5e-8."""
import warnings

import numpy as np
import scipy.special as sp

import hmlib
from oracle import kgeo_oracle as ko

DEG = np.pi / 180
IPOLE = {  # (a, inclination, fac_subkep, beta_r, beta_phi, n0 limits, n1 limits, rtol n0_a, n0_b, n1_a, n1_b)
    'lowspin_keplerian': (0.01, 0.1, 1.0, 1.0, 1.0, [-10, -3, 3, 10, -10, -3, 3, 6],
                          [-6.05, -5.25, 5.25, 6, -6, -5.1, 5.1, 6], (1e-2, 4e-2, 1e-2, 1e-2)),
    'midspin_inclined_keplerian': (0.42, 60., 1.0, 1.0, 1.0, [-10, -4.3125, 5., 10., -10, -1.2, 4.2, 10],
                                   [-5.3, -4.4, 5.7, 6.8, -10, -5, 5.1, 5.4], (1e-2, 3e-2, 1e-2, 1e-2)),
    'midspin_inclined_subkep': (0.7, 45., 0.6, 0.7, 0.8, [-10, -2.7, 4, 10, -10, -1.8, 3.8, 10],
                                [-5., -4, 5.8, 7., -8, -4.7, 5., 5.3], (1e-2, 2e-2, 1e-2, 1e-2)),
}
NX = 800


def rel(x, ref, floor=1e-300):
    d = np.abs(x - ref) / np.maximum(np.abs(ref), floor)
    return np.nanmax(d) if np.isfinite(d).any() else 0.0


def pol_cases(g):
    for i in range(int(g['ncase'])):
        a, th, r_o, mm, et, ek, vt, vk, bt, bk, plen, spec = eval(str(g['case%d' % i]), {'inf': np.inf})
        yield i, a, r_o, th * DEG, mm, (et, ek), (vt, vk), (bt, bk), plen, spec


def check_image(out, g, i, plen, tol, sbtol, names):
    """out: dict with I, Q, U, g, sinthb[, lp, Ie] under the names given by ``names``."""
    I = g['I%d' % i]
    for k in ('I', 'Q', 'U', 'g', 'sinthb'):
        assert np.array_equal(np.isnan(out[names[k]]), np.isnan(g['%s%d' % (k, i)])), (i, k)
    assert np.array_equal(out[names['I']] > 0, I > 0), i
    assert rel(out[names['I']], I) <= tol, (i, rel(out[names['I']], I))
    for k in ('Q', 'U'):
        e = np.nanmax(np.abs(out[names[k]] - g['%s%d' % (k, i)]) / np.maximum(I, 1e-300))
        assert e <= tol, (i, k, e)
    assert rel(out[names['g']], g['g%d' % i]) <= 1e-10, i
    assert np.nanmax(np.abs(out[names['sinthb']] - g['sinthb%d' % i])) <= sbtol, i
    if plen:
        assert rel(out[names['lp']], g['lp%d' % i]) <= tol, i
        assert rel(out[names['Ie']], g['Ie%d' % i]) <= tol, i


def test_oracle_bfield_lab(golden):
    g = golden('bfield_lab')
    for i in range(int(g['nmodel'])):
        bt, bk = eval(str(g['model%d' % i]))
        for j, a in enumerate(g['spins']):
            r, B = g['r_%d_%d' % (i, j)], g['B_%d_%d' % (i, j)]
            with warnings.catch_warnings():
                warnings.simplefilter('ignore')
                Bo = [np.broadcast_to(np.asarray(b, float), r.shape) for b in ko.bfield_lab(float(a), r, bt, bk)]
            if bt == 'bz_monopole':
                assert np.max(np.abs(Bo[0] - B[0])) <= 5e-8 * np.max(np.abs(B[0])), (i, j)
                assert np.max(np.abs(Bo[1] - B[1])) <= 1e-15 * np.max(np.abs(B[0])), (i, j)
                assert rel(Bo[2], B[2]) <= 1e-14, (i, j)
            else:
                for c in range(3):
                    assert rel(Bo[c], B[c]) <= 1e-15, (i, j, c, rel(Bo[c], B[c]))


def test_host_bfield_lab(golden):
    """The kernel's field models (host build) against Bfield.bfield_lab of the reference."""
    g = golden('bfield_lab')
    for i in range(int(g['nmodel'])):
        bt, bk = eval(str(g['model%d' % i]))
        for j, a in enumerate(g['spins']):
            r, B = g['r_%d_%d' % (i, j)], g['B_%d_%d' % (i, j)]
            H = hmlib.bfield(float(a), r, bt, bk)
            if bt == 'bz_monopole':
                assert np.max(np.abs(H[0] - B[0])) <= 5e-8 * np.max(np.abs(B[0])), (i, j)
                assert np.max(np.abs(H[1] - B[1])) <= 1e-15 * np.max(np.abs(B[0])), (i, j)
                assert rel(H[2], B[2]) <= 1e-13, (i, j)
            else:
                for c in range(3):
                    assert rel(H[c], B[c]) <= 1e-12, (i, j, c, rel(H[c], B[c]))


def test_oracle_image_pol(golden):
    g = golden('image_pol')
    for i, a, r_o, th_o, mm, emis, vel, bf, plen, spec in pol_cases(g):
        o = ko.make_image_px(a, r_o, th_o, mm, g['alpha'], g['beta'], emis=emis, vel=vel, specind=spec, bfield=bf,
                             polarization=True, pathlength=plen)
        tol = 5e-8 if bf[0] == 'bz_monopole' else 1e-14
        check_image(o, g, i, plen, tol, 5e-9 if bf[0] == 'bz_monopole' else 1e-14,
                    {k: k for k in ('I', 'Q', 'U', 'g', 'sinthb', 'lp', 'Ie')})
        for k in ('r', 't', 'n', 'np'):
            assert rel(o[k], g['%s%d' % (k, i)]) <= 1e-14, (i, k)


def test_host_image_pol(golden):
    """The polarised image kernel's arithmetic (host build) against make_image of the reference."""
    g = golden('image_pol')
    for i, a, r_o, th_o, mm, emis, vel, bf, plen, spec in pol_cases(g):
        mi, md = hmlib.model_arrays(emis, vel, specind=spec)
        h = hmlib.image_opts(a, r_o, th_o, g['alpha'], g['beta'], mm + 1, mi, md, bfield=bf, polarization=True,
                             pathlength=plen)
        tol = 5e-8 if bf[0] == 'bz_monopole' else 1e-9
        check_image(h, g, i, plen, tol, 5e-9 if bf[0] == 'bz_monopole' else 1e-10,
                    {k: k for k in ('I', 'Q', 'U', 'g', 'sinthb', 'lp', 'Ie')})


def test_pathlength_unpolarised(golden):
    g = golden('image_pol')
    emis, vel = ('bpl', {}), ('kep', {})
    o = ko.make_image_px(0.5, 1.e4, 60 * DEG, 1, g['alpha'], g['beta'], emis=emis, vel=vel, pathlength=True,
                         diskangle=0.2)
    mi, md = hmlib.model_arrays(emis, vel)
    h = hmlib.image_opts(0.5, 1.e4, 60 * DEG, g['alpha'], g['beta'], 2, mi, md, polarization=False, pathlength=True,
                         diskangle=0.2)
    for k in ('I', 'Q', 'U', 'g', 'sinthb', 'lp', 'Ie'):
        ref = g['%s_unpol' % k]
        assert rel(o[k], ref) <= 1e-14, k
        assert rel(h[k], ref) <= 1e-10, (k, rel(h[k], ref))


def evpa_kgeo(Q, U):
    """EVPA in degrees in the reference tests' convention (tests/test_images.py:8-17)."""
    e = 180. / np.pi * 0.5 * np.arctan2(U, Q) + 90.
    e[e > 90] -= 180.
    e[e > 90] -= 180.
    return e


def ipole_check(name, evpa_row, evpa_col, g):
    """The comparisons of tests/test_images.py: EVPA along the middle row (n?_a) and column
    (n?_b) of an 800 x 800 image against ipole, inside the given windows."""
    a, inc, fs, br, bp, l0, l1, tol = IPOLE[name]
    ploc, n0a, n0b, n1a, n1b = g[name]
    for o, (lim, ra, rb) in enumerate([(l0, n0a, n0b), (l1, n1a, n1b)]):
        ma = (ploc > lim[0]) & (ploc < lim[1])
        mb = (ploc > lim[2]) & (ploc < lim[3])
        assert ma.any() and mb.any()
        assert np.allclose(ra[ma], evpa_row[o][ma], rtol=tol[2 * o]), (name, o, 'row')
        assert np.allclose(rb[mb], evpa_col[o][mb], rtol=tol[2 * o + 1]), (name, o, 'col')


def test_oracle_ipole_evpa(golden):
    """The oracle reproduces the reference's ipole comparison on the two lines it checks."""
    g = golden('ipole_evpa')
    psize = 20. / NX
    side = np.linspace(-10., -10. + NX * psize, NX)  # make_image's grid
    A = np.concatenate([side, np.full(NX, side[NX // 2])])
    B = np.concatenate([np.full(NX, side[NX // 2]), side])
    for name, (a, inc, fs, br, bp, *_rest) in IPOLE.items():
        o = ko.make_image_px(a, np.inf, inc * DEG, 2, A, B, emis=('ring', {}),
                             vel=('general', {'fac_subkep': fs, 'beta_phi': bp, 'beta_r': br}), specind=1.,
                             bfield=('bz_guess', {'C': 1.}), polarization=True)
        e = [evpa_kgeo(o['Q'][:, k], o['U'][:, k]) for k in range(2)]
        ipole_check(name, [x[:NX] for x in e], [x[NX:] for x in e], g)


def test_host_special_functions():
    zs = np.concatenate([np.linspace(-1 / np.e, 0, 60)[1:-1], np.linspace(0, 1.4, 30)[1:]])
    for z in zs:
        w = np.real(sp.lambertw(z))
        assert abs(hmlib.lambert_w0(z) - w) <= 1e-14 * max(1.0, abs(w)) + 1e-8 * (z < -0.36), z
    for x in np.linspace(0.005, 2.0, 400):
        ref = np.real(sp.spence(1 - x + 0j))
        assert abs(hmlib.re_li2(x) - ref) <= 4e-15 * max(1.0, abs(ref)), x
    # BZ f(r): closed form of the host build against the oracle's (scipy.special.spence)
    r = np.linspace(1.02, 120., 500)
    f, fp = ko.bz_f(r)
    mi = hmlib.bfield(0.5, r, 'bz_monopole', {'C': 1})
    a2 = 0.25
    fr_h = (1.0 - mi[0] * (r * r + a2 * np.cos(np.pi / 2) ** 2)) / a2  # Br = C (1 - a^2 f) / Sigma
    # both closed forms cancel O(r^3) terms down to f ~ 1/(4r): ~1e-8 relative near r = 100
    assert np.max(np.abs(fr_h - f) / np.abs(f)) <= 5e-8
    assert np.max((np.abs(fr_h - f) / np.abs(f))[r < 10]) <= 1e-12
