"""CPU oracle for the analytic Kerr null-geodesic tracer (FP64, numpy + scipy.special).

TEST INFRASTRUCTURE ONLY. The oracle is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of ``bench.py``
import it. The product package ``kgeo_gb300`` never imports, calls or links it.

It restates, operation for operation, the FP64 algorithm of kgeo (achael/kgeo)
for the hot path: conserved quantities, angular turning points, the radial
quartic, the Mino-time totals, the theta and r antiderivatives, the elliptic-Pi
adapter, the equatorial source radius and the unpolarised equatorial image.
Each function cites the reference file:line it follows. The elementary special
functions are scipy.special's (``ellipkinc``, ``ellipeinc``, ``ellipj``,
``ellipk``, ``elliprf``, ``elliprj``, ``elliprc``), called exactly where the
reference calls them, so on the same platform the oracle reproduces the
reference's output bit for bit. ``tests/golden/`` holds fixtures produced by
running the reference itself (``tests/golden/make_golden.py``); the CPU test
``tests/test_oracle_golden.py`` pins the oracle to them.

scipy.special (third-party, compiled) is the arithmetic the reference relies
on; it is called, never restated here.
"""
import numpy as np
import scipy.special as sp

MINSPIN = 1.0e-4          # kgeo/kerr_raytracing_utils.py:9
EP = 1.0e-12              # kgeo/kerr_raytracing_utils.py:12
MAXTAUFRAC = 1.0 - 1.0e-10  # kgeo/kerr_raytracing_ana.py:26
HALFPI = 0.5 * np.pi

# ----------------------------------------------------------------------------
# argument checks (same messages as the reference)
# ----------------------------------------------------------------------------


def check_spin(a):
    """kgeo/kerr_raytracing_ana.py:59-60"""
    if not (isinstance(a, float) and (0 <= np.abs(a) < 1)):
        raise Exception("|a| should be a float in range [0,1)")


def check_observer(r_o, th_o):
    """kgeo/kerr_raytracing_ana.py:62-65"""
    if not (isinstance(r_o, float) and (r_o >= 100)):
        raise Exception("r_o should be a float > 100")
    if not (isinstance(th_o, float) and (0 < th_o < np.pi) and th_o != 0.5 * np.pi):
        raise Exception("th_o should be a float in range (0,pi/2) or (pi/2,pi)")


def as_pixels(alpha, beta):
    """kgeo/kerr_raytracing_ana.py:68-71"""
    if not isinstance(alpha, np.ndarray):
        alpha = np.array([alpha]).flatten()
    if not isinstance(beta, np.ndarray):
        beta = np.array([beta]).flatten()
    if len(alpha) != len(beta):
        raise Exception("alpha, beta are different lengths!")
    return alpha, beta


# ----------------------------------------------------------------------------
# per-pixel kinematics
# ----------------------------------------------------------------------------


def conserved(a, th_o, alpha, beta, clamp=True):
    """(lambda, eta) of each pixel; kgeo/kerr_raytracing_ana.py:76-82 (151-158).

    With ``clamp`` the a < MINSPIN rule that lifts eta < 0 to EP is applied.
    """
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    if clamp and np.abs(a) < MINSPIN and np.any(eta < 0):
        eta = eta.copy()
        eta[eta < 0] = EP
    return lam, eta


def beta_sign(beta):
    """+1 for beta >= 0, -1 otherwise; kgeo/kerr_raytracing_utils.py:857-864."""
    out = np.zeros(beta.shape)
    out[beta >= 0] = 1
    out[beta < 0] = -1
    return out


def u_roots(a, th_o, lam, eta):
    """u_+, u_-, u_+/u_-, a^2 u_- with the reference's clamps.

    kgeo/kerr_raytracing_utils.py:276-328. Below MINSPIN the reference binds
    u_- and u_+ to the same array, so every clamp applied to one applies to
    both; that aliasing is kept here on purpose.
    """
    c2 = np.cos(th_o) ** 2
    if np.abs(a) < MINSPIN:
        up = eta / (eta + lam * lam)
        um = up
    else:
        half = 0.5 * (1 - (eta + lam * lam) / (a * a))
        up = half + np.sqrt(half ** 2 + eta / (a * a))
        um = half - np.sqrt(half ** 2 + eta / (a * a))
    up[(c2 - up) > 0] = c2
    up[up ** 2 > 1] = 1
    um[(um == 0) * (eta < 0)] = EP
    um[(um == 0) * (eta >= 0)] = -EP
    vort = eta < 0
    lift = np.zeros(eta.shape, dtype=bool)
    lift[vort] = (c2 - um[vort]) < 0
    um[lift] = c2
    if np.abs(a) < MINSPIN:
        ratio = 0.0 * um
        a2um = -(eta + lam ** 2)
    else:
        ratio = up / um
        a2um = a ** 2 * um
    return up, um, ratio, a2um


def theta_turning(a, th_o, lam, eta):
    """(u_+, u_-, th_+, th_-, thclass); kgeo/kerr_raytracing_utils.py:242-274."""
    up, um, _, _ = u_roots(a, th_o, lam, eta)
    th_plus = np.arccos(-np.sqrt(up))
    th_minus = np.arccos(np.sqrt(up))
    th_plus[eta < 0] = np.arccos(np.sqrt(um[eta < 0]))
    thclass = np.zeros(lam.shape).astype(int)
    thclass[eta > 0] = 1
    thclass[eta < 0] = 2
    thclass[eta == 0] = 3
    return up, um, th_plus, th_minus, thclass


def cbrt_max_real(x):
    """Complex cube root with the largest real part; real inputs keep their sign.

    kgeo/kerr_raytracing_utils.py:828-855.
    """
    s = np.sign(x)
    r = np.abs(x)
    th = np.angle(x)
    out = np.empty(x.shape).astype(complex)
    real = np.imag(x) == 0
    out[real] = (s * np.cbrt(r))[real]
    if np.any(~real):
        c0 = np.cbrt(r) * np.exp(1j * th / 3.)
        c1 = np.cbrt(r) * np.exp(1j * th / 3. + 2j * np.pi / 3.)
        c2 = np.cbrt(r) * np.exp(1j * th / 3. - 2j * np.pi / 3.)
        x0, x1, x2 = np.real(c0), np.real(c1), np.real(c2)
        pick0 = ~real * (x0 > x1) * (x0 > x2)
        pick1 = ~real * (x1 > x0) * (x1 > x2)
        pick2 = ~real * (x2 > x0) * (x2 > x1)
        out[pick0] = c0[pick0]
        out[pick1] = c1[pick1]
        out[pick2] = c2[pick2]
    return out


def quartic_roots(a, lam, eta):
    """Radial roots r1..r4 (complex) and rclass; kgeo/kerr_raytracing_utils.py:330-380."""
    rplus = 1 + np.sqrt(1 - a ** 2)
    A = a ** 2 - eta - lam ** 2
    B = 2 * (eta + (lam - a) ** 2)
    C = -(a ** 2) * eta
    P = -(A ** 2) / 12. - C
    Q = (-A / 3.) * ((A ** 2) / 36. - C) - (B ** 2) / 8.
    disc = (4 * (P ** 3) + 27 * (Q ** 2)).astype(complex)
    wp3 = -0.5 * Q + np.sqrt(disc / 108.)
    wm3 = -0.5 * Q - np.sqrt(disc / 108.)
    xi0 = cbrt_max_real(wp3) + cbrt_max_real(wm3) - A / 3.
    z = np.sqrt(0.5 * xi0)
    w_lo = (-0.5 * A - z ** 2 + 0.25 * B / z).astype(complex)
    w_hi = (-0.5 * A - z ** 2 - 0.25 * B / z).astype(complex)
    r1 = -z - np.sqrt(w_lo)
    r2 = -z + np.sqrt(w_lo)
    r3 = z - np.sqrt(w_hi)
    r4 = z + np.sqrt(w_hi)
    rclass = np.zeros(r1.shape).astype(int)
    rclass[np.imag(r2) != 0] = 4
    rclass[(np.imag(r2) == 0) * (np.imag(r4) != 0)] = 3
    rclass[(np.imag(r2) == 0) * (np.imag(r4) == 0) * (np.real(r4) < rplus)] = 2
    rclass[(np.imag(r2) == 0) * (np.imag(r4) == 0) * (np.real(r4) > rplus)] = 1
    return r1, r2, r3, r4, rclass


def _case4_params(a, r_o, r2, r4):
    """Region-IV constants (GL19a B83-B88); kgeo/kerr_raytracing_utils.py:418-433."""
    a1 = np.imag(r4)
    b1 = np.real(r4)
    a2 = np.imag(r2)
    b2 = np.real(r2)
    CC = np.sqrt((a1 - a2) ** 2 + (b1 - b2) ** 2)
    DD = np.sqrt((a1 + a2) ** 2 + (b1 - b2) ** 2)
    k4 = (4 * CC * DD) / ((CC + DD) ** 2)
    g0 = np.sqrt((4 * a2 ** 2 - (CC - DD) ** 2) / ((CC + DD) ** 2 - 4 * a2 ** 2))
    return a1, b1, a2, b2, CC, DD, k4, g0


def _case3_params(r1, r2, r4):
    """Region-III constants (GL19a B55-B59); kgeo/kerr_raytracing_utils.py:451-466."""
    a1 = np.imag(r4)
    b1 = np.real(r4)
    rr1 = np.real(r1)
    rr2 = np.real(r2)
    rr21 = rr2 - rr1
    AA = np.sqrt(a1 ** 2 + (b1 - rr2) ** 2)
    BB = np.sqrt(a1 ** 2 + (b1 - rr1) ** 2)
    k3 = ((AA + BB) ** 2 - rr21 ** 2) / (4 * AA * BB)
    return a1, b1, rr1, rr2, rr21, AA, BB, k3


def mino_total(a, r_o, eta, r1, r2, r3, r4):
    """Total Mino time from the observer to the horizon or back out to infinity.

    kgeo/kerr_raytracing_utils.py:382-548 (regions IV, III, II, I).
    """
    rplus = 1 + np.sqrt(1 - a ** 2)
    rminus = 1 - np.sqrt(1 - a ** 2)
    out = np.zeros(r1.shape)

    m4 = np.imag(r1) != 0
    if np.any(m4):
        a1, b1, a2, b2, CC, DD, k4, g0 = _case4_params(a, r_o, r2[m4], r4[m4])
        x_hor = (rplus + b1) / a2
        x_obs = np.inf if r_o == np.inf else (r_o + b1) / a2
        pref = 2. / (CC + DD)
        i_hor = pref * sp.ellipkinc(np.arctan(x_hor) + np.arctan(g0), k4)
        i_obs = pref * sp.ellipkinc(np.arctan(x_obs) + np.arctan(g0), k4)
        out[m4] = i_obs - i_hor

    m3 = (np.imag(r3) != 0) * (~m4)
    if np.any(m3):
        a1, b1, rr1, rr2, rr21, AA, BB, k3 = _case3_params(r1[m3], r2[m3], r4[m3])
        rrp1 = rplus - rr1
        rrp2 = rplus - rr2
        x_hor = (AA * rrp1 - BB * rrp2) / (AA * rrp1 + BB * rrp2)
        if r_o == np.inf:
            x_obs = (AA - BB) / (AA + BB)
        else:
            x_obs = (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2))
        pref = 1. / np.sqrt(AA * BB)
        out[m3] = pref * sp.ellipkinc(np.arccos(x_obs), k3) - pref * sp.ellipkinc(np.arccos(x_hor), k3)

    m2 = (np.imag(r3) == 0.) * (r3 < rplus) * (~m3)
    if np.any(m2):
        rr1, rr2, rr3, rr4 = (np.real(r)[m2] for r in (r1, r2, r3, r4))
        rr31, rr32, rr41, rr42 = rr3 - rr1, rr3 - rr2, rr4 - rr1, rr4 - rr2
        k2 = (rr32 * rr41) / (rr31 * rr42)
        x_hor = np.sqrt((rr31 * (rplus - rr4)) / (rr41 * (rplus - rr3)))
        if r_o == np.inf:
            x_obs = np.sqrt(rr31 / rr41)
        else:
            x_obs = np.sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)))
        pref = 2. / np.sqrt(rr31 * rr42)
        out[m2] = pref * sp.ellipkinc(np.arcsin(x_obs), k2) - pref * sp.ellipkinc(np.arcsin(x_hor), k2)

    m1 = (np.imag(r3) == 0.) * (r3 > rplus) * (~m2)
    if np.any(m1):
        rr1, rr2, rr3, rr4 = (np.real(r)[m1] for r in (r1, r2, r3, r4))
        rr31, rr32, rr41, rr42 = rr3 - rr1, rr3 - rr2, rr4 - rr1, rr4 - rr2
        k2 = (rr32 * rr41) / (rr31 * rr42)
        if r_o == np.inf:
            x_obs = np.sqrt(rr31 / rr41)
        else:
            x_obs = np.sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)))
        pref = 2. / np.sqrt(rr31 * rr42)
        out[m1] = 2 * (pref * sp.ellipkinc(np.arcsin(x_obs), k2))
    return out


# ----------------------------------------------------------------------------
# elliptic Pi adapter
# ----------------------------------------------------------------------------


def ellip_pi(n, phi, m):
    """Pi(n; phi | m), Abramowitz & Stegun convention, any real phi.

    kgeo/scipy_ellip_binding.py:87-237: the special-case masks in their order
    (phi ~ 0, m -> -inf, y < 0, |phi| > pi/2 with m >= 1 or n == 1, rho == 0,
    n == inf), the periodic reductions for |phi| > pi and pi/2 < |phi| <= pi,
    then sin(phi) R_F + (n/3) sin^3(phi) R_J with the DLMF 19.20.14 transform
    for rho < 0.
    """
    n = np.atleast_1d(np.asarray(n, dtype=float))
    phi = np.atleast_1d(np.asarray(phi, dtype=float))
    m = np.atleast_1d(np.asarray(m, dtype=float))
    if n.ndim != phi.ndim:
        n = np.outer(np.ones(phi.shape[0]), n)
    if m.ndim != phi.ndim:
        m = np.outer(np.ones(phi.shape[0]), m)

    cphi = np.cos(phi)
    sphi = np.sin(phi)
    x = cphi ** 2
    y = 1. - m * sphi ** 2
    z = np.ones(x.shape)
    rho = 1. - n * sphi ** 2

    out = np.zeros(phi.shape)
    done = np.zeros(phi.shape).astype(bool)

    sel = np.abs(phi) <= 1.e-10
    out[sel] = phi[sel]
    done += sel
    sel = (m < -1.e14) * ~done
    out[sel] = 0.
    done += sel
    sel = (y < 0) * ~done
    out[sel] = np.nan
    done += sel
    sel = (np.abs(phi) > HALFPI) * (m >= 1) * ~done
    out[sel] = np.nan
    done += sel
    sel = (np.abs(phi) > HALFPI) * (n == 1) * ~done
    out[sel] = np.inf
    done += sel
    sel = (rho == 0) * ~done
    out[sel] = np.inf
    done += sel
    sel = np.isinf(n) * ~done
    out[sel] = 0
    done += sel

    sel = (np.abs(phi) > np.pi) * ~done
    if np.any(sel):
        s = np.sign(phi[sel])
        k = s * np.floor(np.abs(phi[sel]) / np.pi)
        rem = phi[sel] - k * np.pi
        out[sel] = 2 * k * ellip_pi(n[sel], HALFPI * np.ones(rem.shape), m[sel]) \
            + ellip_pi(n[sel], rem, m[sel])
    done += sel

    sel = (np.abs(phi) > HALFPI) * (np.abs(phi) <= np.pi) * ~done
    if np.any(sel):
        s = np.sign(phi[sel])
        rem = -phi[sel] + s * np.pi
        out[sel] = s * 2 * ellip_pi(n[sel], HALFPI * np.ones(rem.shape), m[sel]) \
            - ellip_pi(n[sel], rem, m[sel])
    done += sel

    sel = ~done
    if np.any(sel):
        xs, ys, zs, rs, ss, ns = x[sel], y[sel], z[sel], rho[sel], sphi[sel], n[sel]
        qs = -rs
        ps = (zs * (xs + ys + qs) - xs * ys) / (zs + qs)
        rf = sp.elliprf(xs, ys, zs)
        rj = np.zeros(xs.shape)
        pos = rs > 0
        if np.any(pos):
            rj[pos] = sp.elliprj(xs[pos], ys[pos], zs[pos], rs[pos])
        neg = ~pos
        if np.any(neg):
            rj0 = sp.elliprj(xs[neg], ys[neg], zs[neg], ps[neg])
            rc = sp.elliprc((xs * ys + ps * qs)[neg], (ps * qs)[neg])
            w = 3 * np.sqrt((xs * ys * zs)[neg] / (xs * ys + ps * qs)[neg])
            rj[neg] = ((ps - zs)[neg] * rj0 - 3 * rf[neg] + w * rc)
            rj[neg] = rj[neg] / (qs + zs)[neg]
        out[sel] = ss * rf + (ns / 3.) * (ss ** 3) * rj
    return out


# ----------------------------------------------------------------------------
# theta motion
# ----------------------------------------------------------------------------


def _am_beyond_quarter(snarg, kk):
    """sin(Phi) and Phi = am(snarg | kk) for kk < 0 via the m = kk/(kk-1) transform.

    kgeo/kerr_raytracing_ana.py:257-277 (and 333-352): sn from ellipj at
    snarg/sqrt(1-m), the amplitude as pi/2 - am(K(m) - x | m).
    """
    sin_amp = np.zeros(snarg.shape)
    amp = np.zeros(snarg.shape)
    small = np.abs(snarg) < EP
    sin_amp[small] = snarg[small]
    amp[small] = snarg[small]
    if np.any(~small):
        m = (kk / (kk - 1))
        m = np.outer(np.ones(snarg.shape[0]), m)[~small]
        sn, cn, dn, ph = sp.ellipj(snarg[~small] / np.sqrt(1 - m), m)
        sin_amp[~small] = np.sqrt(1 - m) * sn / dn
        amp[~small] = 0.5 * np.pi - sp.ellipj(sp.ellipk(m) - snarg[~small] / np.sqrt(1 - m), m)[3]
    return sin_amp, amp


def theta_solution(a, th_o, s_o, lam, eta, up, um, tau, do_phi_and_t=True):
    """theta(tau), G_phi(tau), G_t(tau); kgeo/kerr_raytracing_ana.py:195-365."""
    th_s = np.zeros(tau.shape)
    G_ph = np.zeros(tau.shape)
    G_t = np.zeros(tau.shape)

    # ordinary motion (eta >= 0), only when some eta > 0: :216-296
    if np.any(eta > 0.):
        sel = eta >= 0.
        u_p = up[sel]
        u_m = um[sel]
        s = s_o[sel]
        if np.abs(a) < MINSPIN:
            kk = np.zeros(eta.shape)[sel]
            a2um = -(eta + lam ** 2)[sel]
        else:
            kk = u_p / u_m
            a2um = a ** 2 * u_m
        pref = 1 / np.sqrt(-a2um)
        arg_o = np.arcsin(np.cos(th_o) / np.sqrt(u_p))
        F_o = sp.ellipkinc(arg_o, kk)
        Gth_o = -pref * F_o
        if do_phi_and_t:
            Gph_o = -pref * ellip_pi(u_p, arg_o, kk)
            zk = kk == 0
            Gt_o = np.zeros(kk.shape)
            if np.any(zk):
                Gt_o[zk] = 2 * u_p * pref * 0.125 * (-2 * arg_o + np.sin(2 * arg_o))[zk]
            if np.any(~zk):
                Gt_o[~zk] = 2 * u_p * pref * (sp.ellipeinc(arg_o, kk) - F_o)[~zk] / (2 * kk[~zk])
        snarg = (np.sqrt(-a2um) * (-tau[:, sel] + s * Gth_o)).astype(float)
        sin_amp, amp = _am_beyond_quarter(snarg, kk)
        th_s[:, sel] = (np.arccos(-s * np.sqrt(u_p) * sin_amp)).astype(float)
        if do_phi_and_t:
            G_ph[:, sel] = (pref * ellip_pi(u_p, amp, kk) - s * Gph_o).astype(float)
            zk = kk == 0
            gt = np.zeros(amp.shape)
            if np.any(zk):
                gt[:, zk] = -2 * u_p * pref * 0.125 * (-2 * amp + np.sin(2 * amp))[:, zk]
            if np.any(~zk):
                gt[:, ~zk] = -(2 * u_p * pref * (sp.ellipeinc(amp, kk) - sp.ellipkinc(amp, kk)))[:, ~zk] / (2 * kk[~zk])
            G_t[:, sel] = gt - s * Gt_o

    # vortical motion (eta < 0), entered whenever some eta <= 0: :298-363
    if np.any(eta <= 0.):
        if np.abs(a) < MINSPIN:
            raise Exception("below MINSPIN but there are eta<0 points in th_integrate!")
        sel = eta < 0.
        u_p = up[sel]
        u_m = um[sel]
        s = s_o[sel]
        ratio = u_p / u_m
        a2um = a ** 2 * u_m
        h = 1. if th_o <= np.pi / 2 else -1
        prefA = 1 / np.sqrt(a2um)
        prefB = prefA / (1. - u_m)
        prefC = np.sqrt(u_m / a ** 2)
        nu_o = np.arcsin(np.sqrt((np.cos(th_o) ** 2 - u_m) / (u_p - u_m)))
        kk = 1 - ratio
        upm = (u_p - u_m) / (1. - u_m)
        Gth_o = -h * prefA * sp.ellipkinc(nu_o, kk)
        if do_phi_and_t:
            Gph_o = -h * prefB * ellip_pi(upm, nu_o, kk)
            Gt_o = -h * prefC * sp.ellipeinc(nu_o, kk)
        snarg = (np.sqrt(a2um) * (-tau[:, sel] + s * Gth_o)).astype(float)
        sin_nu, nu = _am_beyond_quarter(snarg, kk)
        th_s[:, sel] = (np.arccos(h * np.sqrt(u_m + (u_p - u_m) * sin_nu ** 2))).astype(float)
        if do_phi_and_t:
            G_ph[:, sel] = (prefB * ellip_pi(upm, nu, kk) - s * Gph_o).astype(float)
            G_t[:, sel] = (prefC * sp.ellipeinc(nu, kk) - s * Gt_o).astype(float)
    return th_s, G_ph, G_t


# ----------------------------------------------------------------------------
# radial motion
# ----------------------------------------------------------------------------


def S1_S2(al, phi, j, ret_s2=True):
    """GL19a B92/B93 building blocks; kgeo/kerr_raytracing_ana.py:638-663."""
    al2 = al * al
    al2p1 = 1 + al2
    al2j = 1 - j + al2
    s2phi = np.sqrt(1. - j * (np.sin(phi)) ** 2)
    p2 = np.sqrt(al2p1 / al2j)
    f2 = 0.5 * p2 * np.log(np.abs(((1 - p2) * (1 + p2 * s2phi)) / ((1 + p2) * (1 - p2 * s2phi))))
    F = sp.ellipkinc(phi, j)
    S1 = (F + al2 * ellip_pi(al2p1, phi, j) - al * f2) / al2p1
    S2 = np.nan
    if ret_s2:
        E = sp.ellipeinc(phi, j)
        tanphi = np.tan(phi)
        S2a = (1 - j) * F + al2 * E + al2 * s2phi * (al - tanphi) / (1 + al * tanphi) - al2 * al
        S2a = -S2a / (al2p1 * al2j)
        S2b = S1 * (1. / al2p1 + (1 - j) / al2j)
        S2 = S2a + S2b
    return S1, S2


def R1_R2(al, phi, j, ret_r2=True):
    """GL19a B62/B65 building blocks; kgeo/kerr_raytracing_ana.py:666-683."""
    al2 = al ** 2
    s2phi = np.sqrt(1 - j * np.sin(phi) ** 2)
    p1 = np.sqrt((al2 - 1) / (j + (1 - j) * al2))
    f1 = 0.5 * p1 * np.log(np.abs((p1 * s2phi + np.sin(phi)) / (p1 * s2phi - np.sin(phi))))
    nn = al2 / (al2 - 1)
    R1 = (ellip_pi(nn, phi, j) - al * f1) / (1 - al2)
    R2 = np.nan
    if ret_r2:
        F = sp.ellipkinc(phi, j)
        E = sp.ellipeinc(phi, j)
        R2 = (F - (al2 / (j + (1 - j) * al2)) * (E - al * np.sin(phi) * s2phi / (1 + al * np.cos(phi)))) / (al2 - 1)
        R2 = R2 + (2 * j - nn) * R1 / (j + (1 - j) * al2)
    return R1, R2


def radial_solution(a, r_o, lam, eta, r1, r2, r3, r4, tau, do_phi_and_t=True):
    """r(tau), I_phi, I_t, I_sigma; kgeo/kerr_raytracing_ana.py:368-633."""
    rplus = 1 + np.sqrt(1 - a ** 2)
    rminus = 1 - np.sqrt(1 - a ** 2)
    r_s = np.zeros(tau.shape)
    I_p = np.zeros(tau.shape)
    I_m = np.zeros(tau.shape)
    I_1 = np.zeros(tau.shape)
    I_2 = np.zeros(tau.shape)
    s = 1

    # region IV: :404-471
    m4 = np.imag(r1) != 0
    if np.any(m4):
        t4 = tau[:, m4]
        a1, b1, a2, b2, CC, DD, k4, g0 = _case4_params(a, r_o, r2[m4], r4[m4])
        x_p = (rplus + b1) / a2
        x_m = (rminus + b1) / a2
        x_o = np.inf if r_o == np.inf else (r_o + b1) / a2
        gp = (g0 * x_p - 1.) / (g0 + x_p)
        gm = (g0 * x_m - 1.) / (g0 + x_m)
        aux = np.arctan(x_o) + np.arctan(g0)
        pref = 2. / (CC + DD)
        Ir_o = pref * sp.ellipkinc(aux, k4)
        X4 = (1. / pref) * (s * (-t4) + Ir_o)
        sn, cn, dn, am = sp.ellipj(X4, k4)
        sc = sn / cn
        r_s[:, m4] = -a2 * (g0 - sc) / (1 + g0 * sc) - b1
        if do_phi_and_t:
            S1a0, S2a0 = S1_S2(g0, am, k4, ret_s2=True)
            S1b0, S2b0 = S1_S2(g0, aux, k4, ret_s2=True)
            S1ap, _ = S1_S2(gp, am, k4, ret_s2=False)
            S1bp, _ = S1_S2(gp, aux, k4, ret_s2=False)
            S1am, _ = S1_S2(gm, am, k4, ret_s2=False)
            S1bm, _ = S1_S2(gm, aux, k4, ret_s2=False)
            aa0 = (a2 / g0) * (1 + g0 ** 2)
            Pi_1 = s * pref * aa0 * (S1a0 - S1b0)
            Pi_2 = s * pref * (aa0 ** 2) * (S2a0 - S2b0)
            Pi_p = s * pref * (1 + g0 ** 2) / (g0 ** 2 + g0 * x_p) * (S1ap - S1bp)
            Pi_m = s * pref * (1 + g0 ** 2) / (g0 ** 2 + g0 * x_m) * (S1am - S1bm)
            aa1 = (a2 / g0 - b1)
            I_1[:, m4] = aa1 * (-t4) - Pi_1
            I_2[:, m4] = (aa1 ** 2) * (-t4) - 2 * aa1 * Pi_1 + Pi_2
            I_p[:, m4] = g0 / (a2 - a2 * g0 * x_p) * (-t4 - Pi_p)
            I_m[:, m4] = g0 / (a2 - a2 * g0 * x_m) * (-t4 - Pi_m)

    # region III: :473-552
    m3 = (np.imag(r3) != 0) * (~m4)
    if np.any(m3):
        t3 = tau[:, m3]
        a1, b1, rr1, rr2, rr21, AA, BB, k3 = _case3_params(r1[m3], r2[m3], r4[m3])
        rrp1, rrp2 = rplus - rr1, rplus - rr2
        rrm1, rrm2 = rminus - rr1, rminus - rr2
        x_p = (AA * rrp1 - BB * rrp2) / (AA * rrp1 + BB * rrp2)
        x_m = (AA * rrm1 - BB * rrm2) / (AA * rrm1 + BB * rrm2)
        if r_o == np.inf:
            x_o = (AA - BB) / (AA + BB)
        else:
            x_o = (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2))
        alp = -1. / x_p
        alm = -1. / x_m
        al0 = (BB + AA) / (BB - AA)
        aux = np.arccos(x_o)
        pref = (1. / np.sqrt(AA * BB))
        Ir_o = pref * sp.ellipkinc(aux, k3)
        X3 = (1. / pref) * (-t3 + s * Ir_o)
        sn, cn, dn, am = sp.ellipj(X3, k3)
        r_s[:, m3] = ((BB * rr2 - AA * rr1) + (BB * rr2 + AA * rr1) * cn) / ((BB - AA) + (BB + AA) * cn)
        if do_phi_and_t:
            R1a0, R2a0 = R1_R2(al0, am, k3)
            R1b0, R2b0 = R1_R2(al0, aux, k3)
            R1ap, _ = R1_R2(alp, am, k3, ret_r2=False)
            R1bp, _ = R1_R2(alp, aux, k3, ret_r2=False)
            if np.abs(a) > MINSPIN:
                R1am, _ = R1_R2(alm, am, k3, ret_r2=False)
                R1bm, _ = R1_R2(alm, aux, k3, ret_r2=False)
            else:
                R1am = np.zeros(R1ap.shape)
                R1bm = np.zeros(R1ap.shape)
            c0 = (2 * rr21 * np.sqrt(AA * BB)) / (BB ** 2 - AA ** 2)
            Pi_1 = c0 * (R1a0 - s * R1b0)
            Pi_2 = c0 ** 2 * (R2a0 - s * R2b0)
            Pi_p = ((2 * rr21 * np.sqrt(AA * BB)) / (BB * rrp2 - AA * rrp1)) * (R1ap - s * R1bp)
            Pi_m = ((2 * rr21 * np.sqrt(AA * BB)) / (BB * rrm2 - AA * rrm1)) * (R1am - s * R1bm)
            pr = ((BB * rr2 + AA * rr1) / (BB + AA))
            I_1[:, m3] = pr * (-t3) + Pi_1
            I_2[:, m3] = pr ** 2 * (-t3) + 2 * pr * Pi_1 + np.sqrt(AA * BB) * Pi_2
            I_p[:, m3] = -((BB + AA) * (-t3) + Pi_p) / (BB * rrp2 + AA * rrp1)
            I_m[:, m3] = -((BB + AA) * (-t3) + Pi_m) / (BB * rrm2 + AA * rrm1)

    # regions II and I (all roots real): :554-624
    m2 = (np.imag(r3) == 0.) * (~m3)
    if np.any(m2):
        t2 = tau[:, m2]
        rr1, rr2, rr3, rr4 = (np.real(r)[m2] for r in (r1, r2, r3, r4))
        rr31, rr32, rr41, rr42, rr43 = rr3 - rr1, rr3 - rr2, rr4 - rr1, rr4 - rr2, rr4 - rr3
        rrp3, rrm3, rrp4, rrm4 = rplus - rr3, rminus - rr3, rplus - rr4, rminus - rr4
        k2 = (rr32 * rr41) / (rr31 * rr42)
        if r_o == np.inf:
            x_o = np.sqrt(rr31 / rr41)
        else:
            x_o = np.sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)))
        aux = np.arcsin(x_o)
        Ir_o = 2 * sp.ellipkinc(aux, k2) / np.sqrt(rr31 * rr42)
        X2 = 0.5 * np.sqrt(rr31 * rr42) * (-t2 + s * Ir_o)
        sn, cn, dn, am = sp.ellipj(X2, k2)
        rs = (rr4 * rr31 - rr3 * rr41 * (sn) ** 2) / (rr31 - rr41 * (sn) ** 2)
        r_s[:, m2] = rs
        if do_phi_and_t:
            dX = -0.5 * np.sqrt(rr31 * rr42)
            dsn2 = 2 * sn * cn * dn * dX
            drs = rr31 * rr43 * rr41 * dsn2 / ((rr31 - rr41 * sn ** 2) ** 2)
            drs *= -1
            Rpot_o = (r_o - rr1) * (r_o - rr2) * (r_o - rr3) * (r_o - rr4)
            drs_o = s * np.sqrt(Rpot_o)
            H = drs / (rs - rr3) - drs_o / (r_o - rr3)
            E = np.sqrt(rr31 * rr42) * (sp.ellipeinc(am, k2) - s * sp.ellipeinc(aux, k2))
            c2 = 2. / np.sqrt(rr31 * rr42)
            Pi_1 = c2 * (ellip_pi(rr41 / rr31, am, k2) - s * ellip_pi(rr41 / rr31, aux, k2))
            npl = (rrp3 * rr41) / (rrp4 * rr31)
            nmi = (rrm3 * rr41) / (rrm4 * rr31)
            Pi_p = c2 * (rr43 / (rrp3 * rrp4)) * (ellip_pi(npl, am, k2) - s * ellip_pi(npl, aux, k2))
            Pi_m = c2 * (rr43 / (rrm3 * rrm4)) * (ellip_pi(nmi, am, k2) - s * ellip_pi(nmi, aux, k2))
            I_1[:, m2] = rr3 * (-t2) + rr43 * Pi_1
            I_2[:, m2] = H - 0.5 * (rr1 * rr4 + rr2 * rr3) * (-t2) - E
            I_p[:, m2] = t2 / rrp3 - Pi_p
            I_m[:, m2] = t2 / rrm3 - Pi_m

    # combination, B1/B2: :626-633
    I_0 = -tau
    I_phi = (2 * a / (rplus - rminus)) * ((rplus - 0.5 * a * lam) * I_p - (rminus - 0.5 * a * lam) * I_m)
    I_tA = (4 / (rplus - rminus)) * ((rplus ** 2 - 0.5 * a * lam * rplus) * I_p - (rminus ** 2 - 0.5 * a * lam * rminus) * I_m)
    I_t = I_tA + 4 * I_0 + 2 * I_1 + I_2
    I_sig = I_2
    return r_s, I_phi, I_t, I_sig


# ----------------------------------------------------------------------------
# drivers
# ----------------------------------------------------------------------------


def coords_at_tau(a, r_o, th_o, alpha, beta, tau, do_phi_and_t=True):
    """(sigma, [t, r, theta, phi]) at Mino times tau; kgeo/kerr_raytracing_ana.py:126-193."""
    if tau.ndim == 1:
        tau = tau.reshape(1, tau.shape[0])
    lam, eta = conserved(a, th_o, alpha, beta)
    s_o = beta_sign(beta)
    up, um, _, _, _ = theta_turning(a, th_o, lam, eta)
    r1, r2, r3, r4, _ = quartic_roots(a, lam, eta)
    th_s, G_ph, G_t = theta_solution(a, th_o, s_o, lam, eta, up, um, tau, do_phi_and_t)
    r_s, I_ph, I_t, I_sig = radial_solution(a, r_o, lam, eta, r1, r2, r3, r4, tau, do_phi_and_t)
    sig = 0 + I_sig + a ** 2 * G_t
    t = 0 + I_t + a ** 2 * G_t
    ph = 0 + I_ph + lam * G_ph
    return sig, [t, r_s, th_s, ph]


def raytrace(a, r_o, th_o, alpha, beta, ngeo, maxtaufrac=MAXTAUFRAC):
    """Full-range analytic trace; kgeo/kerr_raytracing_ana.py:46-122.

    Returns a dict with mino_times (ngeo, npix), affine_times, t, r, th, ph
    and the per-ray classification (lam, eta, rclass, thclass, tau_tot).
    """
    check_spin(a)
    check_observer(r_o, th_o)
    alpha, beta = as_pixels(alpha, beta)
    lam, eta = conserved(a, th_o, alpha, beta)
    r1, r2, r3, r4, rclass = quartic_roots(a, lam, eta)
    tau_tot = mino_total(a, r_o, eta, r1, r2, r3, r4)
    tau = np.linspace(0, maxtaufrac * tau_tot, ngeo)
    sig, (t, r, th, ph) = coords_at_tau(a, r_o, th_o, alpha, beta, tau)
    _, _, _, _, thclass = theta_turning(a, th_o, lam, eta)
    return dict(mino_times=tau, affine_times=sig, t=t, r=r, th=th, ph=ph,
                lam=lam, eta=eta, rclass=rclass, thclass=thclass, tau_tot=tau_tot,
                roots=np.stack([r1, r2, r3, r4]))


def n_equatorial_crossings(a, th_o, alpha, beta, tau):
    """Fractional-floor count of equatorial crossings; kgeo/kerr_raytracing_utils.py:605-684."""
    one = tau.ndim == 1
    if one:
        tau = tau.reshape(1, tau.shape[0])
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    out = np.empty(tau.shape)
    vort = eta <= 0
    out[:, vort] = -2
    if np.any(~vort):
        up, um, ratio, a2um = u_roots(a, th_o, lam[~vort], eta[~vort])
        b = beta[~vort]
        tr = tau[:, ~vort]
        F0 = sp.ellipkinc(np.arcsin(np.cos(th_o) / np.sqrt(up)), ratio)
        K = sp.ellipkinc(0.5 * np.pi, ratio)
        res = np.empty(tr.shape)
        if th_o < (np.pi / 2.):
            lo = b <= 0
            res[:, lo] = (np.floor((tr * np.sqrt(-a2um) - F0) / (2 * K)))[:, lo]
            res[:, ~lo] = (np.floor((tr * np.sqrt(-a2um) + F0) / (2 * K)) - 1)[:, ~lo]
        else:
            hi = b >= 0
            res[:, hi] = (np.floor((tr * np.sqrt(-a2um) + F0) / (2 * K)))[:, hi]
            res[:, ~hi] = (np.floor((tr * np.sqrt(-a2um) - F0) / (2 * K)) - 1)[:, ~hi]
        out[:, ~vort] = res
    return out[0] if one else out


def n_poloidal_orbits(a, th_o, alpha, beta, tau):
    """Fractional number of poloidal orbits; kgeo/kerr_raytracing_utils.py:551-603."""
    one = tau.ndim == 1
    if one:
        tau = tau.reshape(1, tau.shape[0])
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    out = np.empty(tau.shape)
    vort = eta <= 0
    out[:, vort] = -2
    if np.any(~vort):
        up, um, ratio, a2um = u_roots(a, th_o, lam[~vort], eta[~vort])
        K = sp.ellipk(ratio)
        npol = (np.sqrt(-a2um.astype(complex)) * tau[:, ~vort]) / (4 * K)
        out[:, ~vort] = np.real(npol.astype(complex))
    return out[0] if one else out


def n_angular_turnings(a, th_o, alpha, beta, tau):
    """Fractional number of angular turnings; kgeo/kerr_raytracing_utils.py:686-792 (ordinary
    rays as the crossing counts, vortical rays by GL19b Eqs 56, 60 with the reference's
    provisional +1/2 for beta <= 0 counts above 1/2)."""
    one = tau.ndim == 1
    if one:
        tau = tau.reshape(1, tau.shape[0])
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    out = np.empty(tau.shape)
    vort = eta <= 0
    out[:, vort] = 0
    if np.any(~vort):
        up, um, ratio, a2um = u_roots(a, th_o, lam[~vort], eta[~vort])
        F0 = sp.ellipkinc(np.arcsin(np.cos(th_o) / np.sqrt(up)), ratio)
        K = sp.ellipkinc(0.5 * np.pi, ratio)
        b = beta[~vort]
        tr = tau[:, ~vort]
        res = np.empty(tr.shape)
        lo = b <= 0
        res[:, lo] = ((tr * np.sqrt(-a2um) - F0) / (2 * K))[:, lo] + 0.5
        res[:, ~lo] = ((tr * np.sqrt(-a2um) + F0) / (2 * K))[:, ~lo] + 0.5
        out[:, ~vort] = res
    if np.any(vort):
        up, um, ratio, a2um = u_roots(a, th_o, lam[vort], eta[vort])
        Nu = np.arcsin(np.sqrt((np.cos(th_o) ** 2 - um) / (up - um)))
        F0 = sp.ellipkinc(Nu, 1 - ratio)
        K = sp.ellipkinc(0.5 * np.pi, 1 - ratio)
        b = beta[vort]
        tv = tau[:, vort]
        res = np.empty(tv.shape)
        lo = b <= 0
        if np.any(lo):
            norbit = ((tv * np.sqrt(a2um) - F0) / (2 * K))[:, lo] + 0.5
            norbit[norbit > 0.5] += 0.5
            res[:, lo] = norbit
        if np.any(~lo):
            res[:, ~lo] = ((tv * np.sqrt(a2um) + F0) / (2 * K))[:, ~lo] + 0.5
        out[:, vort] = res
    return out[0] if one else out


def outside_critical(a, th_o, alpha, beta):
    """1 where real r4 > r_h and eta >= 0, else 0; kgeo/kerr_raytracing_utils.py:794-826."""
    rh = 1 + np.sqrt(1 - a ** 2)
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * (np.cos(th_o)) ** 2 + beta ** 2
    r1, r2, r3, r4, _ = quartic_roots(a, lam, eta)
    sel = (np.imag(r4) == 0) * (r4 > rh) * ~(eta < 0)
    out = np.empty(alpha.shape)
    out[sel] = 1
    out[~sel] = 0
    return out


# ----------------------------------------------------------------------------
# equatorial lensing
# ----------------------------------------------------------------------------


def r_equatorial(a, r_o, th_o, mbar, alpha, beta):
    """(r_s, Ir, Imax, Nmax) of the mbar-th equatorial crossing.

    kgeo/equatorial_lensing.py:85-196 (GL19b eq. 81 with the C8 typo fixed).
    """
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    r_s = np.empty(alpha.shape)
    Ir = np.empty(alpha.shape)
    Imax = np.empty(alpha.shape)
    Nmax = np.empty(alpha.shape)
    vort = eta <= 0
    r_s[vort] = -1
    Ir[vort] = -1
    Imax[vort] = -1
    Nmax[vort] = -2
    if np.any(~vort):
        lam_r = lam[~vort]
        eta_r = eta[~vort]
        b = beta[~vort]
        up, um, ratio, a2um = u_roots(a, th_o, lam_r, eta_r)
        F0 = sp.ellipkinc(np.arcsin(np.cos(th_o) / np.sqrt(up)), ratio)
        K = sp.ellipkinc(0.5 * np.pi, ratio)
        r1, r2, r3, r4, _ = quartic_roots(a, lam_r, eta_r)
        imax = mino_total(a, r_o, eta_r, r1, r2, r3, r4)
        nmax = np.empty(imax.shape)
        ir = np.empty(imax.shape)
        if th_o < (np.pi / 2.):
            m = mbar + np.heaviside(b, 0)
            lo = b <= 0
            nmax[lo] = (np.floor((imax * np.sqrt(-a2um) - F0) / (2 * K)))[lo]
            ir[lo] = ((2 * m * K + F0) / np.sqrt(-a2um))[lo]
            nmax[~lo] = (np.floor((imax * np.sqrt(-a2um) + F0) / (2 * K)) - 1)[~lo]
            ir[~lo] = ((2 * m * K - F0) / np.sqrt(-a2um))[~lo]
        else:
            m = mbar + np.heaviside(-b, 0)
            hi = b >= 0
            nmax[hi] = (np.floor((imax * np.sqrt(-a2um) + F0) / (2 * K)))[hi]
            ir[hi] = ((2 * m * K - F0) / np.sqrt(-a2um))[hi]
            nmax[~hi] = (np.floor((imax * np.sqrt(-a2um) - F0) / (2 * K)) - 1)[~hi]
            ir[~hi] = ((2 * m * K + F0) / np.sqrt(-a2um))[~hi]
        rs = radial_solution(a, r_o, lam_r, eta_r, r1, r2, r3, r4,
                             ir.reshape(1, len(ir)), do_phi_and_t=False)[0][0]
        rs[nmax < mbar] = 0
        r_s[~vort] = rs
        Ir[~vort] = ir
        Imax[~vort] = imax
        Nmax[~vort] = nmax
    return r_s, Ir, Imax, Nmax


# ----------------------------------------------------------------------------
# equatorial image: velocity and emissivity models (config-5 subset)
# ----------------------------------------------------------------------------


def r_isco(a, s=1):
    """ISCO radius; kgeo/velocities.py:300-302."""
    z1 = 1 + np.cbrt(1 - a ** 2) * (np.cbrt(1 + a) + np.cbrt(1 - a))
    z2 = np.sqrt(3 * a ** 2 + z1 ** 2)
    return 3 + z2 - s * np.sqrt((3 - z1) * (3 + z1 + 2 * z2))


def u_zamo(a, r):
    """Zero-angular-momentum observer at th = pi/2; kgeo/velocities.py:180-206."""
    th = np.pi / 2.
    Delta = r ** 2 - 2 * r + a ** 2
    Sigma = r ** 2 + a ** 2 * np.cos(th) ** 2
    g00 = -(1 - 2 * r / Sigma)
    g33 = (r ** 2 + a ** 2 + 2 * r * (a * np.sin(th)) ** 2 / Sigma) * np.sin(th) ** 2
    g03 = -2 * r * a * np.sin(th) ** 2 / Sigma
    v3 = -g03 / g33
    u0 = np.sqrt(-1. / (g00 + 2 * g03 * v3 + g33 * v3 * v3))
    return u0, 0 * r, 0, u0 * v3


def u_kep(a, r, retrograde=False):
    """Cunningham: Keplerian outside the ISCO, plunging inside; kgeo/velocities.py:229-281."""
    s = -1 if retrograde else 1
    ri = r_isco(a, s)
    u0 = np.zeros(r.shape)
    u1 = np.zeros(r.shape)
    u3 = np.zeros(r.shape)
    out = r >= ri
    spin = np.abs(a)
    asign = np.sign(a)
    if np.any(out):
        rr = r[out]
        Omega = asign * s / (rr ** 1.5 + s * spin)
        u0[out] = (rr ** 1.5 + s * spin) / np.sqrt(rr ** 3 - 3 * rr ** 2 + 2 * s * spin * rr ** 1.5)
        u3[out] = Omega * u0[out]
    if np.any(~out):
        rr = r[~out]
        Delta = (rr ** 2 - 2 * rr + a ** 2)
        ell_i = s * asign * (ri ** 2 + a ** 2 - s * 2 * spin * np.sqrt(ri)) / (ri ** 1.5 - 2 * np.sqrt(ri) + s * spin)
        gam_i = np.sqrt(1 - 2. / (3. * ri))
        H = (2 * rr - a * ell_i) / Delta
        u0[~out] = gam_i * (1 + (2 / rr) * (1 + H))
        u1[~out] = -np.sqrt(2. / (3 * ri)) * (ri / rr - 1) ** 1.5
        u3[~out] = gam_i * (ell_i + a * H) / (rr ** 2)
    return u0, u1, 0, u3


def u_infall(a, r):
    """Geodesic infall from rest at infinity; kgeo/velocities.py:211-226."""
    Delta = r ** 2 + a ** 2 - 2 * r
    Xi = (r ** 2 + a ** 2) ** 2 - Delta * a ** 2
    u0 = Xi / (r ** 2 * Delta)
    u1 = -np.sqrt(2 * r * (r ** 2 + a ** 2)) / (r ** 2)
    u3 = 2 * a / (r * Delta)
    return u0, u1, 0, u3


def u_subkep(a, r, fac_subkep=1, retrograde=False):
    """Sub-Keplerian outside the ISCO, conserved-quantity infall inside; kgeo/velocities.py:284-359."""
    s = -1 if retrograde else 1
    ri = r_isco(a, s)
    u0 = np.zeros(r.shape)
    u1 = np.zeros(r.shape)
    u3 = np.zeros(r.shape)
    out = r >= ri
    spin = np.abs(a)
    asign = np.sign(a)
    if np.any(out):
        rr = r[out]
        Delta = (rr ** 2 - 2 * rr + a ** 2)
        Xi = (rr ** 2 + a ** 2) ** 2 - Delta * a ** 2
        ell = asign * s * (rr ** 2 + spin ** 2 - s * 2 * spin * np.sqrt(rr)) / (rr ** 1.5 - 2 * np.sqrt(rr) + s * spin)
        ell *= fac_subkep
        gam = np.sqrt(Delta / (Xi / rr ** 2 - 4 * a * ell / rr - (1 - 2 / rr) * ell ** 2))
        H = (2 * rr - a * ell) / Delta
        chi = 1 / (1 + (2 / rr) * (1 + H))
        Omega = (chi / rr ** 2) * (ell + a * H)
        u0[out] = gam / chi
        u3[out] = (gam / chi) * Omega
    if np.any(~out):
        rr = r[~out]
        Delta = (rr ** 2 - 2 * rr + a ** 2)
        Xi = (rr ** 2 + a ** 2) ** 2 - Delta * a ** 2
        Delta_i = (ri ** 2 - 2 * ri + a ** 2)
        Xi_i = (ri ** 2 + a ** 2) ** 2 - Delta_i * a ** 2
        ell_i = asign * s * (ri ** 2 + spin ** 2 - s * 2 * spin * np.sqrt(ri)) / (ri ** 1.5 - 2 * np.sqrt(ri) + s * spin)
        ell_i *= fac_subkep
        gam_i = np.sqrt(Delta_i / (Xi_i / ri ** 2 - 4 * a * ell_i / ri - (1 - 2 / ri) * ell_i ** 2))
        H = (2 * rr - a * ell_i) / Delta
        chi = 1 / (1 + (2 / rr) * (1 + H))
        Omega = (chi / rr ** 2) * (ell_i + a * H)
        nu = (rr / Delta) * np.sqrt(Xi / rr ** 2 - 4 * a * ell_i / rr - (1 - 2 / rr) * ell_i ** 2 - Delta / gam_i ** 2)
        u0[~out] = gam_i / chi
        u1[~out] = -gam_i * (Delta / rr ** 2) * nu
        u3[~out] = (gam_i / chi) * Omega
    return u0, u1, 0, u3


def u_general(a, r, fac_subkep=1, beta_phi=1, beta_r=1, retrograde=False):
    """Infall / sub-Keplerian mix (AART); kgeo/velocities.py:442-470."""
    Delta = r ** 2 + a ** 2 - 2 * r
    u0i, u1i, _, u3i = u_infall(a, r)
    Om_i = u3i / u0i
    u0s, u1s, _, u3s = u_subkep(a, r, retrograde=retrograde, fac_subkep=fac_subkep)
    Om_s = u3s / u0s
    u1 = u1s + (1 - beta_r) * (u1i - u1s)
    Omega = Om_s + (1 - beta_phi) * (Om_i - Om_s)
    u0 = np.sqrt(1 + (r ** 2) * (u1 ** 2) / Delta)
    u0 /= np.sqrt(1 - (r ** 2 + a ** 2) * Omega ** 2 - (2 / r) * (1 - a * Omega) ** 2)
    u3 = u0 * Omega
    return u0, u1, 0, u3


def emis_bpl(a, r, p1=-2.0, p2=-0.5):
    """Broken power law; kgeo/emissivities.py:121-127."""
    rh = 1 + np.sqrt(1 - a ** 2)
    return np.exp(p1 * np.log(r / rh) + p2 * np.log(r / rh) ** 2)


def emis_glm(a, r, gamma_off=-1.5, sigma=0.5, mu_ring=False):
    """GLM / ring profile; kgeo/emissivities.py:130-139."""
    mu = mu_ring if mu_ring else 1 - np.sqrt(1 - a ** 2)
    return np.exp(-0.5 * (gamma_off + np.arcsinh((r - mu) / sigma)) ** 2) / np.sqrt((r - mu) ** 2 + sigma ** 2)


def velocity(a, r, veltype, kw):
    """Velocity(veltype, **kw).u_lab(a, r) for the supported models; kgeo/velocities.py:69-95."""
    retro = kw.get('retrograde', False)
    if veltype == 'zamo':
        return u_zamo(a, r)
    if veltype == 'infall':
        return u_infall(a, r)
    if veltype in ('kep', 'cunningham'):
        return u_kep(a, r, retrograde=retro)
    if veltype in ('subkep', 'cunningham_subkep'):
        return u_subkep(a, r, fac_subkep=kw.get('fac_subkep', 1), retrograde=retro)
    if veltype == 'general':
        return u_general(a, r, fac_subkep=kw.get('fac_subkep', 1), beta_phi=kw.get('beta_phi', 1),
                         beta_r=kw.get('beta_r', 1), retrograde=retro)
    raise ValueError(veltype)


def emissivity(a, r, emistype, kw):
    """Emissivity(emistype, **kw).jrest(a, r) without the spectral factors; kgeo/emissivities.py:38-127."""
    if emistype == 'constant':
        return np.ones(r.shape)
    if emistype == 'bpl':
        return emis_bpl(a, r, p1=kw.get('p1', -2.0), p2=kw.get('p2', -0.5))
    if emistype == 'glm':
        return emis_glm(a, r, gamma_off=kw.get('gamma_off', -1.5), sigma=kw.get('sigma', 0.5), mu_ring=False)
    if emistype == 'ring':
        return emis_glm(a, r, gamma_off=kw.get('gamma_off', 0), sigma=kw.get('sigma', 0.3),
                        mu_ring=kw.get('r_ring', 4.5))
    raise ValueError(emistype)


# ----------------------------------------------------------------------------
# polarised equatorial image: lab-frame B-field models, comoving tetrads,
# calc_polquantities, calc_evpa, calc_pathlength_equatorial
# ----------------------------------------------------------------------------


BZ_TABLE_N = 100000   # nodes of the reference's f(r) table generator (kgeo/bfields.py:16-20)


def bz_f_table(r):
    """f(r), f'(r) as the reference evaluates them: the linear interpolant of f on
    linspace(1, 100, 100000) (UnivariateSpline(k=1, s=0)) and its piecewise-constant slope
    (kgeo/bfields.py:23-31), with 1/(4r), -1/(4r^2) beyond r = 100. The node values here are the
    closed form of bz_f."""
    r = np.asarray(r, dtype=float)
    nodes = np.linspace(1, 100, BZ_TABLE_N)
    fn = bz_f(nodes)[0]
    f = np.interp(r, nodes, fn)
    k = np.clip(np.floor((r - 1.) / (nodes[1] - nodes[0])).astype(np.int64), 0, BZ_TABLE_N - 2)
    fp = (fn[k + 1] - fn[k]) / (nodes[k + 1] - nodes[k])
    big = r > 100.
    return np.where(big, 1. / (4. * r), f), np.where(big, -1. / (4. * r * r), fp)


def bz_f(r):
    """BZ monopole radial function f(r) (kgeo/bfields.py:7-13) and its derivative, in closed
    form: Re Li2(2/r) through scipy.special.spence (spence(z) = Li2(1 - z)). The reference
    evaluates f by linear interpolation of a table of f on [1, 100] that it does not ship
    (kgeo/bfields.py:21-31), and 1/(4r), -1/(4r^2) beyond r = 100 (:540-543), as here."""
    r = np.asarray(r, dtype=float)
    x = 2. / r
    li2 = np.real(sp.spence(1 - x + 0j))
    lr = np.log(r / 2.)
    with np.errstate(divide='ignore', invalid='ignore'):
        P = li2 - np.where(r == 2., 0., np.log(np.abs(1 - x)) * lr)  # ln|1 - 2/r| ln(r/2) -> 0 at r = 2
    f = P * r * r * (2 * r - 3) / 8.
    f += (1 + 3 * r - 6 * r * r) * lr / 12.
    f += 11. / 72. + 1. / (3. * r) + r / 2. - r * r / 2.
    with np.errstate(invalid='ignore', divide='ignore'):
        q = np.where(r == 2., 0.5, np.log1p((r - 2.) / 2.) / (r - 2.))
    dP = -2. * q / r
    fp = dP * r * r * (2 * r - 3) / 8. + P * 3. * r * (r - 1) / 4.
    fp += (3 - 12 * r) * lr / 12. + (1 + 3 * r - 6 * r * r) / (12. * r)
    fp += -1. / (3. * r * r) + 0.5 - r
    big = r > 100.
    f = np.where(big, 1. / (4. * r), f)
    fp = np.where(big, -1. / (4. * r * r), fp)
    return f, fp


def bfield_lab(a, r, fieldtype, kw, th=np.pi / 2):
    """Lab-frame B^i = *F^{i0} of Bfield(fieldtype, **kw).bfield_lab(a, r, th)
    (kgeo/bfields.py:93-131) with the model functions :429-736."""
    r = np.asarray(r, dtype=float)
    a2 = a ** 2
    r2 = r ** 2
    sth = np.sin(th)
    cth = np.cos(th)
    abscth = np.abs(cth)
    cth2 = cth ** 2
    sth2 = sth ** 2
    Delta = r2 - 2 * r + a2
    Sigma = r2 + a2 * cth2
    gdet = sth * Sigma
    rp = 1 + np.sqrt(1 - a2)
    if fieldtype in ('rad', 'vert', 'tor', 'simple', 'simple_rm1'):
        coef = {'rad': (1, 0, 0), 'vert': (0, 1, 0), 'tor': (0, 0, 1)}.get(
            fieldtype, (kw.get('Cr', 0), kw.get('Cvert', 0), kw.get('Cph', 0)))
        arad, avert, ator = coef
        gd = np.abs(sth) * Sigma
        if fieldtype == 'simple_rm1':
            Br = arad * (r * sth / gd) + avert * (r * cth / gd)
        else:
            Br = arad * (sth / gd) + avert * (r * cth / gd)
        return Br, avert * (-sth / gd), ator * (1. / gd)
    C = kw.get('C', 1)
    if fieldtype == 'monopoleA':
        omegah = a / (2 * rp)
        phih = 4 * np.pi * C
        omegaf = kw.get('omegafac', 0.5) * omegah
        I = phih * (sth ** 2) * rp * (omegaf - omegah) / (rp ** 2 + a ** 2 * cth ** 2)
        return (phih / (4 * np.pi)) / Sigma, 0 * r, I / (2 * np.pi * Delta * (sth ** 2))
    if fieldtype == 'bz_guess':
        Pi = (r2 + a2) ** 2 - a2 * Delta * sth2
        OmegaH = a / (2 * rp)
        spin = np.abs(a)
        f2 = (6 * np.pi * np.pi - 49.) / 72.
        omega2 = 1. / 32. - (4 * f2 - 1) * sth2 / 64.
        OmegaBZ = spin * (1. / 8.) + (spin ** 3) * omega2
        if a < 0:
            OmegaBZ *= -1
        Br = C / r2
        return Br, 0 * Br, (-1 * (OmegaH - OmegaBZ) * np.sqrt(Pi) / Delta) * Br
    if fieldtype == 'bz_monopole':
        fr, frp = bz_f_table(r) if kw.get('table', False) else bz_f(r)
        f2 = (6 * np.pi * np.pi - 49.) / 72.
        omega2 = 1. / 32. - sth2 * (4 * f2 - 1) / 64.
        if kw.get('secondorder_only', False):
            Br = C / r2 + C * a2 * (-cth2 / (r2 * r2) + fr * (0.5 + 1.5 * np.cos(2 * th)) / r2)
            Bth = -C * a2 * frp * cth * sth / r2
            Bph = -C * 0.125 * a / (r2 - 2 * r) + C * (a ** 3) * (0.125 / ((r2 - 2 * r) ** 2)
                                                                - (omega2 + 0.25 * cth2 * fr) / (r2 - 2 * r))
            return Br, Bth, Bph
        dphidtheta = C * sth * (1 + 0.5 * a2 * fr * (1 + 3 * np.cos(2 * th)))
        dphidr = C * a2 * sth2 * cth * frp
        I = -1 * C * 2 * np.pi * sth2 * (a / 8. + (a ** 3) * (omega2 + 0.25 * fr * cth2))
        return dphidtheta / gdet, -dphidr / gdet, I / (2 * np.pi * Delta * sth2)
    if fieldtype == 'bz_para':
        psi = r * (1 - abscth) + rp * (1 + abscth) * (1 - np.log(1 + abscth)) - 2 * rp * (1 - np.log(2))
        dpsidtheta = np.sign(cth) * sth * (r + rp * np.log(1 + abscth))
        dpsidr = 1 - abscth
        argvals = -psi / rp + np.log(4)
        w = sp.lambertw(argvals, k=0)
        x = np.exp(w)
        y = 1 + psi / (1 + w) / (x * (2 - x))
        om = np.real(a / 4 / y)
        OmegaBZ = np.where(argvals >= -1 / np.e, C * om, 0.)
        I = -4 * np.pi * psi * OmegaBZ * np.sign(cth)
        return C * dpsidtheta / gdet, -C * dpsidr / gdet, I / (2 * np.pi * Delta * sth2)
    if fieldtype == 'power':
        p = kw.get('p', 1)
        psi = r ** p * (1 - abscth)
        dpsidtheta = np.sign(cth) * sth * (r ** p)
        dpsidr = p * psi / r
        if kw.get('usemono', False) or p == 0:
            OmegaBZ = a / 8
        else:
            cthh = 1 - psi * rp ** (-p)
            OmegaBZ = a / (4 + 8 / (1 + cthh))
        if p > 0:
            I = -4 * np.pi * psi * OmegaBZ * np.sign(cth)
        else:
            I = -2 * np.pi * psi * (2 - psi) * OmegaBZ * np.sign(cth)
        return C * dpsidtheta / gdet, -C * dpsidr / gdet, I / (2 * np.pi * Delta * sth2)
    if fieldtype == 'gen_power':
        n_I = kw.get('n_I', 0)
        p_val = kw.get('p_val', 1)
        I_0 = (a * np.pi * sth2) / (rp * rp + a2 * cth2)
        dpsidtheta = sth * ((r / rp) ** p_val)
        if not kw.get('isAbove', True):
            I_0 = -1 * I_0
            dpsidtheta = -1 * dpsidtheta
        I = I_0 * (r / rp) ** (-1 * n_I)
        dpsidr = (1 - np.abs(cth)) * ((p_val * (r ** (p_val - 1))) / (rp ** p_val))
        return dpsidtheta / gdet, -1 * (dpsidr / gdet), I / (2 * np.pi * Delta * sth2)
    raise ValueError(fieldtype)


def pol_quantities(a, r, lam, eta, kr_sign, kth_sign, u, B, th=np.pi / 2, full=False):
    """(sinthb, kappa, cos2chi-free pieces) of calc_polquantities for a lab-frame field
    (kgeo/equatorial_images.py:336-487) with the tetrads of Velocity.tetrades
    (kgeo/velocities.py:124-176). u = (u0, u1, u2, u3), B = (B1, B2, B3). Returns
    (sinthb, kappa) with kappa the complex Penrose-Walker constant."""
    a2 = a ** 2
    r2 = r ** 2
    cth2 = np.cos(th) ** 2
    sth2 = np.sin(th) ** 2
    Delta = r2 - 2 * r + a2
    Sigma = r2 + a2 * cth2
    g00 = -(1 - 2 * r / Sigma)
    g11 = Sigma / Delta
    g22 = Sigma
    g33 = (r2 + a2 + 2 * r * a2 * sth2 / Sigma) * sth2
    g03 = -2 * r * a * sth2 / Sigma
    g00_up = -(r2 + a2 + 2 * r * a2 * sth2 / Sigma) / Delta
    g11_up = Delta / Sigma
    g22_up = 1. / Sigma
    g33_up = (Delta - a2 * sth2) / (Sigma * Delta * sth2)
    g03_up = -(2 * a * r) / (Sigma * Delta)
    u0, u1, u2, u3 = u
    u0_l = g00 * u0 + g03 * u3
    u1_l = g11 * u1
    u2_l = g22 * u2
    u3_l = g33 * u3 + g03 * u0
    # tetrads (kgeo/velocities.py:145-168)
    Nr = np.sqrt(-g11 * (u0_l * u0 + u3_l * u3) * (1 + u2_l * u2))
    Nth = np.sqrt(g22 * (1 + u2_l * u2))
    Nph = np.sqrt(-Delta * sth2 * (u0_l * u0 + u3_l * u3))
    e0_x, e1_x, e2_x, e3_x = u1_l * u0 / Nr, -(u0_l * u0 + u3_l * u3) / Nr, 0, u1_l * u3 / Nr
    e0_y, e1_y, e2_y, e3_y = u2_l * u0 / Nth, u2_l * u1 / Nth, (1 + u2_l * u2) / Nth, u2_l * u3 / Nth
    e0_z, e1_z, e2_z, e3_z = u3_l / Nph, 0, 0, -u0_l / Nph
    # fluid-frame field, e^mu = 0 (kgeo/equatorial_images.py:395-414)
    B1, B2, B3 = B
    b0 = B1 * u1_l + B2 * u2_l + B3 * u3_l
    b1 = (B1 + b0 * u1) / u0
    b2 = (B2 + b0 * u2) / u0
    b3 = (B3 + b0 * u3) / u0
    b0_l = g00 * b0 + g03 * b3
    b1_l = g11 * b1
    b2_l = g22 * b2
    b3_l = g33 * b3 + g03 * b0
    Bp_x = e0_x * b0_l + e1_x * b1_l + e2_x * b2_l + e3_x * b3_l
    Bp_y = e0_y * b0_l + e1_y * b1_l + e2_y * b2_l + e3_y * b3_l
    Bp_z = e0_z * b0_l + e1_z * b1_l + e2_z * b2_l + e3_z * b3_l
    Bp_mag = np.sqrt(Bp_x ** 2 + Bp_y ** 2 + Bp_z ** 2)
    # normal to the field surface in the comoving frame (kgeo/equatorial_images.py:390-393, 416-419)
    gdet = Sigma * np.sqrt(sth2)
    norm1_l = -B2 * gdet
    norm2_l = B1 * gdet
    norm_x = e1_x * norm1_l + e2_x * norm2_l
    norm_y = e1_y * norm1_l + e2_y * norm2_l
    norm_z = e1_z * norm1_l + e2_z * norm2_l
    norm_mag = np.sqrt(norm_x ** 2 + norm_y ** 2 + norm_z ** 2)
    # photon wavevector (kgeo/equatorial_images.py:442-462)
    R = (r2 + a2 - a * lam) ** 2 - Delta * (eta + (lam - a) ** 2)
    TH = eta + a2 * cth2 - lam * lam * cth2 / sth2
    k0_l = -1
    k1_l = kr_sign * np.sqrt(R) / Delta
    k2_l = kth_sign * np.sqrt(TH)
    k3_l = lam
    k0 = g00_up * k0_l + g03_up * k3_l
    k1 = g11_up * k1_l
    k2 = g22_up * k2_l
    k3 = g33_up * k3_l + g03_up * k0_l
    kp_x = e0_x * k0_l + e1_x * k1_l + e2_x * k2_l + e3_x * k3_l
    kp_y = e0_y * k0_l + e1_y * k1_l + e2_y * k2_l + e3_y * k3_l
    kp_z = e0_z * k0_l + e1_z * k1_l + e2_z * k2_l + e3_z * k3_l
    kp_mag = np.sqrt(kp_x ** 2 + kp_y ** 2 + kp_z ** 2)
    # polarisation vector and emission angle (:470-485)
    f_x = (kp_y * Bp_z - kp_z * Bp_y) / kp_mag
    f_y = (kp_z * Bp_x - kp_x * Bp_z) / kp_mag
    f_z = (kp_x * Bp_y - kp_y * Bp_x) / kp_mag
    sinthb = np.sqrt(f_x ** 2 + f_y ** 2 + f_z ** 2) / Bp_mag
    f0 = e0_x * f_x + e0_y * f_y + e0_z * f_z
    f1 = e1_x * f_x + e1_y * f_y + e1_z * f_z
    f2 = e2_x * f_x + e2_y * f_y + e2_z * f_z
    f3 = e3_x * f_x + e3_y * f_y + e3_z * f_z
    A = k0 * f1 - k1 * f0 + a * sth2 * (k1 * f3 - k3 * f1)
    Bk = ((r2 + a2) * (k3 * f2 - k2 * f3) - a * (k0 * f2 - k2 * f0)) * np.sin(th)
    kappa = (r - 1j * a * np.cos(th)) * (A - 1j * Bk)
    if full:
        kdotnorm = kp_x * (norm_x / norm_mag) + kp_y * (norm_y / norm_mag) + kp_z * (norm_z / norm_mag)
        pathlength = np.abs(kp_mag / kdotnorm)
        return sinthb, kappa, pathlength, Bp_mag ** 2
    return sinthb, kappa


def evpa(a, th_o, alpha, beta, kappa):
    """(cos 2chi, sin 2chi) at the observer by the Penrose-Walker constant;
    kgeo/equatorial_images.py:524-544."""
    mu = -(alpha + a * np.sin(th_o))
    k1 = np.real(kappa)
    k2 = np.imag(kappa)
    den = (beta ** 2 + mu ** 2) * (k1 ** 2 + k2 ** 2)
    c2 = ((beta * k1 + mu * k2) ** 2 - (mu * k1 - beta * k2) ** 2) / den
    s2 = (2 * (beta * k1 + mu * k2) * (mu * k1 - beta * k2)) / den
    return c2, s2


def pathlength_equatorial(a, r, lam, eta, kth_sign, g, diskangle=0.1, th=np.pi / 2):
    """Rest-frame path length through a disk of opening angle diskangle (Narayan+2021 eq 13);
    kgeo/equatorial_images.py:489-522 (u^theta = 0, th = pi/2)."""
    cth2 = np.cos(th) ** 2
    sth2 = np.sin(th) ** 2
    TH = eta + a * a * cth2 - lam * lam * cth2 / sth2
    k2_l = kth_sign * np.sqrt(TH)
    kyhat = -k2_l / r
    return (diskangle * r) * ((1 / g) / kyhat)


def make_image_px(a, r_o, th_o, mbar_max, alpha, beta, emis=('bpl', {}), vel=('zamo', {}), specind=1,
                  sinthb=np.pi / 4., bfield=('rad', {}), polarization=False, pathlength=False, diskangle=0.1):
    """make_image's (I, Q, U, r, t, g, sinthb, n, np [, lp, Ie]) on given pixels.

    kgeo/equatorial_images.py:23-122 (the pixel grid is image_grid's) with Iobs :124-264:
    polarization=True takes sin(theta_B) and the EVPA from calc_polquantities / calc_evpa
    (:336-487, :524-544) for the lab-frame field ``bfield`` = (fieldtype, kwargs);
    pathlength=True multiplies the emission by |calc_pathlength_equatorial| (:489-522) and one
    more power of g.
    """
    emistype, ekw = emis
    veltype, vkw = vel
    cut_in = ekw.get('emiscut_in', 0)
    cut_out = ekw.get('emiscut_out', 1.e10)
    rh = 1 + np.sqrt(1 - a ** 2)
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    n_pix = len(alpha)
    keys = ('I', 'Q', 'U', 'r', 't', 'g', 'sinthb') + (('lp', 'Ie') if pathlength else ())
    out = {k: np.zeros((n_pix, mbar_max + 1)) for k in keys}
    nmax_out = None
    for mbar in range(mbar_max + 1):
        r_s, Ir, Imax, Nmax = r_equatorial(a, r_o, th_o, mbar, alpha, beta)
        zero = (Nmax < mbar) + (Nmax == -1) + (r_s <= rh)
        if cut_in > 0:
            zero = zero + (r_s < cut_in)
        if cut_out > 0:
            zero = zero + (r_s > cut_out)
        cols = {k: np.zeros(n_pix) for k in keys}
        if np.any(~zero):
            live = ~zero
            rl = r_s[live]
            inside = ~outside_critical(a, th_o, alpha[live], beta[live]).astype(bool)
            kr = np.where(inside + (Ir[live] <= 0.5 * Imax[live]), 1., -1.)
            kth = -1 * np.power(-1, np.mod(mbar, 2)) if th_o < 0.5 * np.pi else 1 * np.power(-1, np.mod(mbar, 2))
            u0, u1, u2, u3 = velocity(a, rl, veltype, vkw)
            gg = redshift(a, rl, lam[live], eta[live], kr, kth, u0, u1, u2, u3)
            if polarization:
                B = bfield_lab(a, rl, bfield[0], bfield[1])
                sb, kappa = pol_quantities(a, rl, lam[live], eta[live], kr, kth, (u0, u1, u2, u3), B)
                c2, s2 = evpa(a, th_o, alpha[live], beta[live], kappa)
            else:
                sb = sinthb
            j = emissivity(a, rl, emistype, ekw)
            j = j * gg ** specind
            j = j * sb ** (1 + specind)
            if pathlength:
                lp = pathlength_equatorial(a, rl, lam[live], eta[live], kth, gg, diskangle=diskangle)
                j = j * np.abs(lp)
                cols['I'][live] = (gg ** 3) * j
                cols['Ie'][live] = j
                cols['lp'][live] = lp
            else:
                cols['I'][live] = (gg ** 2) * j
            if polarization:
                cols['Q'][live] = c2 * cols['I'][live]
                cols['U'][live] = s2 * cols['I'][live]
            cols['g'][live] = gg
            cols['sinthb'][live] = sb
        cols['r'] = r_s
        cols['t'] = Ir
        for k in keys:
            out[k][:, mbar] = cols[k]
        nmax_out = Nmax
    r1, r2, r3, r4, _ = quartic_roots(a, lam, eta)
    tau_tot = mino_total(a, r_o, eta, r1, r2, r3, r4)
    out['n'] = nmax_out
    out['np'] = n_poloidal_orbits(a, th_o, alpha, beta, tau_tot)
    return out


def redshift(a, r, lam, eta, kr_sign, kth_sign, u0, u1, u2, u3, th=np.pi / 2):
    """g = 1 / (-k.u); kgeo/equatorial_images.py:307-334."""
    a2 = a ** 2
    r2 = r ** 2
    cth2 = np.cos(th) ** 2
    sth2 = np.sin(th) ** 2
    Delta = r2 - 2 * r + a2
    R = (r2 + a2 - a * lam) ** 2 - Delta * (eta + (lam - a) ** 2)
    TH = eta + a2 * cth2 - lam * lam * cth2 / sth2
    return 1 / (1 * u0 - lam * u3 - np.sign(kth_sign) * u2 * np.sqrt(TH) - np.sign(kr_sign) * u1 * np.sqrt(R) / Delta)


def image_order(a, r_o, th_o, mbar, alpha, beta, p1=-2.0, p2=-0.5,
                fac_subkep=1, beta_phi=1, beta_r=1, retrograde=False,
                specind=1, sinthb=np.pi / 4., emiscut_in=0, emiscut_out=1.e10):
    """Unpolarised I, g, r_s, Ir, Imax, Nmax of one image order (bpl emissivity, general velocity).

    kgeo/equatorial_images.py:124-264 with kgeo/emissivities.py:83-127 and
    kgeo/velocities.py:442-470.
    """
    rh = 1 + np.sqrt(1 - a ** 2)
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    r_s, Ir, Imax, Nmax = r_equatorial(a, r_o, th_o, mbar, alpha, beta)
    g = np.zeros(alpha.shape)
    I = np.zeros(alpha.shape)
    zero = (Nmax < mbar) + (Nmax == -1) + (r_s <= rh)
    if emiscut_in > 0:
        zero = zero + (r_s < emiscut_in)
    if emiscut_out > 0:
        zero = zero + (r_s > emiscut_out)
    if np.any(~zero):
        live = ~zero
        inside = ~outside_critical(a, th_o, alpha[live], beta[live]).astype(bool)
        kr = np.empty(inside.shape)
        outgoing = inside + (Ir[live] <= 0.5 * Imax[live])
        kr[outgoing] = 1
        kr[~outgoing] = -1
        kth = -1 * np.power(-1, np.mod(mbar, 2)) if th_o < 0.5 * np.pi else 1 * np.power(-1, np.mod(mbar, 2))
        u0, u1, u2, u3 = u_general(a, r_s[live], fac_subkep=fac_subkep, beta_phi=beta_phi,
                                   beta_r=beta_r, retrograde=retrograde)
        gg = redshift(a, r_s[live], lam[live], eta[live], kr, kth, u0, u1, u2, u3)
        g[live] = gg
        j = emis_bpl(a, r_s[live], p1=p1, p2=p2)
        j *= (gg ** specind)
        j *= (sinthb ** (1 + specind))
        I[live] = (gg ** 2) * j
    return I, g, r_s, Ir, Imax, Nmax


def image_grid(alpha_min, alpha_max, beta_min, beta_max, psize):
    """Pixel grid of make_image; kgeo/equatorial_images.py:48-55 (spacing is (max-min)/(n-1))."""
    n_a = int(np.floor(alpha_max - alpha_min) / psize)
    alphas = np.linspace(alpha_min, alpha_min + n_a * psize, n_a)
    n_b = int(np.floor(beta_max - beta_min) / psize)
    betas = np.linspace(beta_min, beta_min + n_b * psize, n_b)
    A, B = np.meshgrid(alphas, betas)
    return A.flatten(), B.flatten()


# ----------------------------------------------------------------------------
# lensed curves of constant equatorial radius and the critical curve
# ----------------------------------------------------------------------------

CURVE_INF = 1.e50   # kgeo/equatorial_lensing.py:17


def r_equatorial2(rho, varphi, a, th0, mbar=0):
    """r_s at image-plane polar point (rho, varphi) for r_o = inf, with INF outside / 1 inside
    the critical curve where there is no crossing; kgeo/equatorial_lensing.py:198-216."""
    alpha = np.array([np.cos(varphi) * rho])
    beta = np.array([np.sin(varphi) * rho])
    r = r_equatorial(a, np.inf, th0, mbar, alpha, beta)[0][0]
    out = outside_critical(a, th0, alpha, beta)[0]
    if r <= 0 and out == 1:
        r = CURVE_INF
    elif r <= 0:
        r = 1
    return r


def rho_bracket(mbar, req):
    """rho_of_req's bracket, kgeo/equatorial_lensing.py:227-236."""
    if mbar == 0:
        return 0, req + 5
    if mbar == 1:
        return 0, 100
    return 1, 10


def rho_of_req(a, th0, req, mbar=0, varphis=None):
    """(varphis, rhos, alphas, betas) by scipy.optimize.brentq per angle on objfunc;
    kgeo/equatorial_lensing.py:218-243."""
    from scipy.optimize import brentq
    if varphis is None:
        varphis = np.linspace(-180, 179, 360) * np.pi / 180.
    lo, hi = rho_bracket(mbar, req)
    rhos = np.array([brentq(lambda rho: r_equatorial2(rho, vp, a, th0, mbar=mbar) - req, lo, hi)
                     for vp in varphis])
    return varphis, rhos, np.cos(varphis) * rhos, np.sin(varphis) * rhos


def critical_curve(a, th0, n=100000):
    """Critical curve (alpha, beta) with the reference's NaN mask and mirror;
    kgeo/equatorial_lensing.py:260-289."""
    rminus = 2 * (1 + np.cos(2. * np.arccos(-a) / 3.))
    rplus = 2 * (1 + np.cos(2. * np.arccos(a) / 3.))
    r = np.linspace(rminus, rplus, n)
    lam = -(r ** 3 + a ** 2 + r * (a ** 2) - 3 * r ** 2) / (a * r - a)
    eta = (r ** 2) * (3 * r ** 2 + a ** 2 - lam ** 2) / (r ** 2 - a ** 2)
    alpha = -lam / np.sin(th0)
    with np.errstate(invalid='ignore'):
        beta = np.sqrt(eta + (a * np.cos(th0)) ** 2 - (lam / np.tan(th0)) ** 2)
    mask = np.isnan(alpha) + np.isnan(beta)
    alpha = alpha[~mask]
    beta = beta[~mask]
    return np.hstack((alpha, np.flip(alpha))), np.hstack((beta, -np.flip(beta)))


# ----------------------------------------------------------------------------
# off-equatorial jet: crossings of the geodesics with a field line psi = psi_target
# ----------------------------------------------------------------------------

JET_MAXTAUFRAC = 1. - 1.e-10   # kgeo/solver.py:12


def psifunc(r, theta, a, model='para', pval=1):
    """Stream function psi(r, theta) of the jet models; kgeo/solver.py:14-38."""
    abscth = np.abs(np.cos(theta))
    if model == 'para':
        rp = 1 + np.sqrt(1 - a ** 2)
        return r * (1 - abscth) + rp * (1 + abscth) * (1 - np.log(1 + abscth)) - 2 * rp * (1 - np.log(2))
    if model == 'mono':
        return 1 - abscth
    if model == 'power':
        return r ** pval * (1 - abscth)
    return 0


def get_maxtau_forwardjet(a, r_o, th_o, alpha, beta, neqmax=1):
    """Mino time bound of the crossing search (the neqmax-th equatorial crossing, or the
    total); kgeo/solver.py:57-87."""
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    r1, r2, r3, r4, _ = quartic_roots(a, lam, eta)
    tau_tot2 = mino_total(a, r_o, eta, r1, r2, r3, r4) * JET_MAXTAUFRAC
    if neqmax is None:
        return tau_tot2
    up, um, ratio, a2um = u_roots(a, th_o, lam, eta)
    F0 = sp.ellipkinc(np.arcsin(np.cos(th_o) / np.sqrt(up)), ratio)
    K = sp.ellipkinc(0.5 * np.pi, ratio)
    mmax = (neqmax - 1) + np.heaviside(beta, 0)
    taumax = (2 * mmax * K - np.sign(beta) * F0) / np.sqrt(-um * a ** 2)
    taumax[eta <= 0] = tau_tot2[eta <= 0]
    return np.min(np.array([taumax, tau_tot2]), axis=0)


def getguesses(geo, a, rout, inc, alphas, betas, psitarget, ngeo, neqmax=1, model='para', pval=1):
    """Mino-time guesses of the crossings: midpoints of the sampled geodesic's sign changes of
    psi - psi_target before the search bound (endpoints excluded), or the flat-space guesses
    of nearly face-on views at large impact parameter; padded with -1 to (guesses, npix).
    kgeo/solver.py:97-134. geo: dict with 'r', 'th', 'mino_times' (ngeo, npix)."""
    out = []
    taumaxes = get_maxtau_forwardjet(a, rout, inc, alphas, betas, neqmax=neqmax)
    psig = psifunc(geo['r'], geo['th'], a, model=model, pval=pval) - psitarget
    for i in range(len(alphas)):
        b = np.sqrt(alphas[i] ** 2 + betas[i] ** 2)
        if np.abs(np.sin(inc)) < .1 and b > 100:
            if model == 'power' and pval > 0:
                rparam = (b ** 2 / (2 * psitarget)) ** (1 / (2 - pval))
                out.append(np.array([1 / rparam, 2 / b - 1 / rparam]))
                continue
            elif model == 'para':
                rparam = (b ** 2 + psitarget ** 2) / (2 * psitarget)
                out.append(np.array([1 / rparam, 2 / b - 1 / rparam]))
                continue
        mf = np.roll(psig[:, i], -1) * psig[:, i]
        indmax = np.argmin(np.abs(geo['mino_times'][:, i] - taumaxes[i]))
        mf = mf[:indmax + 1][1:-2]
        js = np.where(mf < 0)[0] + 1
        if len(js) == 0:
            out.append(np.array([-1]))
            continue
        out.append(np.array([(geo['mino_times'][j, i] + geo['mino_times'][j + 1, i]) / 2 for j in js]))
    n = max(len(x) for x in out)
    res = -np.ones((len(out), n))
    for i, x in enumerate(out):
        res[i, :len(x)] = x
    return np.transpose(res)


def getneq(a, tau, u_minus, u_plus, th_o, betas):
    """Equatorial crossings before Mino time tau (GL19b Eqs 81-82); kgeo/solver.py:40-55."""
    ratio = u_plus / u_minus
    F0 = sp.ellipkinc(np.arcsin(np.cos(th_o) / np.sqrt(u_plus)), ratio)
    K = sp.ellipkinc(0.5 * np.pi, ratio)
    mval = (np.sqrt(-u_minus * a ** 2) * tau + np.sign(betas) * F0) / (2 * K)
    return np.ceil(np.nan_to_num(mval - np.heaviside(betas, 0)))


def findroot(geo, psitarget, alpha, beta, r_o, th_o, a, ngeo, model='para', neqmax=1, tol=1e-8, pval=1,
             converged=False):
    """(tau, r_s, th_s, sign p_r, sign p_theta, n_eq, guesses shape) of every crossing of the
    geodesics with psi = psi_target: scipy.optimize.newton (secant) from getguesses' Mino times
    on coords_at_tau; kgeo/solver.py:136-207. converged=True appends newton's per-guess
    convergence flags."""
    from scipy.optimize import newton
    guesses = getguesses(geo, a, r_o, th_o, alpha, beta, psitarget, ngeo, neqmax=neqmax, model=model, pval=pval)
    shape = guesses.shape
    G = shape[0]
    At = np.tile(alpha, G)
    Bt = np.tile(beta, G)
    g = guesses.flatten()

    def f(tau):
        _, (t, r, th, ph) = coords_at_tau(a, r_o, th_o, At, Bt, np.reshape(tau, (1, len(tau))))
        v = psifunc(r[0], th[0], a, model=model, pval=pval) - psitarget
        v[g == -1] = 0
        return v

    with np.errstate(all='ignore'):
        root, conv, _ = newton(f, g, maxiter=500, tol=tol, full_output=True)[:3]
        _, (t0, r0, th0, ph0) = coords_at_tau(a, r_o, th_o, At, Bt, root.reshape(1, -1))
        _, (t1, r1, th1, ph1) = coords_at_tau(a, r_o, th_o, At, Bt, (root * (1 + 1e-5)).reshape(1, -1))
    signpr = np.sign(r0 - r1)[0]
    signpth = np.sign(th0 - th1)[0]
    r_s = np.copy(r0[0])
    th_s = np.copy(th0[0])
    lam, eta = conserved(a, th_o, At, Bt)
    up, um, _, _ = u_roots(a, th_o, lam, eta)
    with np.errstate(all='ignore'):
        neq = getneq(a, root, um, up, th_o, Bt)
    none = g == -1
    root[none] = r_s[none] = th_s[none] = signpr[none] = signpth[none] = 0
    if converged:
        return root, r_s, th_s, signpr, signpth, neq, shape, conv
    return root, r_s, th_s, signpr, signpth, neq, shape


# ----------------------------------------------------------------------------
# off-equatorial jet emission (the monopole field-line model of getstokes)
# ----------------------------------------------------------------------------


def omega_field(a, r, th, fieldtype, kw):
    """Field-line angular speed Omega_F (kgeo/bfields.py:175-196) of the models the
    monopole jet uses: 'bz_monopole' (:590-593) and 'power' (:609-615)."""
    sth2 = np.sin(th) ** 2
    if fieldtype == 'bz_monopole':
        f2 = (6 * np.pi * np.pi - 49.) / 72.
        omega2 = 1. / 32. - sth2 * (4 * f2 - 1) / 64.
        om = np.abs(a) / 8. + np.abs(a) ** 3 * omega2
        return -om if a < 0 else om
    if fieldtype == 'power':
        p = kw.get('p', 1)
        if kw.get('usemono', False) or p == 0:
            return a / 8 + 0 * r
        rp = 1 + np.sqrt(1 - a ** 2)
        psi = r ** p * (1 - np.abs(np.cos(th)))
        return a / (4 + 8 / (1 + (1 - psi * rp ** (-p))))
    raise ValueError(fieldtype)


def u_driftframe(a, r, th, fieldtype, kw, nu_parallel=0):
    """Drift-frame four-velocity of the force-free field (kgeo/velocities.py:487-623) for a
    numeric parallel boost and no Lorentz-factor cap."""
    nu = nu_parallel * np.ones_like(r)
    if np.any(np.logical_or(nu > 1, nu < -1)):
        raise Exception("nu_parallel should be in the range (-1,1)")
    a2 = a ** 2
    r2 = r ** 2
    cth2 = np.cos(th) ** 2
    sth2 = np.sin(th) ** 2
    Delta = r2 - 2 * r + a2
    Sigma = r2 + a2 * cth2
    Xi = (r2 + a2) ** 2 - Delta * a2 * sth2
    omegaz = 2 * a * r / Xi
    gdet = Sigma * np.sin(th)
    g11 = Sigma / Delta
    g22 = Sigma
    g33 = Xi * sth2 / Sigma
    alpha = np.sqrt(Delta * Sigma / Xi)
    eta3 = 2 * a * r / np.sqrt(Delta * Sigma * Xi)
    omegaf = omega_field(a, r, th, fieldtype, kw)
    B1, B2, B3 = bfield_lab(a, r, fieldtype, kw, th=th)
    E1 = (omegaf - omegaz) * Xi * np.sin(th) * B2 / Sigma
    E2 = -(omegaf - omegaz) * Xi * np.sin(th) * B1 / (Sigma * Delta)
    E3 = 0
    Bsq = g11 * B1 * B1 + g22 * B2 * B2 + g33 * B3 * B3
    Esq = g11 * E1 * E1 + g22 * E2 * E2 + g33 * E3 * E3
    B1c, B2c, B3c = g11 * B1, g22 * B2, g33 * B3
    E1c, E2c, E3c = g11 * E1, g22 * E2, g33 * E3
    vperp1 = (alpha / (Bsq * gdet)) * (E2c * B3c - B2c * E3c)
    vperp2 = (alpha / (Bsq * gdet)) * (E3c * B1c - B3c * E1c)
    vperp3 = (alpha / (Bsq * gdet)) * (E1c * B2c - B1c * E2c)
    vpar_max = np.sqrt(1 - Esq / Bsq)
    v1 = vperp1 + nu * vpar_max * B1 / np.sqrt(Bsq)
    v2 = vperp2 + nu * vpar_max * B2 / np.sqrt(Bsq)
    v3 = vperp3 + nu * vpar_max * B3 / np.sqrt(Bsq)
    vsq = g11 * v1 * v1 + g22 * v2 * v2 + g33 * v3 * v3
    gamma = 1. / np.sqrt(1 - vsq)
    return gamma / alpha, gamma * (v1 + 0), gamma * (v2 + 0), gamma * (v3 + eta3)


def r0min_mono(theta, Omegaf, spin, M=1.0):
    """Stagnation radius of the monopole outflow: a root of the quintic of
    kgeo/ff_boost.py:7-18 (numpy's sorted roots, index 4)."""
    theta = np.arccos(np.abs(np.cos(theta)))
    c0 = -spin ** 2 / 2 * M * np.cos(theta) ** 2 * (2 - spin * Omegaf + spin * Omegaf * np.cos(2 * theta)) ** 2
    c1 = -2 * spin ** 4 * Omegaf ** 2 * np.cos(theta) ** 4 * np.sin(theta) ** 2
    c2 = M / 2 * (2 - spin * Omegaf + spin * Omegaf * np.cos(2 * theta)) ** 2
    c3 = -spin ** 2 * Omegaf ** 2 * np.sin(2 * theta) ** 2
    c5 = -2 * Omegaf ** 2 * np.sin(theta) ** 2
    roots = np.polynomial.polynomial.Polynomial([c0, c1, c2, c3, 0.0, c5]).roots()
    return np.real(roots[4])


def eta_mono(r, theta, r0, spin, sigma):
    """Mass loading of the monopole outflow, a Gaussian source of width sigma about the
    stagnation radius integrated in closed form; kgeo/densityfuncs.py:32-44."""
    if sigma == 0:
        return np.sign(r - r0)
    cth = np.cos(theta)
    t1 = 2 * sigma * (2 * r0 - (r + r0) * np.exp(-(r - r0) ** 2 / (2 * sigma ** 2)))
    t2 = np.sqrt(2 * np.pi) * sp.erf((r - r0) / (np.sqrt(2) * sigma)) * (r0 ** 2 + sigma ** 2 + spin ** 2 * cth ** 2)
    den = 4 * r0 * sigma + np.sqrt(2 * np.pi) * sigma ** 2 + np.sqrt(2 * np.pi) * (r0 ** 2 + spin ** 2 * cth ** 2)
    return (t1 + t2) / den


def jet_stagnation(rvals, thvals, shape, spin):
    """(r0, Omega) of density_mono_all (kgeo/densityfuncs.py:47-60): the first crossing of the
    first guess row fixes the field line's Omega and stagnation radius."""
    rnew = np.reshape(rvals, shape)
    thnew = np.arccos(np.abs(np.cos(np.reshape(thvals, shape))))
    i0 = np.where(rnew[0] != 0)[0][0]
    om = omega_field(spin, rnew[0][i0], thnew[0][i0], 'bz_monopole', {})
    return r0min_mono(thnew[0][i0], om, spin, 1.0), om


def density_mono_all(rvals, thvals, shape, spin, nu_parallel, sigma, table=False):
    """Continuity-equation density rho = eta B^r / u^r along the monopole field line at the
    reflected crossings; kgeo/densityfuncs.py:47-78."""
    r0, _ = jet_stagnation(rvals, thvals, shape, spin)
    rr = np.reshape(rvals, shape)
    tt = np.arccos(np.abs(np.cos(np.reshape(thvals, shape))))
    out = []
    for k in range(shape[0]):
        B1 = bfield_lab(spin, rr[k], 'bz_monopole', {'C': 1, 'table': table}, th=tt[k])[0]
        u1 = u_driftframe(spin, rr[k], tt[k], 'bz_monopole', {'C': 1, 'table': table}, nu_parallel)[1]
        out.append(eta_mono(rr[k], tt[k], r0, spin, sigma) * B1 / u1)
    return np.nan_to_num(np.array(out).flatten(), nan=0.0)


def iobs_off(a, r_o, r_s, th_o, alpha, beta, kr, kth, field, nu_parallel, th_s, density, specind=1):
    """(I, Q, U) of the off-equatorial crossings (kgeo/off_eq.py:15-119) for the constant
    emissivity with a density, the drift-frame velocity and polarisation."""
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    rh = 1 + np.sqrt(1 - a ** 2)
    u = u_driftframe(a, r_s, th_s, field[0], field[1], nu_parallel)
    gg = redshift(a, r_s, lam, eta, kr, kth, *u, th=th_s)
    B = bfield_lab(a, r_s, field[0], field[1], th=th_s)
    sinthb, kappa, plen, bsq = pol_quantities(a, r_s, lam, eta, kr, kth, u, B, th=th_s, full=True)
    c2, s2 = evpa(a, th_o, alpha, beta, kappa)
    Iemis = np.ones(r_s.shape) * density
    Iemis = Iemis * bsq ** ((1 + specind) / 2)
    I = (gg ** 3) * (gg ** specind) * plen * Iemis * (sinthb ** (1 + specind))
    Q = c2 * I
    U = s2 * I
    I[r_s <= rh] = Q[r_s <= rh] = U[r_s <= rh] = 0
    return I, Q, U


def sort_image(iobs, qobs, uobs, neqvals, shape, ashape, neqmax):
    """Per-subring and total images (kgeo/geometry.py:38-61)."""
    outs = ([], [], [])
    for neq in np.arange(0, neqmax, 1):
        for o, v in zip(outs, (iobs, qobs, uobs)):
            h = np.copy(v)
            h[neqvals != neq] = 0
            o.append(np.reshape(np.sum(np.reshape(h, shape), axis=0), ashape))
    for o, v in zip(outs, (iobs, qobs, uobs)):
        o.append(np.reshape(np.sum(np.reshape(v, shape), axis=0), ashape))
    return tuple(np.array(o) for o in outs)


def getstokes_mono(psitarget, alphavals, betavals, r_o, th_o, a, ngeo, neqmax=1, model='mono', pval=0,
                   nu_parallel=0, sigma=2, tol=1e-8, table=False):
    """getstokes (kgeo/off_eq.py:124-233) of the monopole field-line model ('mono', or 'power'
    with p = 0): crossings, densities, the emission of each crossing, the per-subring sums.
    Returns (I, Q, U, evpa) of shape (neqmax + 1, ...) and the crossings (r, th). table=True
    evaluates the BZ f(r) as the reference does (bz_f_table) instead of in closed form."""
    ashape = alphavals.shape
    A = alphavals.flatten()
    B = betavals.flatten()
    geo = raytrace(a, r_o, th_o, A, B, ngeo)
    tau, rv, tv, spr, spt, neq, shape = findroot(geo, psitarget, A, B, r_o, th_o, a, ngeo, model=model,
                                                 neqmax=neqmax, tol=tol, pval=pval)
    At = np.tile(A, shape[0])
    Bt = np.tile(B, shape[0])
    dv = density_mono_all(rv, tv, shape, a, nu_parallel, sigma, table=table)
    field = ('bz_monopole', {'C': 1, 'table': table}) if model == 'mono' else ('power', {'p': pval})
    with np.errstate(all='ignore'):
        I, Q, U = iobs_off(a, r_o, rv, th_o, At, Bt, spr, spt, field, nu_parallel, tv, dv)
    I = np.copy(I)
    Q = np.copy(Q)
    U = np.copy(U)
    I[rv == 0] = Q[rv == 0] = U[rv == 0] = 0
    I, Q, U = (np.real(np.nan_to_num(np.array(x))) for x in (I, Q, U))
    iv, qv, uv = sort_image(I, Q, U, neq, shape, ashape, neqmax)
    ev = np.nan_to_num(0.5 * np.arctan2(uv, qv))
    return iv, qv, uv, ev, np.nan_to_num(rv), np.nan_to_num(tv)


# ----------------------------------------------------------------------------
# conditioning helper for the parity tests
# ----------------------------------------------------------------------------


def pole_distance(a, r_o, th_o, alpha, beta, tau):
    """Smallest |1 - n sin^2(amplitude)| over the elliptic-Pi characteristics n > 0 that the
    reference evaluates at each sample (the r-part Pi's of kgeo/kerr_raytracing_ana.py:447-612
    and the theta-part Pi of :243-285, 326-360). Near 0 the reference's Pi, and the R1/S1
    combinations that cancel its pole, carry rounding amplified by ~1/rho.
    """
    if tau.ndim == 1:
        tau = tau.reshape(1, tau.shape[0])
    lam, eta = conserved(a, th_o, alpha, beta)
    s_o = beta_sign(beta)
    up, um, _, _, _ = theta_turning(a, th_o, lam, eta)
    r1, r2, r3, r4, _ = quartic_roots(a, lam, eta)
    rplus = 1 + np.sqrt(1 - a ** 2)
    rminus = 1 - np.sqrt(1 - a ** 2)
    out = np.full(tau.shape, np.inf)

    def upd(cols, ns, amp):
        s2 = np.sin(amp) ** 2
        for nn in ns:
            rho = np.where(nn > 0, np.abs(1 - nn * s2), np.inf)
            out[:, cols] = np.minimum(out[:, cols], rho)

    m4 = np.imag(r1) != 0
    if np.any(m4):
        a1, b1, a2, b2, CC, DD, k4, g0 = _case4_params(a, r_o, r2[m4], r4[m4])
        x_p = (rplus + b1) / a2
        x_m = (rminus + b1) / a2
        x_o = np.inf if r_o == np.inf else (r_o + b1) / a2
        gp = (g0 * x_p - 1.) / (g0 + x_p)
        gm = (g0 * x_m - 1.) / (g0 + x_m)
        Ir_o = 2. / (CC + DD) * sp.ellipkinc(np.arctan(x_o) + np.arctan(g0), k4)
        X = ((CC + DD) / 2.) * (-tau[:, m4] + Ir_o)
        am = sp.ellipj(X, k4)[3]
        upd(m4, [1 + g0 ** 2, 1 + gp ** 2, 1 + gm ** 2], am)
    m3 = (np.imag(r3) != 0) * (~m4)
    if np.any(m3):
        a1, b1, rr1, rr2, rr21, AA, BB, k3 = _case3_params(r1[m3], r2[m3], r4[m3])
        rrp1, rrp2, rrm1, rrm2 = rplus - rr1, rplus - rr2, rminus - rr1, rminus - rr2
        x_p = (AA * rrp1 - BB * rrp2) / (AA * rrp1 + BB * rrp2)
        x_m = (AA * rrm1 - BB * rrm2) / (AA * rrm1 + BB * rrm2)
        x_o = (AA - BB) / (AA + BB) if r_o == np.inf else \
            (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2))
        als = [(BB + AA) / (BB - AA), -1. / x_p, -1. / x_m]
        pref = 1. / np.sqrt(AA * BB)
        X = (1. / pref) * (-tau[:, m3] + pref * sp.ellipkinc(np.arccos(x_o), k3))
        am = sp.ellipj(X, k3)[3]
        upd(m3, [al ** 2 / (al ** 2 - 1) for al in als], am)
    m2 = (np.imag(r3) == 0.) * (~m3)
    if np.any(m2):
        rr1, rr2, rr3, rr4 = (np.real(r)[m2] for r in (r1, r2, r3, r4))
        rr31, rr32, rr41, rr42 = rr3 - rr1, rr3 - rr2, rr4 - rr1, rr4 - rr2
        k2 = (rr32 * rr41) / (rr31 * rr42)
        x_o = np.sqrt(rr31 / rr41) if r_o == np.inf else np.sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)))
        Ir_o = 2 * sp.ellipkinc(np.arcsin(x_o), k2) / np.sqrt(rr31 * rr42)
        X = 0.5 * np.sqrt(rr31 * rr42) * (-tau[:, m2] + Ir_o)
        am = sp.ellipj(X, k2)[3]
        ns = [rr41 / rr31, ((rplus - rr3) * rr41) / ((rplus - rr4) * rr31),
              ((rminus - rr3) * rr41) / ((rminus - rr4) * rr31)]
        upd(m2, ns, am)
    # theta part
    if np.any(eta > 0.):
        sel = eta >= 0.
        if np.abs(a) >= MINSPIN:
            kk = up[sel] / um[sel]
            a2um = a ** 2 * um[sel]
            pref = 1 / np.sqrt(-a2um)
            arg = np.arcsin(np.cos(th_o) / np.sqrt(up[sel]))
            Gth_o = -pref * sp.ellipkinc(arg, kk)
            snarg = np.sqrt(-a2um) * (-tau[:, sel] + s_o[sel] * Gth_o)
            _, amp = _am_beyond_quarter(snarg, kk)
            upd(sel, [up[sel]], amp)
    if np.any(eta < 0.) and np.abs(a) >= MINSPIN:
        sel = eta < 0.
        u_p, u_m = up[sel], um[sel]
        a2um = a ** 2 * u_m
        h = 1. if th_o <= np.pi / 2 else -1
        kk = 1 - u_p / u_m
        nu_o = np.arcsin(np.sqrt((np.cos(th_o) ** 2 - u_m) / (u_p - u_m)))
        Gth_o = -h * (1 / np.sqrt(a2um)) * sp.ellipkinc(nu_o, kk)
        snarg = np.sqrt(a2um) * (-tau[:, sel] + s_o[sel] * Gth_o)
        _, amp = _am_beyond_quarter(snarg, kk)
        upd(sel, [(u_p - u_m) / (1. - u_m)], amp)
    return out
