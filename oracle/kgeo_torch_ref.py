"""Pure-torch FP64 restatement of the unpolarised equatorial image, differentiable by
torch.autograd with respect to (a, th_o, e0, e1, v0, v1, v2).

TEST INFRASTRUCTURE ONLY (like kgeo_oracle.py): the gradient oracle for the image adjoint
kernel. Only tests/ import it; the product package never does.

It follows the same reference code as kgeo_oracle.make_image_px (kgeo/equatorial_images.py:
124-264, kgeo/equatorial_lensing.py:85-196, kgeo/kerr_raytracing_ana.py:404-595,
kgeo/velocities.py, kgeo/emissivities.py) but every differentiable step is a torch
operation, so autograd differentiates the closed forms themselves: the radial quartic is
solved by the reference's resolvent-cubic formula in complex arithmetic
(kgeo/kerr_raytracing_utils.py:330-380, cube roots as my_cbrt :828-855), F(phi|m) by
Carlson's duplication for R_F (a fixed number of steps), K(m) by the arithmetic-geometric
mean, and sn / cn / am by the AGM descent of DLMF 22.20. Piecewise-constant decisions (the
radial case, masks, momentum signs, half-period and branch indices) are taken from the
values and carry no gradient, as in the adjoint kernel.
"""
import numpy as np
import torch

PI = np.pi
MINSPIN = 1e-4
EP = 1e-12
COS2_EQ = np.cos(np.pi / 2.) ** 2


def rf(x, y, z, steps=32):
    """Carlson R_F by duplication (Carlson 1995) with a fixed step count, then the
    fifth-order series."""
    for _ in range(steps):
        sx, sy, sz = torch.sqrt(x), torch.sqrt(y), torch.sqrt(z)
        lam = sx * sy + sx * sz + sy * sz
        x, y, z = 0.25 * (x + lam), 0.25 * (y + lam), 0.25 * (z + lam)
    A = (x + y + z) / 3.
    X, Y = 1 - x / A, 1 - y / A
    Z = -(X + Y)
    E2 = X * Y - Z * Z
    E3 = X * Y * Z
    return (1 - E2 / 10 + E3 / 14 + E2 * E2 / 24 - 3 * E2 * E3 / 44) / torch.sqrt(A)


def agm_k(m, steps=12):
    """K(m) = pi / (2 AGM(1, sqrt(1 - m)))."""
    a = torch.ones_like(m)
    b = torch.sqrt(1 - m)
    for _ in range(steps):
        a, b = 0.5 * (a + b), torch.sqrt(a * b)
    return PI / (a + b)


def ellip_f(phi, m):
    """F(phi|m) for any real phi: F(n pi + phi0) = 2 n K + F(phi0)."""
    n = torch.round(phi.detach() / PI)
    p0 = phi - n * PI
    s, c = torch.sin(p0), torch.cos(p0)
    inc = s * rf(c * c, 1 - m * s * s, torch.ones_like(m))
    return torch.where(n != 0, inc + 2 * n * agm_k(m), inc)


def jacobi_am(u, m, steps=10):
    """Amplitude am(u|m), 0 < m < 1, by the AGM descent (DLMF 22.20.1-22.20.2)."""
    a = [torch.ones_like(m)]
    b = torch.sqrt(1 - m)
    c = [torch.sqrt(m)]
    for _ in range(steps):
        an = a[-1]
        c.append(0.5 * (an - b))
        a.append(0.5 * (an + b))
        b = torch.sqrt(an * b)
    phi = (2.0 ** steps) * a[-1] * u
    for k in range(steps, 0, -1):
        phi = 0.5 * (phi + torch.asin(c[k] * torch.sin(phi) / a[k]))
    return phi


def cbrt_max_real(z, real_mask):
    """my_cbrt: real cube root for real inputs, else the complex root of largest real part."""
    zr = torch.where(real_mask, z, torch.ones_like(z))
    c0 = torch.exp(torch.log(torch.where(real_mask, torch.ones_like(z), z)) / 3.)
    w = complex(np.cos(2 * PI / 3), np.sin(2 * PI / 3))
    c1, c2 = c0 * w, c0 * np.conj(w)
    re = torch.stack([c0.real, c1.real, c2.real]).detach()
    pick = torch.argmax(re, dim=0)
    cc = torch.where(pick == 0, c0, torch.where(pick == 1, c1, c2))
    rr = zr.real
    real_root = (torch.sign(rr) * torch.abs(rr) ** (1. / 3.)).to(z.dtype)
    return torch.where(real_mask, real_root, cc)


def quartic_roots(a, lam, eta):
    """Radial roots r1..r4 by the reference's resolvent-cubic formula, complex128."""
    A = a ** 2 - eta - lam ** 2
    B = 2 * (eta + (lam - a) ** 2)
    C = -(a ** 2) * eta
    P = -(A ** 2) / 12. - C
    Q = (-A / 3.) * ((A ** 2) / 36. - C) - (B ** 2) / 8.
    disc = (4 * P ** 3 + 27 * Q ** 2).to(torch.complex128)
    sd = torch.sqrt(disc / 108.)
    wp3 = -0.5 * Q + sd
    wm3 = -0.5 * Q - sd
    xi0 = cbrt_max_real(wp3, wp3.imag.detach() == 0) + cbrt_max_real(wm3, wm3.imag.detach() == 0) - A / 3.
    z = torch.sqrt(0.5 * xi0)
    base = -0.5 * A - z * z
    s_lo = torch.sqrt(base + 0.25 * B / z)
    s_hi = torch.sqrt(base - 0.25 * B / z)
    return -z - s_lo, -z + s_lo, z - s_hi, z + s_hi


def radial_r(r_o, r1, r2, r3, r4, tau, case):
    """r(tau) of kgeo/kerr_raytracing_ana.py:404-595 (cases 4, 3, 2) for the rays of one case."""
    if case == 4:
        a1, b1, a2, b2 = r4.imag, r4.real, r2.imag, r2.real
        CC = torch.sqrt((a1 - a2) ** 2 + (b1 - b2) ** 2)
        DD = torch.sqrt((a1 + a2) ** 2 + (b1 - b2) ** 2)
        k4 = (4 * CC * DD) / ((CC + DD) ** 2)
        g0 = torch.sqrt((4 * a2 ** 2 - (CC - DD) ** 2) / ((CC + DD) ** 2 - 4 * a2 ** 2))
        aux = torch.atan((r_o + b1) / a2) + torch.atan(g0)
        pref = 2. / (CC + DD)
        X = (1. / pref) * (-tau + pref * ellip_f(aux, k4))
        am = jacobi_am(X, k4)
        sc = torch.tan(am)
        return -a2 * (g0 - sc) / (1 + g0 * sc) - b1
    if case == 3:
        a1, b1, rr1, rr2 = r4.imag, r4.real, r1.real, r2.real
        rr21 = rr2 - rr1
        AA = torch.sqrt(a1 ** 2 + (b1 - rr2) ** 2)
        BB = torch.sqrt(a1 ** 2 + (b1 - rr1) ** 2)
        k3 = ((AA + BB) ** 2 - rr21 ** 2) / (4 * AA * BB)
        x_o = (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2))
        pref = 1. / torch.sqrt(AA * BB)
        X = (1. / pref) * (-tau + pref * ellip_f(torch.acos(x_o), k3))
        cn = torch.cos(jacobi_am(X, k3))
        return ((BB * rr2 - AA * rr1) + (BB * rr2 + AA * rr1) * cn) / ((BB - AA) + (BB + AA) * cn)
    rr1, rr2, rr3, rr4 = r1.real, r2.real, r3.real, r4.real
    rr31, rr32, rr41, rr42 = rr3 - rr1, rr3 - rr2, rr4 - rr1, rr4 - rr2
    k2 = (rr32 * rr41) / (rr31 * rr42)
    x_o = torch.sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)))
    X = 0.5 * torch.sqrt(rr31 * rr42) * (-tau + 2 * ellip_f(torch.asin(x_o), k2) / torch.sqrt(rr31 * rr42))
    sn = torch.sin(jacobi_am(X, k2))
    return (rr4 * rr31 - rr3 * rr41 * sn ** 2) / (rr31 - rr41 * sn ** 2)


def r_isco(a, s):
    z1 = 1 + torch.pow(1 - a ** 2, 1. / 3.) * (torch.pow(1 + a, 1. / 3.) + torch.pow(1 - a, 1. / 3.))
    z2 = torch.sqrt(3 * a ** 2 + z1 ** 2)
    return 3 + z2 - s * torch.sqrt((3 - z1) * (3 + z1 + 2 * z2))


def u_infall(a, r):
    Delta = r ** 2 + a ** 2 - 2 * r
    Xi = (r ** 2 + a ** 2) ** 2 - Delta * a ** 2
    return Xi / (r ** 2 * Delta), -torch.sqrt(2 * r * (r ** 2 + a ** 2)) / r ** 2, 2 * a / (r * Delta)


def u_subkep(a, r, fac, retro):
    s = -1. if retro else 1.
    ri = r_isco(a, s)
    spin = torch.abs(a)
    asign = torch.sign(a).detach()
    out = (r >= ri).detach()
    Delta = r ** 2 - 2 * r + a ** 2
    Xi = (r ** 2 + a ** 2) ** 2 - Delta * a ** 2
    rr = torch.where(out, r, ri + 1.0)  # keep the unused branch finite
    ell = fac * asign * s * (rr ** 2 + spin ** 2 - s * 2 * spin * torch.sqrt(rr)) / (rr ** 1.5 - 2 * torch.sqrt(rr) + s * spin)
    Do = rr ** 2 - 2 * rr + a ** 2
    Xo = (rr ** 2 + a ** 2) ** 2 - Do * a ** 2
    gam = torch.sqrt(Do / (Xo / rr ** 2 - 4 * a * ell / rr - (1 - 2 / rr) * ell ** 2))
    H = (2 * rr - a * ell) / Do
    chi = 1 / (1 + (2 / rr) * (1 + H))
    Om = (chi / rr ** 2) * (ell + a * H)
    u0_o, u3_o = gam / chi, (gam / chi) * Om
    Delta_i = ri ** 2 - 2 * ri + a ** 2
    Xi_i = (ri ** 2 + a ** 2) ** 2 - Delta_i * a ** 2
    ell_i = fac * asign * s * (ri ** 2 + spin ** 2 - s * 2 * spin * torch.sqrt(ri)) / (ri ** 1.5 - 2 * torch.sqrt(ri) + s * spin)
    gam_i = torch.sqrt(Delta_i / (Xi_i / ri ** 2 - 4 * a * ell_i / ri - (1 - 2 / ri) * ell_i ** 2))
    ri_r = torch.where(out, ri - 0.5, r)
    Dl = ri_r ** 2 - 2 * ri_r + a ** 2
    Xl = (ri_r ** 2 + a ** 2) ** 2 - Dl * a ** 2
    H = (2 * ri_r - a * ell_i) / Dl
    chi = 1 / (1 + (2 / ri_r) * (1 + H))
    Om = (chi / ri_r ** 2) * (ell_i + a * H)
    nu = (ri_r / Dl) * torch.sqrt(Xl / ri_r ** 2 - 4 * a * ell_i / ri_r - (1 - 2 / ri_r) * ell_i ** 2 - Dl / gam_i ** 2)
    u0 = torch.where(out, u0_o, gam_i / chi)
    u1 = torch.where(out, torch.zeros_like(r), -gam_i * (Dl / ri_r ** 2) * nu)
    u3 = torch.where(out, u3_o, (gam_i / chi) * Om)
    return u0, u1, u3


def u_general(a, r, fac, beta_phi, beta_r, retro):
    Delta = r ** 2 + a ** 2 - 2 * r
    u0i, u1i, u3i = u_infall(a, r)
    u0s, u1s, u3s = u_subkep(a, r, fac, retro)
    Om_i, Om_s = u3i / u0i, u3s / u0s
    u1 = u1s + (1 - beta_r) * (u1i - u1s)
    Om = Om_s + (1 - beta_phi) * (Om_i - Om_s)
    u0 = torch.sqrt(1 + r ** 2 * u1 ** 2 / Delta) / torch.sqrt(1 - (r ** 2 + a ** 2) * Om ** 2 - (2 / r) * (1 - a * Om) ** 2)
    return u0, u1, u0 * Om


def image(params, r_o, alpha, beta, mbar_max, retrograde=False, specind=1., sinthb=np.pi / 4, geo=None):
    """I (npix, mbar_max + 1) for a 'bpl' emissivity and 'general' velocity; params = (a, th_o,
    p1, p2, fac_subkep, beta_phi, beta_r) (torch float64, requires_grad as wanted).

    geo: the piecewise-constant decisions from the numpy oracle (dict with per order m the
    lit mask 'lit%d' and radial sign 'kr%d', and the per-pixel radial case 'case')."""
    a, th_o, p1, p2, fac, bphi, br = params
    npix = len(alpha)
    # only pixels lit in some order enter the graph: elementwise backward passes through
    # NaN-valued intermediates of dark pixels (vortical rays) would turn zero gradients into NaN
    any_lit = np.zeros(npix, dtype=bool)
    for mbar in range(mbar_max + 1):
        any_lit |= np.asarray(geo['lit%d' % mbar])
    idx = torch.from_numpy(np.nonzero(any_lit)[0])
    alpha = torch.as_tensor(np.asarray(alpha)[any_lit], dtype=torch.float64)
    beta = torch.as_tensor(np.asarray(beta)[any_lit], dtype=torch.float64)
    lam = -alpha * torch.sin(th_o)
    cos2 = torch.cos(th_o) ** 2
    eta = (alpha ** 2 - a ** 2) * cos2 + beta ** 2
    half = 0.5 * (1 - (eta + lam ** 2) / a ** 2)
    root = torch.sqrt(half ** 2 + eta / a ** 2)
    up, um = half + root, half - root
    up = torch.where((cos2 - up).detach() > 0, cos2 * torch.ones_like(up), up)
    ratio = up / um
    a2um = a ** 2 * um
    F0 = ellip_f(torch.asin(torch.cos(th_o) / torch.sqrt(up)), ratio)
    K = ellip_f(PI / 2 * torch.ones_like(ratio), ratio)
    sqa = torch.sqrt(-a2um)
    r1, r2, r3, r4 = quartic_roots(a, lam, eta)
    rh = 1 + torch.sqrt(1 - a ** 2)
    north = float(th_o.detach()) < PI / 2
    out = []
    for mbar in range(mbar_max + 1):
        lit = torch.as_tensor(np.asarray(geo['lit%d' % mbar])[any_lit])
        kr = torch.as_tensor(np.asarray(geo['kr%d' % mbar])[any_lit], dtype=torch.float64)
        if north:
            m = mbar + (beta > 0).double()
            ir = torch.where(beta <= 0, (2 * m * K + F0) / sqa, (2 * m * K - F0) / sqa)
        else:
            m = mbar + (-beta > 0).double()
            ir = torch.where(beta >= 0, (2 * m * K - F0) / sqa, (2 * m * K + F0) / sqa)
        rs = torch.zeros_like(alpha)
        case = torch.as_tensor(np.asarray(geo['case'])[any_lit])
        for c in (2, 3, 4):
            sel = lit & (case == c)
            if bool(sel.any()):
                rs = rs.index_put((sel,), radial_r(r_o, r1[sel], r2[sel], r3[sel], r4[sel], ir[sel], c))
        I = torch.zeros_like(alpha)
        if bool(lit.any()):
            r = rs[lit]
            u0, u1, u3 = u_general(a, r, fac, bphi, br, retrograde)
            l, e = lam[lit], eta[lit]
            Delta = r ** 2 - 2 * r + a ** 2
            R = (r ** 2 + a ** 2 - a * l) ** 2 - Delta * (e + (l - a) ** 2)
            g = 1 / (u0 - l * u3 - kr[lit] * u1 * torch.sqrt(R) / Delta)
            x = torch.log(r / rh)
            j = torch.exp(p1 * x + p2 * x ** 2) * g ** specind * sinthb ** (1 + specind)
            I = I.index_put((lit,), g ** 2 * j)
        out.append(I)
    full = torch.zeros((npix, mbar_max + 1), dtype=torch.float64)
    return full.index_put((idx,), torch.stack(out, dim=1))


def geometry(ko, a, r_o, th_o, alpha, beta, mbar_max, emis, vel):
    """The piecewise-constant decisions for image(), from the numpy oracle ko."""
    o = ko.make_image_px(a, r_o, th_o, mbar_max, alpha, beta, emis=emis, vel=vel)
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    r1, r2, r3, r4, _ = ko.quartic_roots(a, lam, eta)
    case = np.where(np.imag(r1) != 0, 4, np.where(np.imag(r3) != 0, 3, 2))
    outside = ko.outside_critical(a, th_o, alpha, beta).astype(bool)
    tau_tot = ko.mino_total(a, r_o, eta, r1, r2, r3, r4)
    geo = {'case': case}
    for m in range(mbar_max + 1):
        lit = o['sinthb'][:, m] > 0
        geo['lit%d' % m] = lit
        Ir = o['t'][:, m]
        geo['kr%d' % m] = np.where(~outside | (Ir <= 0.5 * tau_tot), 1., -1.)
    return geo, o
