"""Drop-in for kgeo.equatorial_lensing (source radius of the m-th equatorial crossing)
and the per-pixel crossing counts of kgeo.kerr_raytracing_utils, on the GPU.

r_equatorial: kgeo/equatorial_lensing.py:85-196; nmax_equatorial / nmax_poloidal:
:22-82; n_equatorial_crossings / n_poloidal_orbits / is_outside_crit:
kgeo/kerr_raytracing_utils.py:551-684, 794-826. Same signatures, checks and outputs;
the work runs in the CUDA kernels behind the C ABI (include/kgeo_gb300.h).
"""
import ctypes
import os

import numpy as np
import torch

from . import _lib
from . import device as _dev


def _check(a, r_o=None, th_o=None):
    if not (isinstance(a, float) and (0 <= np.abs(a) < 1)):
        raise Exception("|a| should be a float in range [0,1)")
    if r_o is not None and not (isinstance(r_o, float) and (r_o >= 100)):
        raise Exception("r_o should be a float > 100")
    if th_o is not None and not (isinstance(th_o, float) and (0 < th_o < np.pi) and th_o != 0.5 * np.pi):
        raise Exception("th_o should be a float in range (0,pi/2) or (pi/2,pi)")


def _pixels(alpha, beta):
    if not isinstance(alpha, (np.ndarray, torch.Tensor)):
        alpha = np.array([alpha]).flatten()
    if not isinstance(beta, (np.ndarray, torch.Tensor)):
        beta = np.array([beta]).flatten()
    if len(alpha) != len(beta):
        raise Exception("alpha, beta are different lengths!")
    return alpha, beta


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def r_equatorial_device(a, r_o, th_o, mbars, alpha, beta, stream=None):
    """r_s, Ir (len(mbars), npix), Imax, Nmax (npix) as CUDA tensors for consecutive orders mbars."""
    _dev.require_cuda()
    lib = _lib.load()
    mbars = list(mbars)
    lo, n = (mbars[0], len(mbars)) if mbars else (0, 0)
    assert mbars == list(range(lo, lo + n)), 'orders must be consecutive'
    npix = alpha.numel()
    dev = alpha.device
    r_s = torch.empty((n, npix), dtype=torch.float64, device=dev)
    Ir = torch.empty((n, npix), dtype=torch.float64, device=dev)
    Imax = torch.empty(npix, dtype=torch.float64, device=dev)
    Nmax = torch.empty(npix, dtype=torch.float64, device=dev)
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.check(lib.kgeo_r_equatorial(ctypes.byref(ob), lo, n, _p(alpha), _p(beta), npix, _p(r_s), _p(Ir),
                                     _p(Imax), _p(Nmax), ctypes.c_void_p(s.cuda_stream)))
    return r_s, Ir, Imax, Nmax


def r_equatorial(a, r_o, th_o, mbar, alpha, beta):
    """Return (r_s, Ir, Imax, Nmax) of the mbar-th equatorial crossing (kgeo/equatorial_lensing.py:85)."""
    _check(a, r_o, th_o)
    if not (isinstance(mbar, int) and (mbar >= 0)):
        raise Exception("mbar should be an integer >=0!")
    alpha, beta = _pixels(alpha, beta)
    r_s, Ir, Imax, Nmax = r_equatorial_device(a, r_o, th_o, [mbar], _dev.as_device(alpha), _dev.as_device(beta))
    return tuple(_dev.to_host([r_s[0], Ir[0], Imax, Nmax]))


def _crossings(a, th_o, alpha, beta, tau, want):
    _dev.require_cuda()
    lib = _lib.load()
    al = _dev.as_device(alpha)
    be = _dev.as_device(beta)
    npix = al.numel()
    one = False
    if tau is not None:
        tau = np.asarray(tau, dtype=float) if not isinstance(tau, torch.Tensor) else tau
        if len(tau.shape) == 1:
            tau = tau.reshape(1, tau.shape[0])
            one = True
        if not (tau.shape[1] == npix):
            raise Exception("tau has incompatible shape in n_poloidal_orbits!")
        tt = _dev.as_device(tau)
        ntau = tt.shape[0]
    else:
        tt, ntau = None, 0
    out = {k: (torch.empty((ntau, npix) if k != 'outside' else npix, dtype=torch.float64, device=al.device)
               if k in want else None) for k in ('n_eq', 'n_pol', 'outside')}
    ob = _lib.Observer(float(a), 1.e4, float(th_o))
    s = torch.cuda.current_stream(al.device)
    _lib.check(lib.kgeo_equatorial_crossings(ctypes.byref(ob), _p(al), _p(be), npix, _p(tt), ntau,
                                             _p(out['n_eq']), _p(out['n_pol']), _p(out['outside']),
                                             ctypes.c_void_p(s.cuda_stream)))
    res = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
    if one:
        res = {k: (v[0] if k != 'outside' else v) for k, v in res.items()}
    return res


def n_equatorial_crossings(a, th_o, alpha, beta, tau):
    """kgeo/kerr_raytracing_utils.py:605-684."""
    _check(a)
    alpha, beta = _pixels(alpha, beta)
    return _crossings(a, th_o, alpha, beta, tau, ('n_eq',))['n_eq']


def n_poloidal_orbits(a, th_o, alpha, beta, tau):
    """kgeo/kerr_raytracing_utils.py:551-603."""
    _check(a)
    alpha, beta = _pixels(alpha, beta)
    return _crossings(a, th_o, alpha, beta, tau, ('n_pol',))['n_pol']


def n_angular_turnings(a, th_o, alpha, beta, tau):
    """Fractional number of angular turnings at Mino times tau (ntau, npix) or (npix)
    (kgeo/kerr_raytracing_utils.py:686-792), through kgeo_angular_turnings."""
    _check(a)
    if not (isinstance(th_o, float) and (0 <= th_o <= np.pi / 2.)):
        raise Exception("th_o should be a float in range (0,pi/2]")
    if not isinstance(alpha, np.ndarray):
        alpha = np.array([alpha]).flatten()
    if not isinstance(beta, np.ndarray):
        beta = np.array([beta]).flatten()
    if len(alpha) != len(beta):
        raise Exception("alpha, beta are different lengths!")
    tau = np.asarray(tau, dtype=float) if not isinstance(tau, torch.Tensor) else tau
    one = len(tau.shape) == 1
    if one:
        tau = tau.reshape(1, tau.shape[0])
    if not (tau.shape[1] == len(alpha)):
        raise Exception("tau has incompatible shape in n_poloidal_orbits!")
    _dev.require_cuda()
    lib = _lib.load()
    al, be, tt = _dev.as_device(alpha), _dev.as_device(beta), _dev.as_device(tau)
    out = torch.empty(tuple(tt.shape), dtype=torch.float64, device=al.device)
    ob = _lib.Observer(float(a), 1.e4, float(th_o))
    s = torch.cuda.current_stream(al.device)
    _lib.check(lib.kgeo_angular_turnings(ctypes.byref(ob), _p(al), _p(be), al.numel(), _p(tt), tt.shape[0], _p(out),
                                         ctypes.c_void_p(s.cuda_stream)))
    res = out.cpu().numpy()
    return res[0] if one else res


def equatorial_consistency(a, r_o, th_o, alpha, beta, mbar_max=1, raise_on_failure=True):
    """The consistency check of the reference's scripts/calc_t_equatorial.py:50-71 on the GPU:
    for each order m <= mbar_max, the coordinates of the geodesics at the crossing Mino times
    Ir of r_equatorial must lie on the equator (|1 - theta / (pi/2)| <= 1e-14) at the source
    radius r_s, on every pixel with Nmax >= m.

    The reference evaluates both sides with the same radial code and holds r to 1e-12; here
    r_equatorial's radius and the tracer's radius come from two kernels, so each keeps its own
    rounding, and r(tau) amplifies a Mino-time rounding by d ln r / d ln tau = tau sqrt(R) / r,
    ~ tau r at large r (a crossing at r_s = 1e5 M, met just before the ray escapes): the bound
    on |1 - r / r_s| is max(1e-12, 32 eps tau r_s). Returns {m: (max theta deviation, max r
    deviation, max r deviation / its bound)}; raises as the script does when a bound fails."""
    _check(a, r_o, th_o)
    alpha, beta = _pixels(alpha, beta)
    al, be = _dev.as_device(alpha), _dev.as_device(beta)
    out = {}
    r_s, Ir, Imax, Nmax = r_equatorial_device(a, r_o, th_o, list(range(mbar_max + 1)), al, be)
    rays = _dev.PreparedRays(a, r_o, th_o, al, be)
    eps = np.finfo(float).eps
    for m in range(mbar_max + 1):
        ring = Nmax >= m
        res = rays.samples(rays.alloc(nsamp=1, keys=('r', 'th')), tau=Ir[m:m + 1].contiguous(), do_phi_and_t=True)
        th = res['th'][0][ring]
        r = res['r'][0][ring]
        rs = r_s[m][ring]
        dev_r = torch.abs(1 - r / rs)
        bound = torch.clamp(32 * eps * torch.abs(Ir[m][ring]) * torch.abs(rs), min=1e-12)
        dth = float(torch.max(torch.abs(1 - th / (0.5 * np.pi)))) if th.numel() else 0.0
        dr = float(torch.max(dev_r)) if r.numel() else 0.0
        q = float(torch.max(dev_r / bound)) if r.numel() else 0.0
        out[m] = (dth, dr, q)
        if raise_on_failure and dth > 1.e-14:
            raise Exception("raytrace_ana not finding eqauatorial crossings for mbar=%i!" % m)
        if raise_on_failure and q > 1:
            raise Exception("raytrace_ana not finding consistent r_s for mbar=%i!" % m)
    return out


def is_outside_crit(a, th_o, alpha, beta):
    """kgeo/kerr_raytracing_utils.py:794-826."""
    _check(a)
    if not isinstance(alpha, np.ndarray):
        alpha = np.array([alpha]).flatten()
    if not isinstance(beta, np.ndarray):
        beta = np.array([beta]).flatten()
    if len(alpha) != len(beta):
        raise Exception("alpha, beta are different shapes!")
    return _crossings(a, th_o, alpha, beta, None, ('outside',))['outside']


def nmax_equatorial(a, r_o, th_o, alpha, beta):
    """Maximum number of equatorial crossings (kgeo/equatorial_lensing.py:22-51)."""
    _check(a, r_o, th_o)
    alpha, beta = _pixels(alpha, beta)
    return _imax_counts(a, r_o, th_o, alpha, beta, 'n_eq')


def nmax_poloidal(a, r_o, th_o, alpha, beta):
    """Maximum number of poloidal orbits (kgeo/equatorial_lensing.py:53-82)."""
    _check(a, r_o, th_o)
    alpha, beta = _pixels(alpha, beta)
    return _imax_counts(a, r_o, th_o, alpha, beta, 'n_pol')


def _imax_counts(a, r_o, th_o, alpha, beta, key):
    # the counts at mino_total (eta <= 0 pixels report -2 whatever their total)
    res = _dev.trace(a, r_o, th_o, _dev.as_device(alpha), _dev.as_device(beta), ngeo=1, outputs=(),
                     per_ray=('tau_tot',))
    return _crossings(a, th_o, alpha, beta, res['tau_tot'], (key,))[key]


def critical_curve(a, th0, n=100000):
    """Parametrised critical curve (alpha, beta), 2 x (valid points) long
    (kgeo/equatorial_lensing.py:260-289): the n photon-orbit radii between the retrograde and
    prograde circular orbits, their conserved quantities and screen coordinates (GL19b Eqs
    38-40) from kgeo_critical_curve; the points the reference drops (NaN) are dropped and the
    lower half mirrored."""
    _dev.require_cuda()
    lib = _lib.load()
    al = torch.empty(int(n), dtype=torch.float64, device='cuda')
    be = torch.empty(int(n), dtype=torch.float64, device='cuda')
    s = torch.cuda.current_stream()
    _lib.check(lib.kgeo_critical_curve(float(a), float(th0), int(n), _p(al), _p(be), ctypes.c_void_p(s.cuda_stream)))
    keep = ~(torch.isnan(al) | torch.isnan(be))
    al, be = al[keep], be[keep]
    alpha, beta = _dev.to_host([torch.cat((al, torch.flip(al, (0,)))), torch.cat((be, -torch.flip(be, (0,))))])
    return alpha, beta


# ---------------------------------------------------------------------------
# lensed curves of constant equatorial radius (kgeo/equatorial_lensing.py:198-423)
# ---------------------------------------------------------------------------

INF = 1.e50
R0 = np.inf
BRENTQ_XTOL = 2e-12
BRENTQ_RTOL = 4 * np.finfo(float).eps
BRENTQ_MAXITER = 100


def rho_bracket(mbar, req):
    """rho_of_req's bracket, "eyeballed from Gralla+Lupsasca Fig 6" (kgeo/equatorial_lensing.py:227-236)."""
    if mbar == 0:
        return 0, req + 5
    if mbar == 1:
        return 0, 100
    return 1, 10


def rho_of_req_device(curves, varphis, xtol=BRENTQ_XTOL, rtol=BRENTQ_RTOL, maxiter=BRENTQ_MAXITER, stream=None):
    """kgeo_rho_of_req for many curves at once. curves: iterable of (a, th0, r_eq, mbar) or
    (a, th0, r_eq, mbar, rho_min, rho_max); varphis: angles (numpy or CUDA tensor). Returns
    (rho, status) CUDA tensors (ncurves, nphi)."""
    _dev.require_cuda()
    lib = _lib.load()
    curves = list(curves)
    arr = (_lib.Curve * max(1, len(curves)))()
    for i, c in enumerate(curves):
        a, th0, req, mbar = c[:4]
        lo, hi = (c[4], c[5]) if len(c) > 4 else rho_bracket(mbar, req)
        arr[i] = _lib.Curve(float(a), float(th0), float(req), float(lo), float(hi), int(mbar), 0)
    vp = _dev.as_device(varphis)
    nphi = vp.numel()
    rho = torch.empty((len(curves), nphi), dtype=torch.float64, device=vp.device)
    st = torch.zeros((len(curves), nphi), dtype=torch.int32, device=vp.device)
    s = stream if stream is not None else torch.cuda.current_stream(vp.device)
    _lib.check(lib.kgeo_rho_of_req(arr, len(curves), _p(vp), nphi, float(xtol), float(rtol), int(maxiter), _p(rho),
                                   _p(st), ctypes.c_void_p(s.cuda_stream)))
    return rho, st


def _raise_status(st):
    if (st == 1).any():
        raise ValueError("f(a) and f(b) must have different signs")
    if (st == 2).any():
        raise RuntimeError("Failed to converge after %d iterations" % BRENTQ_MAXITER)


def rho_of_req(a, th0, req, mbar=0, varphis=None):
    """(varphis, rhos, alphas, betas) of the curve of equatorial radius req for image order
    mbar (kgeo/equatorial_lensing.py:223-243): at every angle the root of objfunc on the
    reference's bracket, all angles in one kernel launch."""
    if varphis is None:
        varphis = np.linspace(-180, 179, 360) * np.pi / 180.
    varphis = np.asarray(varphis, dtype=float)
    rho, st = rho_of_req_device([(a, th0, req, mbar)], varphis)
    rho, st = _dev.to_host([rho[0], st[0]])
    _raise_status(st)
    return varphis, rho, np.cos(varphis) * rho, np.sin(varphis) * rho


def rho_of_req_single(a, th0, req, varphi, mbar=0):
    """rho at one angle (kgeo/equatorial_lensing.py:245-258)."""
    return float(rho_of_req(a, th0, req, mbar=mbar, varphis=np.array([varphi]))[1][0])


def r_equatorial2(rho, varphi, a, th0, mbar=0):
    """r_s at (rho, varphi) for r_o = inf, INF / 1 where there is no crossing outside / inside
    the critical curve (kgeo/equatorial_lensing.py:198-216)."""
    alpha = np.array([np.cos(varphi) * rho])
    beta = np.array([np.sin(varphi) * rho])
    r = r_equatorial(a, R0, th0, mbar, alpha, beta)[0][0]
    outside = is_outside_crit(a, th0, alpha, beta)[0]
    if r <= 0 and outside == 1:
        r = INF
    elif r <= 0:
        r = 1
    return r


def objfunc(rho, varphi, a, th0, r_target, mbar=0):
    """r_equatorial2 - r_target (kgeo/equatorial_lensing.py:218-221)."""
    return r_equatorial2(rho, varphi, a, th0, mbar=mbar) - r_target


LIBRARY_RADII = {'r10': 10., 'r100': 100., 'r1000': 1000., 'r10000': 10000.}


def _library_file(outpath, spin, inc, which):
    return '%s/a%02.0f_i%02.0f_%s.txt' % (outpath, 100 * spin, inc, which)


def make_library(spins, incs, which='rh', mmax=5, outpath=None, varphis=None):
    """The curve library of generate_library / make_curves2 (kgeo/equatorial_lensing.py:
    327-423) for every (spin, inclination) pair: rho(varphi) of the curves of equatorial radius
    r_h (which='rh') or 10, 100, 1000, 10000 for orders 0..mmax, all (spin, inc, order, angle)
    roots in one kernel launch. Returns {(spin, inc): (nphi, mmax + 2) array of varphi and the
    rho columns}, leaving out a pair whose solve fails at any angle (the reference skips its
    file). With outpath, writes each pair's table as make_curves2 does (np.savetxt,
    'a%02.0f_i%02.0f_<which>.txt'), skipping files that exist."""
    if which != 'rh' and which not in LIBRARY_RADII:
        raise Exception()
    if varphis is None:
        varphis = np.linspace(-180, 179, 360) * np.pi / 180.
    varphis = np.asarray(varphis, dtype=float)
    pairs = [(float(sp), float(inc)) for sp, inc in zip(np.ravel(spins), np.ravel(incs))]
    if outpath is not None:
        pairs = [p for p in pairs if not os.path.isfile(_library_file(outpath, p[0], p[1], which))]
    curves = []
    for sp, inc in pairs:
        req = 1 + np.sqrt(1 - sp ** 2) if which == 'rh' else LIBRARY_RADII[which]
        for m in range(mmax + 1):
            curves.append((sp, inc * np.pi / 180., req, m))
    out = {}
    if not curves:
        return out
    rho, st = rho_of_req_device(curves, varphis)
    rho, st = _dev.to_host([rho, st])
    rho = rho.reshape(len(pairs), mmax + 1, -1)
    ok = (st.reshape(len(pairs), mmax + 1, -1) == 0).all(axis=(1, 2))
    for k, (sp, inc) in enumerate(pairs):
        if not ok[k]:
            continue
        tab = np.hstack((varphis.reshape(-1, 1), rho[k].T))
        out[(sp, inc)] = tab
        if outpath is not None:
            np.savetxt(_library_file(outpath, sp, inc, which), tab)
    return out


def make_curves2(i, which, n, spin, inc, mmax, outpath):
    """One library file (kgeo/equatorial_lensing.py:362-418); the progress counter of the
    reference's process pool is not kept."""
    make_library([spin], [inc], which=which, mmax=mmax, outpath=outpath)


def generate_library(which='rh', outpath=None, spins=None, incs=None, mmax=5):
    """generate_library (kgeo/equatorial_lensing.py:327-357): spins 0.01..0.99 (99) x
    inclinations 1..89 deg (89) x orders 0..mmax, 360 angles each, written to
    './curve_library_<which>' (created if missing), in one kernel launch instead of a
    process pool."""
    if outpath is None:
        outpath = './curve_library_' + which
    if spins is None:
        spins = np.linspace(0.01, 0.99, 99)
    if incs is None:
        incs = np.linspace(1, 89, 89)
    allincs, allspins = np.meshgrid(incs, spins)
    os.makedirs(outpath, exist_ok=True)
    return make_library(allspins.flatten(), allincs.flatten(), which=which, mmax=mmax, outpath=outpath)


def critical_band(a, th0, n_angles=4096, n_radii=256, half_width=0.05, n_curve=100000):
    """Polar band of pixels around the critical curve: n_radii offsets in
    [-half_width, half_width] M around the curve's radius at n_angles screen angles."""
    al, be = critical_curve(a, th0, n_curve)
    ang = np.arctan2(be, al)
    rad = np.hypot(al, be)
    order = np.argsort(ang)
    ang, rad = ang[order], rad[order]
    phis = np.linspace(-np.pi, np.pi, n_angles, endpoint=False)
    rc = np.interp(phis, ang, rad, period=2 * np.pi)
    offs = np.linspace(-half_width, half_width, n_radii)
    R = rc[None, :] + offs[:, None]
    return (R * np.cos(phis)[None, :]).flatten(), (R * np.sin(phis)[None, :]).flatten()
