"""Drop-in for kgeo.equatorial_lensing (source radius of the m-th equatorial crossing)
and the per-pixel crossing counts of kgeo.kerr_raytracing_utils, on the GPU.

r_equatorial: kgeo/equatorial_lensing.py:85-196; nmax_equatorial / nmax_poloidal:
:22-82; n_equatorial_crossings / n_poloidal_orbits / is_outside_crit:
kgeo/kerr_raytracing_utils.py:551-684, 794-826. Same signatures, checks and outputs;
the work runs in the CUDA kernels behind the C ABI (include/kgeo_gb300.h).
"""
import ctypes

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
    """Parametrised critical curve (alpha, beta), 2 x (valid points) long.

    GL19b eqs. 38-40 as kgeo/equatorial_lensing.py:264-293 evaluates them: photon-orbit radii
    between the retrograde and prograde circular orbits, their conserved quantities, the
    screen coordinates, NaN points dropped, the lower half mirrored. Host-side numpy: it is a
    closed form evaluated once per image, not part of the traced path.
    """
    rminus = 2 * (1 + np.cos(2. * np.arccos(-a) / 3.))
    rplus = 2 * (1 + np.cos(2. * np.arccos(a) / 3.))
    r = np.linspace(rminus, rplus, n)
    lam = -(r ** 3 + a ** 2 + r * (a ** 2) - 3 * r ** 2) / (a * r - a)
    eta = (r ** 2) * (3 * r ** 2 + a ** 2 - lam ** 2) / (r ** 2 - a ** 2)
    with np.errstate(invalid='ignore'):
        alpha = -lam / np.sin(th0)
        beta = np.sqrt(eta + (a * np.cos(th0)) ** 2 - (lam / np.tan(th0)) ** 2)
    bad = np.isnan(alpha) + np.isnan(beta)
    alpha = alpha[~bad]
    beta = beta[~bad]
    return np.hstack((alpha, np.flip(alpha))), np.hstack((beta, -np.flip(beta)))


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
