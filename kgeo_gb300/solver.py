"""Drop-in for kgeo.solver: crossings of null geodesics with a jet field line
psi(r, theta) = psi_target, on the GPU.

kgeo/solver.py:14-207. The stream functions and getneq keep the reference's numpy form (small
helpers); get_maxtau_forwardjet, getguesses and findroot run in the CUDA kernels behind
kgeo_jet_guesses / kgeo_jet_findroot (include/kgeo_gb300.h): one thread scans each pixel's
samples for Mino-time guesses, one thread iterates each (guess, pixel) pair with the secant
steps of scipy.optimize.newton on the tracer's direct theta / r evaluators.
"""
import ctypes

import numpy as np
import scipy.special as sp
import torch

from . import _lib
from . import device as _dev
from .kerr_raytracing_utils import EP, MINSPIN

MAXTAUFRAC = (1. - 1.e-10)


def psi_BZ_para(r, theta, a):
    """psi of the BZ paraboloid (kgeo/solver.py:15-18)."""
    abscth = np.abs(np.cos(theta))
    rp = 1 + np.sqrt(1 - a ** 2)
    return r * (1 - abscth) + rp * (1 + abscth) * (1 - np.log(1 + abscth)) - 2 * rp * (1 - np.log(2))


def psi_BZ_mono(theta):
    """psi of the BZ monopole (kgeo/solver.py:21-22)."""
    return 1 - np.abs(np.cos(theta))


def psi_power(r, theta, pval):
    """psi = r^p (1 - |cos theta|) (kgeo/solver.py:25-26)."""
    return r ** pval * (1 - np.abs(np.cos(theta)))


def psifunc(r, theta, a, model='para', pval=1):
    """kgeo/solver.py:29-37."""
    if model == 'para':
        return psi_BZ_para(r, theta, a)
    elif model == 'mono':
        return psi_BZ_mono(theta)
    elif model == 'power':
        return psi_power(r, theta, pval)
    else:
        return 0


def getneq(a, tau, u_minus, u_plus, th_s, th_o, signptheta, betas):
    """Equatorial crossings before Mino time tau (kgeo/solver.py:40-55)."""
    uratio = u_plus / u_minus
    xFarg = np.cos(th_o) / np.sqrt(u_plus)
    F0 = sp.ellipkinc(np.arcsin(xFarg), uratio)
    K = sp.ellipkinc(0.5 * np.pi, uratio)
    mval = (np.sqrt(-u_minus * a ** 2) * tau + np.sign(betas) * F0) / (2 * K)
    mbarval = mval - np.heaviside(betas, 0)
    return np.ceil(np.nan_to_num(mbarval))


def makegoodarray(arr):
    """Ragged guesses to a (max length, n) array padded with -1 (kgeo/solver.py:89-95)."""
    max_length = max(len(a) for a in arr)
    result = -np.ones((len(arr), max_length))
    for i, a in enumerate(arr):
        result[i, :len(a)] = a
    return np.transpose(np.copy(result))


def _field(model, psitarget, pval):
    if model not in _lib.JET:
        raise NotImplementedError("jet model %r is not on the GPU path" % (model,))
    return _lib.JetField(_lib.JET[model], 0, float(psitarget), float(pval))


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _guesses_device(a, r_o, th_o, alpha, beta, r, th, mino, psitarget, neqmax, model, pval, taumax_only=False):
    _dev.require_cuda()
    lib = _lib.load()
    al, be = _dev.as_device(alpha), _dev.as_device(beta)
    npix = al.numel()
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    fld = _field(model if model in _lib.JET else 'para', psitarget, pval)
    nq = -1 if neqmax is None else int(neqmax)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    tmax = torch.empty(npix, dtype=torch.float64, device=al.device)
    if taumax_only:
        _lib.check(lib.kgeo_jet_guesses(ctypes.byref(ob), _p(al), _p(be), npix, None, None, None, 0,
                                        ctypes.byref(fld), nq, _p(tmax), None, None, 0, s))
        return tmax
    r, th, mino = _dev.as_device(r), _dev.as_device(th), _dev.as_device(mino)
    ngeo = r.shape[0]
    count = torch.empty(npix, dtype=torch.int32, device=al.device)
    _lib.check(lib.kgeo_jet_guesses(ctypes.byref(ob), _p(al), _p(be), npix, _p(r), _p(th), _p(mino), ngeo,
                                    ctypes.byref(fld), nq, None, _p(count), None, 0, s))
    G = int(count.max()) if npix else 1
    g = torch.empty((G, npix), dtype=torch.float64, device=al.device)
    _lib.check(lib.kgeo_jet_guesses(ctypes.byref(ob), _p(al), _p(be), npix, _p(r), _p(th), _p(mino), ngeo,
                                    ctypes.byref(fld), nq, None, None, _p(g), G, s))
    return g


def get_maxtau_forwardjet(a, r_o, th_o, alpha, beta, neqmax=1):
    """Mino-time bound of the crossing search (kgeo/solver.py:57-87)."""
    return _guesses_device(a, r_o, th_o, alpha, beta, None, None, None, 0.0, neqmax, 'para', 1,
                           taumax_only=True).cpu().numpy()


def getguesses(outgeo, a, rout, inc, alphas, betas, psitarget, ngeo, neqmax=1, model='para', pval=1):
    """(guesses, npix) Mino-time guesses padded with -1 (kgeo/solver.py:97-134). outgeo: a
    Geodesics (numpy or CUDA arrays)."""
    if model not in _lib.JET:
        raise NotImplementedError("jet model %r is not on the GPU path" % (model,))
    g = _guesses_device(a, rout, inc, alphas, betas, outgeo.r_s, outgeo.th_s, outgeo.mino_times, psitarget, neqmax,
                        model, pval)
    return g.cpu().numpy()


def findroot_device(a, r_o, th_o, alpha, beta, guesses, psitarget, model='para', tol=1e-8, pval=1, maxiter=500):
    """kgeo_jet_findroot on CUDA tensors: dict of (nguess, npix) tensors tau, r, th, signpr,
    signpth, neq, status."""
    _dev.require_cuda()
    lib = _lib.load()
    al, be = _dev.as_device(alpha), _dev.as_device(beta)
    g = _dev.as_device(guesses)
    npix = al.numel()
    G = g.shape[0] if g.ndim == 2 else 1
    out = {k: torch.empty((G, npix), dtype=torch.float64, device=al.device)
           for k in ('tau', 'r', 'th', 'signpr', 'signpth', 'neq')}
    out['status'] = torch.empty((G, npix), dtype=torch.int32, device=al.device)
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    fld = _field(model, psitarget, pval)
    _lib.check(lib.kgeo_jet_findroot(ctypes.byref(ob), _p(al), _p(be), npix, _p(g), G, ctypes.byref(fld), float(tol),
                                     int(maxiter), None, 0, *[_p(out[k]) for k in
                                                               ('tau', 'r', 'th', 'signpr', 'signpth', 'neq',
                                                                'status')],
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def crossings_device(a, r_o, th_o, alpha, beta, r, th, mino, psitarget, model='para', neqmax=1, tol=1e-8, pval=1):
    """findroot's crossings on CUDA tensors: (dict of (nguess, npix) tensors tau, r, th, signpr,
    signpth, neq, status; the guesses' shape). r, th, mino: the (ngeo, npix) samples. Warns as
    scipy does when some guesses did not converge and raises when none did."""
    if model not in _lib.JET:
        raise NotImplementedError("jet model %r is not on the GPU path" % (model,))
    if np.abs(a) < MINSPIN:
        al = alpha.cpu().numpy() if isinstance(alpha, torch.Tensor) else np.asarray(alpha)
        be = beta.cpu().numpy() if isinstance(beta, torch.Tensor) else np.asarray(beta)
        eta = (al ** 2 - a ** 2) * np.cos(th_o) ** 2 + be ** 2
        if np.any(eta < 0):
            print("WARNING: there were eta<0 points for spin %f<MINSPIN!" % a)
    g = _guesses_device(a, r_o, th_o, alpha, beta, r, th, mino, psitarget, neqmax, model, pval)
    shape = tuple(g.shape)
    out = findroot_device(a, r_o, th_o, alpha, beta, g, psitarget, model=model, tol=tol, pval=pval)
    st = out['status']
    if bool((st != 0).any()):
        import warnings
        msg = '%s failed to converge after %d iterations' % ('all' if bool((st != 0).all()) else 'some', 500)
        if bool((st != 0).all()):
            raise RuntimeError(msg)
        warnings.warn(msg, RuntimeWarning, stacklevel=3)
    return out, shape


def findroot(outgeo, psitarget, alpha, beta, r_o, th_o, a, ngeo, model='para', neqmax=1, tol=1e-8, pval=1):
    """(tau, r_s, th_s, sign p_r, sign p_theta, neq, guesses_shape) of every crossing of the
    geodesics with psi = psi_target (kgeo/solver.py:136-207); arrays flattened guess-major like
    the reference's. Warns as scipy does when some guesses did not converge and raises when
    none did."""
    out, shape = crossings_device(a, r_o, th_o, alpha, beta, outgeo.r_s, outgeo.th_s, outgeo.mino_times, psitarget,
                                  model=model, neqmax=neqmax, tol=tol, pval=pval)
    res = _dev.to_host([out[k].reshape(-1) for k in ('tau', 'r', 'th', 'signpr', 'signpth', 'neq')])
    return tuple(res) + (shape,)


__all__ = ['psi_BZ_para', 'psi_BZ_mono', 'psi_power', 'psifunc', 'getneq', 'get_maxtau_forwardjet', 'makegoodarray',
           'getguesses', 'findroot', 'findroot_device', 'crossings_device', 'EP']
