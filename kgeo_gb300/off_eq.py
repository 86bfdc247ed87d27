"""Drop-in for kgeo.off_eq: polarised images of the emission along a jet field line, on the GPU.

kgeo/off_eq.py:124-233 (getstokes) for the monopole field-line model ('mono', and 'power'
with p = 0, whose density is the monopole's): the geodesics (kgeo_raytrace), their crossings
with the field line (kgeo_jet_guesses, kgeo_jet_findroot) and the emission of every crossing
summed into the per-subring images (kgeo_jet_stokes, include/kgeo_gb300.h) stay on the device;
only the images come back to the host.

The reference's paraboloid ('para') and p > 0 power models compute their densities with
scipy.integrate.quad over array bounds (kgeo/densityfuncs.py) and fail before any image is
made with the numpy and scipy of this build; they, the Lorentz-factor cap (gammamax) and the
per-crossing sin(theta_B) (retsin) raise NotImplementedError.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import device as _dev
from . import solver as _solver
from .kerr_raytracing_ana import _check_args, _flags_check, _pixels

SPECIND = 1  # kgeo/off_eq.py:13


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _supported(model, pval, gammamax, retsin, nu_parallel):
    if not (model == 'mono' or (model == 'power' and pval == 0)):
        raise NotImplementedError("getstokes of model %r (pval %r) is not on the GPU path: only the monopole "
                                  "field-line models ('mono', 'power' with pval=0) are" % (model, pval))
    if gammamax is not None:
        raise NotImplementedError("the drift-frame Lorentz-factor cap (gammamax) is not on the GPU path")
    if retsin:
        raise NotImplementedError("retsin is not on the GPU path")
    if isinstance(nu_parallel, str):
        raise NotImplementedError("nu_parallel=%r is not on the GPU path: give a number in [-1, 1]" % nu_parallel)
    if not (-1 <= nu_parallel <= 1):
        raise Exception("nu_parallel should be in the range (-1,1)")


def stokes_device(a, r_o, th_o, alpha, beta, crossings, neqmax=1, model='mono', pval=0, nu_parallel=0, sigma=2,
                  specind=SPECIND, per_crossing=False):
    """kgeo_jet_stokes on CUDA tensors. crossings: kgeo_jet_findroot's outputs (a dict with r,
    th, signpr, signpth, neq of shape (nguess, npix)). Returns a dict of CUDA tensors: I, Q, U,
    evpa of shape (neqmax + 1, npix) (subrings neq = 0 .. neqmax - 1, then the total),
    stagnation (r0, Omega_F), and with per_crossing the (nguess, npix) Ic, Qc, Uc."""
    _dev.require_cuda()
    lib = _lib.load()
    al, be = _dev.as_device(alpha), _dev.as_device(beta)
    npix = al.numel()
    cr = {k: _dev.as_device(crossings[k]).contiguous() for k in ('r', 'th', 'signpr', 'signpth', 'neq')}
    G = cr['r'].shape[0] if cr['r'].ndim == 2 else 1
    dev = al.device
    out = {k: torch.empty((neqmax + 1, npix), dtype=torch.float64, device=dev) for k in ('I', 'Q', 'U', 'evpa')}
    if per_crossing:
        out.update({k: torch.empty((G, npix), dtype=torch.float64, device=dev) for k in ('Ic', 'Qc', 'Uc')})
    out['stagnation'] = torch.zeros(2, dtype=torch.float64, device=dev)
    out['status'] = torch.zeros(1, dtype=torch.int32, device=dev)
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    em = _lib.JetEmission(_lib.JET[model], int(neqmax), float(pval), float(nu_parallel), float(sigma), float(specind))
    s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(lib.kgeo_jet_stokes(ctypes.byref(ob), _p(al), _p(be), npix, *[_p(cr[k]) for k in
                                                                                ('r', 'th', 'signpr', 'signpth',
                                                                                 'neq')],
                                   G, ctypes.byref(em), *[_p(out.get(k)) for k in ('I', 'Q', 'U', 'evpa', 'Ic', 'Qc',
                                                                                   'Uc', 'stagnation', 'status')],
                                   s))
    return out


def _stagnation_error(status):
    if status == 1:
        raise IndexError("index 0 is out of bounds for axis 0 with size 0")
    if status != 0:
        raise np.linalg.LinAlgError("no stagnation radius: the monopole outflow's quintic has fewer than 5 roots")


def getstokes(psitarget, alphavals, betavals, r_o, th_o, a, ngeo, do_phi_and_t=True, neqmax=1, outgeo=None,
              tol=1e-8, model='para', pval=1, nu_parallel=0, gammamax=None, retvals=False, sigma=2,
              sumsubring=True, usemono=False, retsin=False):
    """Stokes images of the emission along the field line psi = psitarget
    (kgeo/off_eq.py:124-233). Returns (I, Q, U, evpa), each (neqmax + 1, *alphavals.shape):
    the images of the crossings after neq = 0 .. neqmax - 1 equatorial crossings, then their
    total; retvals adds the crossing radii and angles; sumsubring=False returns the per-crossing
    (I, Q, U, neq, r, th, guesses_shape) instead."""
    _supported(model, pval, gammamax, retsin, nu_parallel)
    _check_args(a, r_o, th_o)
    ashape = np.shape(alphavals)
    if isinstance(alphavals, torch.Tensor):
        alphavals, betavals = alphavals.flatten(), betavals.flatten()
    else:
        alphavals, betavals = np.asarray(alphavals).flatten(), np.asarray(betavals).flatten()
    alphavals, betavals = _pixels(alphavals, betavals)
    al, be = _dev.as_device(alphavals), _dev.as_device(betavals)
    if outgeo is None:
        geo = _dev.trace(a, r_o, th_o, al, be, ngeo=ngeo, outputs=('r', 'th', 'mino'), per_ray=())
        _flags_check(a, geo['flags'])
        r, th, mino = geo['r'], geo['th'], geo['mino']
    else:
        r, th, mino = outgeo.r_s, outgeo.th_s, outgeo.mino_times
    cr, shape = _solver.crossings_device(a, r_o, th_o, al, be, r, th, mino, psitarget, model=model, neqmax=neqmax,
                                         tol=tol, pval=pval)
    st = stokes_device(a, r_o, th_o, al, be, cr, neqmax=neqmax, model=model, pval=pval, nu_parallel=nu_parallel,
                       sigma=sigma, per_crossing=not sumsubring)
    _stagnation_error(int(st['status'].item()))
    rv = torch.nan_to_num(cr['r'].reshape(-1))
    tv = torch.nan_to_num(cr['th'].reshape(-1))
    if not sumsubring:
        vals = _dev.to_host([st['Ic'].reshape(-1), st['Qc'].reshape(-1), st['Uc'].reshape(-1),
                             cr['neq'].reshape(-1), rv, tv])
        return tuple(vals) + (shape,)
    keys = ('I', 'Q', 'U', 'evpa')
    vals = _dev.to_host([st[k] for k in keys] + ([rv, tv] if retvals else []))
    imgs = [v.reshape((neqmax + 1,) + tuple(ashape)) for v in vals[:4]]
    if not retvals:
        return tuple(imgs)
    return tuple(imgs) + (vals[4], vals[5])


__all__ = ['getstokes', 'stokes_device', 'SPECIND']
