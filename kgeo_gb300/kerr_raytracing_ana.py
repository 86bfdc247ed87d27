"""Drop-in for kgeo.kerr_raytracing_ana: raytrace_ana and coords_at_tau on the GPU.

Same signatures, argument checks, messages and outputs as
kgeo/kerr_raytracing_ana.py:46-193; the work runs in the sm_103a kernels behind the
C ABI (include/kgeo_gb300.h). Plotting and HDF5 saving of the reference are not
part of this package: `plotdata` and `savedata` are accepted and ignored.
"""
import warnings

import numpy as np
import torch

from . import device as _dev
from . import _lib
from .kerr_raytracing_utils import Geodesics, MINSPIN

SPIN = 0.94                      # kgeo/kerr_raytracing_ana.py:21-26
INC = 20 * np.pi / 180.
ROUT = 100000.
NGEO = 250
NPIX = 1000
MAXTAUFRAC = (1. - 1.e-10)

alpha_default = np.linspace(-6, 6, NPIX)
beta_default = 0 * alpha_default


def _check_args(a, r_o, th_o):
    """kgeo/kerr_raytracing_ana.py:59-66 (messages and warnings verbatim)."""
    if not (isinstance(a, float) and (0 <= np.abs(a) < 1)):
        raise Exception("|a| should be a float in range [0,1)")
    if (a < 0):
        print("WARNING a<0! Not fully verified!")
    if not (isinstance(r_o, float) and (r_o >= 100)):
        raise Exception("r_o should be a float > 100")
    if not (isinstance(th_o, float) and (0 < th_o < np.pi) and th_o != 0.5 * np.pi):
        raise Exception("th_o should be a float in range (0,pi/2) or (pi/2,pi)")
    if (th_o > np.pi / 2.):
        print("WARNING th_o>pi/2! Not fully verified!")


def _pixels(alpha, beta):
    """kgeo/kerr_raytracing_ana.py:68-71 (tensors are accepted as they are)."""
    if not isinstance(alpha, (np.ndarray, torch.Tensor)):
        alpha = np.array([alpha]).flatten()
    if not isinstance(beta, (np.ndarray, torch.Tensor)):
        beta = np.array([beta]).flatten()
    if len(alpha) != len(beta):
        raise Exception("alpha, beta are different lengths!")
    return alpha, beta


class ConvergenceWarning(RuntimeWarning):
    """An iterative loop of the device's elliptic arithmetic stopped at its iteration cap."""


def warn_loop_cap(f):
    if f & _lib.FLAG_LOOP_CAP:
        warnings.warn("kgeo_gb300: an elliptic-integral loop (Carlson duplication or Landen descent) stopped "
                      "at its iteration cap; some samples may be inaccurate", ConvergenceWarning, stacklevel=3)


def _flags_check(a, flags):
    f = flags if isinstance(flags, int) else int(flags.item())
    if f & _lib.FLAG_MINSPIN_VORTICAL:
        raise Exception("below MINSPIN but there are eta<0 points in th_integrate!")
    if np.abs(a) < MINSPIN and (f & _lib.FLAG_ANY_ETA_NONPOS):
        print("WARNING: there were eta<0 points for spin %f<MINSPIN!" % a)
    warn_loop_cap(f)


def raytrace_ana(a=SPIN, observer_coords=[0, ROUT, INC, 0], image_coords=[alpha_default, beta_default],
                 ngeo=NGEO, maxtaufrac=MAXTAUFRAC, do_phi_and_t=True, savedata=False, plotdata=True,
                 device_arrays=False):
    """Analytically raytrace over the full range of Mino times (kgeo/kerr_raytracing_ana.py:46-122).

    Returns a Geodesics whose arrays are numpy (default) or CUDA tensors
    (device_arrays=True, no host copy).
    """
    [_, r_o, th_o, _] = observer_coords
    [alpha, beta] = image_coords
    _check_args(a, r_o, th_o)
    alpha, beta = _pixels(alpha, beta)
    keys = ('mino', 'sig', 't', 'r', 'th', 'ph')
    if not device_arrays and not (isinstance(alpha, torch.Tensor) and alpha.is_cuda):
        # host arrays in and out: kgeo_raytrace_host overlaps the copies with the kernels
        _dev.require_cuda()
        al = alpha.cpu().numpy() if isinstance(alpha, torch.Tensor) else alpha
        be = beta.cpu().numpy() if isinstance(beta, torch.Tensor) else beta
        res = _dev.trace_host(a, r_o, th_o, al, be, ngeo, maxtaufrac=maxtaufrac)
        _flags_check(a, res['flags'])
        vals = [res[k] for k in keys]
    else:
        al = _dev.as_device(alpha)
        be = _dev.as_device(beta)
        res = _dev.trace(a, r_o, th_o, al, be, ngeo=ngeo, maxtaufrac=maxtaufrac)
        _flags_check(a, res['flags'])
        vals = [res[k] for k in keys] if device_arrays else _dev.to_host([res[k] for k in keys])
    return Geodesics(a, observer_coords, image_coords, vals[0], vals[1], list(vals[2:]))


def coords_at_tau(a, observer_coords, image_coords, tau, do_phi_and_t=True, device_arrays=False):
    """Coordinates at Mino times tau (ntau, npix) or (npix) (kgeo/kerr_raytracing_ana.py:126-193).

    Returns (sig_s, [t_s, r_s, th_s, ph_s]).
    """
    [_, r_o, th_o, _] = observer_coords
    [alpha, beta] = image_coords
    _check_args(a, r_o, th_o)
    alpha, beta = _pixels(alpha, beta)
    if len(tau.shape) == 1:
        tau = tau.reshape(1, tau.shape[0])
    if not (tau.shape[1] == len(alpha)):
        raise Exception("tau has incompatible shape in coords_at_tau!")
    res = _dev.trace(a, r_o, th_o, _dev.as_device(alpha), _dev.as_device(beta), tau=_dev.as_device(tau),
                     do_phi_and_t=do_phi_and_t, outputs=('t', 'r', 'th', 'ph', 'sig'), per_ray=())
    _flags_check(a, res['flags'])
    keys = ('sig', 't', 'r', 'th', 'ph')
    vals = [res[k] for k in keys] if device_arrays else _dev.to_host([res[k] for k in keys])
    return vals[0], list(vals[1:])
