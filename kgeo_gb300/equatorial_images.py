"""Drop-in for kgeo.equatorial_images (images of an equatorial source) on the GPU.

make_image: kgeo/equatorial_images.py:23-122; Iobs: :124-264. Same signatures, argument
checks, defaults and output tuples. Every order of every pixel runs in one CUDA kernel
(kgeo_image_ex in include/kgeo_gb300.h): r_equatorial's source radius, the zero mask, the
momentum signs, the lab-frame velocity, the redshift, the emissivity and, with
polarization=True, the B-field, sin(theta_B) and the EVPA (calc_polquantities, calc_evpa),
with pathlength=True the rest-frame path length (calc_pathlength_equatorial).

Scope: equatorial emission (th_s = pi/2); emissivities 'bpl' / 'constant' / 'glm' / 'ring';
velocities 'zamo' / 'infall' / 'kep' / 'cunningham' / 'subkep' / 'cunningham_subkep' /
'general'; the lab-frame B-field models of kgeo_gb300.bfields. The thermal emissivity,
tabulated ('fromfile') inputs and comoving-frame fields raise NotImplementedError.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import device as _dev
from .bfields import Bfield, field_struct
from .emissivities import Emissivity
from .velocities import Velocity

SPECIND = 1
DISKANGLE = 0.1
SINTHB = np.pi / 4.
OBSFREQ = 230.e9

emis_default = Emissivity('bpl')
vel_default = Velocity('zamo')
bfield_default = Bfield('rad')


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _check_obs(a, r_o, th_o):
    if not (isinstance(a, float) and (0 <= np.abs(a) < 1)):
        raise Exception("|a| should be a float in range [0,1)")
    if not (isinstance(r_o, float) and (r_o >= 100)):
        raise Exception("r_o should be a float > 100")
    if not (isinstance(th_o, float) and (0 < th_o < np.pi) and th_o != 0.5 * np.pi):
        raise Exception("th_o should be a float in range (0,pi/2) or (pi/2,pi)")


def emission_model(emissivity=emis_default, velocity=vel_default, specind=SPECIND, sinthb=SINTHB):
    """kgeo_emission for an Emissivity / Velocity pair (this package's or the reference's
    objects: only their attributes are read). Raises the reference's exceptions for
    out-of-range velocity parameters (kgeo/velocities.py:315-317, 446-451)."""
    et = getattr(emissivity, 'emistype', None)
    vt = getattr(velocity, 'veltype', None)
    if et not in _lib.EMIS:
        raise NotImplementedError("emissivity %r is not on the GPU image path" % (et,))
    if vt not in _lib.VEL:
        raise NotImplementedError("velocity %r is not on the GPU image path" % (vt,))
    m = _lib.Emission()
    m.emissivity = _lib.EMIS[et]
    m.velocity = _lib.VEL[vt]
    m.retrograde = int(bool(getattr(velocity, 'retrograde', False)))
    if et == 'bpl':
        m.emis_p[0], m.emis_p[1] = float(emissivity.p1), float(emissivity.p2)
    elif et in ('glm', 'ring'):
        m.emis_p[0], m.emis_p[1] = float(emissivity.gamma_off), float(emissivity.sigma)
        m.mu_ring = float(emissivity.mu_ring) if emissivity.mu_ring else 0.0
    vp = [1.0, 1.0, 1.0]
    if vt in ('subkep', 'cunningham_subkep', 'general'):
        vp[0] = float(velocity.fac_subkep)
        if not (0 <= vp[0] <= 1):
            raise Exception("fac_subkep should be in the range [0,1]")
    if vt == 'general':
        vp[1], vp[2] = float(velocity.beta_phi), float(velocity.beta_r)
        if not (0 <= vp[1] <= 1):
            raise Exception("beta_phi should be in the range [0,1]")
        if not (0 <= vp[2] <= 1):
            raise Exception("beta_r should be in the range [0,1]")
    for k in range(3):
        m.vel_p[k] = vp[k]
    m.emiscut_in = float(getattr(emissivity, 'emiscut_in', 0))
    m.emiscut_out = float(getattr(emissivity, 'emiscut_out', 1.e10))
    m.specind = float(specind)
    m.sinthb = float(sinthb)
    return m


def model_params(model):
    """The seven differentiable parameters of a kgeo_emission after (a, th_o):
    (emis_p[0], emis_p[1], vel_p[0], vel_p[1], vel_p[2])."""
    return [model.emis_p[0], model.emis_p[1], model.vel_p[0], model.vel_p[1], model.vel_p[2]]


def image_options(bfield=bfield_default, polarization=False, pathlength=False, diskangle=DISKANGLE):
    """kgeo_image_options, or None for the plain unpolarised image."""
    if getattr(bfield, 'fieldframe', 'lab') != 'lab':
        raise NotImplementedError("comoving-frame fields are not on the GPU image path")
    if not polarization and not pathlength:
        return None
    o = _lib.ImageOptions()
    o.polarization = int(bool(polarization))
    o.pathlength = int(bool(pathlength))
    o.diskangle = float(diskangle)
    if polarization:
        o.bfield = field_struct(bfield)
    return o


def image_device(a, r_o, th_o, mbar_lo, n_orders, alpha, beta, model, outputs=('I',), stream=None, options=None):
    """Run kgeo_image_ex on CUDA tensors alpha, beta (npix). Returns a dict of CUDA tensors:
    per-order outputs (npix, n_orders) among I, g, r_s, Ir, sinthb, Q, U, lp, Ie; per-pixel
    imax, nmax, npol. options: kgeo_image_options (image_options) or None."""
    _dev.require_cuda()
    lib = _lib.load()
    npix = alpha.numel()
    dev = alpha.device
    res = {}
    per_order = ('I', 'g', 'r_s', 'Ir', 'sinthb', 'Q', 'U', 'lp', 'Ie')
    for k in set(outputs) | {'I'}:
        shape = (npix, n_orders) if k in per_order else (npix,)
        res[k] = torch.empty(shape, dtype=torch.float64, device=dev)
    out = _lib.ImageOut(*[_p(res.get(k)) for k in ('I', 'g', 'r_s', 'Ir', 'sinthb', 'imax', 'nmax', 'npol',
                                                   'Q', 'U', 'lp', 'Ie')])
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    opt = ctypes.byref(options) if options is not None else None
    _lib.check(lib.kgeo_image_ex(ctypes.byref(ob), int(mbar_lo), int(n_orders), _p(alpha), _p(beta), npix,
                                 ctypes.byref(model), opt, ctypes.byref(out), ctypes.c_void_p(s.cuda_stream)))
    for k in ('Q', 'U', 'lp', 'Ie'):
        if k in res and (options is None or (k in ('Q', 'U') and not options.polarization)
                         or (k in ('lp', 'Ie') and not options.pathlength)):
            res[k].zero_()
    return res


def image_adjoint_device(a, r_o, th_o, mbar_lo, n_orders, alpha, beta, model, grad_I, stream=None):
    """kgeo_image_adjoint: dL/d(a, th_o, emis_p[0..1], vel_p[0..2]) (7,) CUDA tensor for
    grad_I = dL/dI (npix, n_orders)."""
    _dev.require_cuda()
    lib = _lib.load()
    npix = alpha.numel()
    dev = alpha.device
    grad_I = grad_I.to(dtype=torch.float64).contiguous()
    nbytes = int(lib.kgeo_image_adjoint_workspace_size(npix))
    ws = torch.empty(max(nbytes, 8), dtype=torch.uint8, device=dev)
    grad = torch.empty(_lib.N_IMAGE_PARAMS, dtype=torch.float64, device=dev)
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.check(lib.kgeo_image_adjoint(ctypes.byref(ob), int(mbar_lo), int(n_orders), _p(alpha), _p(beta), npix,
                                      ctypes.byref(model), _p(grad_I), _p(grad), _p(ws), nbytes,
                                      ctypes.c_void_p(s.cuda_stream)))
    return grad


def _unsupported(emissivity, th_s=np.pi / 2):
    if getattr(emissivity, 'emistype', None) == 'thermal':
        raise NotImplementedError("the thermal emissivity is not on the GPU image path")
    if th_s != np.pi / 2:
        raise NotImplementedError("only equatorial emission (th_s = pi/2) is on the GPU path")


def image_pixels(alpha_min, alpha_max, beta_min, beta_max, psize):
    """make_image's pixel grid (kgeo/equatorial_images.py:48-55), flattened alpha, beta."""
    n_alpha = int(np.floor(alpha_max - alpha_min) / psize)
    alphas = np.linspace(alpha_min, alpha_min + n_alpha * psize, n_alpha)
    n_beta = int(np.floor(beta_max - beta_min) / psize)
    betas = np.linspace(beta_min, beta_min + n_beta * psize, n_beta)
    alpha_arr, beta_arr = np.meshgrid(alphas, betas)
    return alpha_arr.flatten(), beta_arr.flatten()


def make_image(a, r_o, th_o, mbar_max, alpha_min, alpha_max, beta_min, beta_max, psize,
               nmax_only=False,
               emissivity=emis_default,
               bfield=bfield_default,
               velocity=vel_default,
               polarization=False,
               pathlength=False,
               specind=SPECIND,
               diskangle=DISKANGLE,
               nu_obs=OBSFREQ,
               device_arrays=False):
    """Image in (alpha_min, alpha_max) x (beta_min, beta_max) for all orders m <= mbar_max
    (kgeo/equatorial_images.py:23-122). Returns (I, Q, U, r, t, g, sinthb, n, np), plus
    (lp, Ie) with pathlength=True; the per-order arrays are (npix, mbar_max + 1). With
    nmax_only=True only n and np are computed (the reference leaves its return value
    unassigned on that branch; here the tuple is returned with zero images).
    device_arrays=True returns CUDA tensors."""
    if not (isinstance(a, float) and (0 <= np.abs(a) < 1)):
        raise Exception("|a| should be a float in range [0,1)")
    if not (isinstance(r_o, float) and (r_o >= 100)):
        raise Exception("r_o should be a float > 100")
    if not (isinstance(th_o, float) and (0 < th_o < np.pi) and th_o != 0.5 * np.pi):
        raise Exception("th_o should be a float in range (0,pi/2) or (pi/2,pi)")
    if not (isinstance(mbar_max, int) and (mbar_max >= 0)):
        raise Exception("mbar_max should be an integer >=0!")
    _unsupported(emissivity)
    A, B = image_pixels(alpha_min, alpha_max, beta_min, beta_max, psize)
    model = emission_model(emissivity, velocity, specind)
    opts = image_options(bfield, polarization, pathlength, diskangle)
    al, be = _dev.as_device(A), _dev.as_device(B)
    n = mbar_max + 1
    extra = ('lp', 'Ie') if pathlength else ()
    res = image_device(a, r_o, th_o, 0, n, al, be, model,
                       outputs=('I', 'Q', 'U', 'g', 'r_s', 'Ir', 'sinthb', 'nmax', 'npol') + extra, options=opts)
    if nmax_only:
        from .equatorial_lensing import nmax_equatorial
        zeros = torch.zeros((A.size, n), dtype=torch.float64, device=al.device)
        nmax = torch.as_tensor(nmax_equatorial(a, r_o, th_o, A, B), device=al.device)
        outs = [zeros, zeros.clone(), zeros.clone(), zeros.clone(), zeros.clone(), zeros.clone(), zeros.clone(),
                nmax, res['npol']]
    else:
        outs = [res['I'], res['Q'], res['U'], res['r_s'], res['Ir'], res['g'], res['sinthb'], res['nmax'],
                res['npol']] + [res[k] for k in extra]
    if device_arrays:
        return tuple(outs)
    return tuple(_dev.to_host(outs))


def Iobs(a, r_o, th_o, mbar, alpha, beta,
         emissivity=emis_default, velocity=vel_default, bfield=bfield_default,
         polarization=False, pathlength=False, specind=SPECIND, diskangle=DISKANGLE, nu_obs=OBSFREQ,
         th_s=np.pi / 2, device_arrays=False):
    """(Iobs, Qobs, Uobs, g, r_s, sin_thb, Ir, Imax, Nmax), plus (lp, Ie) with
    pathlength=True, of image order mbar (kgeo/equatorial_images.py:124-264)."""
    if not (isinstance(a, float) and (0 <= np.abs(a) < 1)):
        raise Exception("|a| should be a float in range [0,1)")
    if not (isinstance(r_o, float) and (r_o >= 100)):
        raise Exception("r_o should be a float > 100")
    if not (isinstance(th_o, float) and (0 < th_o < np.pi) and th_o != 0.5 * np.pi):
        raise Exception("th_o should be a float in range (0,pi/2) or (pi/2,pi)")
    if not (isinstance(mbar, int) and (mbar >= 0)):
        raise Exception("mbar should be an integer >=0!")
    if not isinstance(alpha, (np.ndarray, torch.Tensor)):
        alpha = np.array([alpha]).flatten()
    if not isinstance(beta, (np.ndarray, torch.Tensor)):
        beta = np.array([beta]).flatten()
    if len(alpha) != len(beta):
        raise Exception("alpha, beta are different lengths!")
    _unsupported(emissivity, th_s)
    model = emission_model(emissivity, velocity, specind)
    opts = image_options(bfield, polarization, pathlength, diskangle)
    al, be = _dev.as_device(alpha), _dev.as_device(beta)
    extra = ('lp', 'Ie') if pathlength else ()
    res = image_device(a, r_o, th_o, mbar, 1, al, be, model,
                       outputs=('I', 'Q', 'U', 'g', 'r_s', 'Ir', 'sinthb', 'imax', 'nmax') + extra, options=opts)
    outs = [res['I'][:, 0], res['Q'][:, 0], res['U'][:, 0], res['g'][:, 0], res['r_s'][:, 0], res['sinthb'][:, 0],
            res['Ir'][:, 0], res['imax'], res['nmax']] + [res[k][:, 0] for k in extra]
    if device_arrays:
        return tuple(outs)
    return tuple(_dev.to_host([o.contiguous() for o in outs]))
