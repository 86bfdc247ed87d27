"""The drop-in functions as torch operators on CUDA tensors (namespace ``kgeo``).

    torch.ops.kgeo.raytrace(alpha, beta, a, r_o, th_o, ngeo, maxtaufrac)
        -> (mino, sig, t, r, th, ph), each (ngeo, npix)          kgeo/kerr_raytracing_ana.py:46
    torch.ops.kgeo.coords_at_tau(alpha, beta, tau, a, r_o, th_o, do_phi_and_t)
        -> (sig, t, r, th, ph), each shaped like tau (ntau, npix)  kgeo/kerr_raytracing_ana.py:126
    torch.ops.kgeo.r_equatorial(alpha, beta, a, r_o, th_o, mbar_lo, n_orders)
        -> (r_s, Ir) (n_orders, npix), (Imax, Nmax) (npix)         kgeo/equatorial_lensing.py:85
    torch.ops.kgeo.image(params, alpha, beta, r_o, mbar_max, emissivity, velocity, retrograde,
                         specind, sinthb, mu_ring, emiscut_in, emiscut_out)
        -> I (npix, mbar_max + 1), differentiable in params       kgeo/equatorial_images.py:23, 124
    torch.ops.kgeo.image_adjoint(grad_I, params, alpha, beta, ...) -> (7,) dL/dparams
    torch.ops.kgeo.jet_stokes(alpha, beta, r, th, signpr, signpth, neq, a, r_o, th_o, neqmax, model,
                              pval, nu_parallel, sigma, specind)
        -> (I, Q, U, evpa), each (neqmax + 1, npix)               kgeo/off_eq.py:124

Every operator runs the CUDA library on the current stream of the inputs' device, raises the
reference's exceptions for invalid arguments, and has a fake implementation (shapes only) for
FakeTensor / meta tracing. params of kgeo::image are (a, th_o, e0, e1, v0, v1, v2) as in
image_grad; the op reads them on the host, and its backward is kgeo::image_adjoint.
"""
import torch
from torch import Tensor

from . import device as _dev
from .equatorial_images import SINTHB, SPECIND, image_adjoint_device, image_device
from .equatorial_lensing import r_equatorial_device
from .image_grad import _model
from .kerr_raytracing_ana import _check_args, _flags_check

_TRACE_KEYS = ('mino', 'sig', 't', 'r', 'th', 'ph')


def _pixels(alpha, beta):
    if alpha.numel() != beta.numel():
        raise Exception("alpha, beta are different lengths!")
    return alpha.reshape(-1).to(torch.float64).contiguous(), beta.reshape(-1).to(torch.float64).contiguous()


@torch.library.custom_op('kgeo::raytrace', mutates_args=())
def raytrace(alpha: Tensor, beta: Tensor, a: float, r_o: float, th_o: float, ngeo: int,
             maxtaufrac: float = 1.0 - 1.0e-10) -> tuple[Tensor, Tensor, Tensor, Tensor, Tensor, Tensor]:
    _check_args(float(a), float(r_o), float(th_o))
    al, be = _pixels(alpha, beta)
    res = _dev.trace(a, r_o, th_o, al, be, ngeo=ngeo, maxtaufrac=maxtaufrac, outputs=_TRACE_KEYS, per_ray=())
    _flags_check(a, res['flags'])
    return tuple(res[k] for k in _TRACE_KEYS)


@raytrace.register_fake
def _(alpha, beta, a, r_o, th_o, ngeo, maxtaufrac=1.0 - 1.0e-10):
    n = alpha.numel()
    return tuple(alpha.new_empty((ngeo, n), dtype=torch.float64) for _ in _TRACE_KEYS)


@torch.library.custom_op('kgeo::coords_at_tau', mutates_args=())
def coords_at_tau(alpha: Tensor, beta: Tensor, tau: Tensor, a: float, r_o: float, th_o: float,
                  do_phi_and_t: bool = True) -> tuple[Tensor, Tensor, Tensor, Tensor, Tensor]:
    _check_args(float(a), float(r_o), float(th_o))
    al, be = _pixels(alpha, beta)
    if tau.shape[-1] != al.numel() or tau.dim() > 2:
        raise Exception("tau has incompatible shape in coords_at_tau!")
    t2 = tau.to(torch.float64).reshape(-1, al.numel()).contiguous()
    res = _dev.trace(a, r_o, th_o, al, be, tau=t2, do_phi_and_t=do_phi_and_t, outputs=('sig', 't', 'r', 'th', 'ph'),
                     per_ray=())
    _flags_check(a, res['flags'])
    return tuple(res[k].reshape(tau.shape) for k in ('sig', 't', 'r', 'th', 'ph'))


@coords_at_tau.register_fake
def _(alpha, beta, tau, a, r_o, th_o, do_phi_and_t=True):
    return tuple(tau.new_empty(tau.shape, dtype=torch.float64) for _ in range(5))


@torch.library.custom_op('kgeo::r_equatorial', mutates_args=())
def r_equatorial(alpha: Tensor, beta: Tensor, a: float, r_o: float, th_o: float, mbar_lo: int,
                 n_orders: int) -> tuple[Tensor, Tensor, Tensor, Tensor]:
    _check_args(float(a), float(r_o), float(th_o))
    if mbar_lo < 0:
        raise Exception("mbar should be an integer >=0!")
    al, be = _pixels(alpha, beta)
    r_s, Ir, Imax, Nmax = r_equatorial_device(a, r_o, th_o, range(mbar_lo, mbar_lo + n_orders), al, be)
    return r_s, Ir, Imax, Nmax


@r_equatorial.register_fake
def _(alpha, beta, a, r_o, th_o, mbar_lo, n_orders):
    n = alpha.numel()
    e = lambda *s: alpha.new_empty(s, dtype=torch.float64)  # noqa: E731
    return e(n_orders, n), e(n_orders, n), e(n), e(n)


@torch.library.custom_op('kgeo::image', mutates_args=())
def image(params: Tensor, alpha: Tensor, beta: Tensor, r_o: float = 1.e4, mbar_max: int = 2,
          emissivity: str = 'bpl', velocity: str = 'general', retrograde: bool = False, specind: float = SPECIND,
          sinthb: float = SINTHB, mu_ring: float = 0.0, emiscut_in: float = 0.0,
          emiscut_out: float = 1.e10) -> Tensor:
    p = [float(x) for x in params.detach().cpu().tolist()]
    _check_args(p[0], float(r_o), p[1])
    al, be = _pixels(alpha, beta)
    model = _model(emissivity, velocity, p, retrograde, specind, sinthb, mu_ring, emiscut_in, emiscut_out)
    return image_device(p[0], r_o, p[1], 0, mbar_max + 1, al, be, model)['I']


@image.register_fake
def _(params, alpha, beta, r_o=1.e4, mbar_max=2, emissivity='bpl', velocity='general', retrograde=False,
      specind=SPECIND, sinthb=SINTHB, mu_ring=0.0, emiscut_in=0.0, emiscut_out=1.e10):
    return alpha.new_empty((alpha.numel(), mbar_max + 1), dtype=torch.float64)


@torch.library.custom_op('kgeo::image_adjoint', mutates_args=())
def image_adjoint(grad_I: Tensor, params: Tensor, alpha: Tensor, beta: Tensor, r_o: float = 1.e4, mbar_max: int = 2,
                  emissivity: str = 'bpl', velocity: str = 'general', retrograde: bool = False,
                  specind: float = SPECIND, sinthb: float = SINTHB, mu_ring: float = 0.0, emiscut_in: float = 0.0,
                  emiscut_out: float = 1.e10) -> Tensor:
    p = [float(x) for x in params.detach().cpu().tolist()]
    al, be = _pixels(alpha, beta)
    model = _model(emissivity, velocity, p, retrograde, specind, sinthb, mu_ring, emiscut_in, emiscut_out)
    g = image_adjoint_device(p[0], r_o, p[1], 0, mbar_max + 1, al, be, model, grad_I)
    return g.to(params.device)


@image_adjoint.register_fake
def _(grad_I, params, alpha, beta, *args):
    return params.new_empty((7,), dtype=torch.float64)


def _image_setup(ctx, inputs, output):
    ctx.inputs = inputs


def _image_backward(ctx, grad_I):
    params, alpha, beta = ctx.inputs[:3]
    g = image_adjoint(grad_I.contiguous(), params, alpha, beta, *ctx.inputs[3:])
    return (g,) + (None,) * (len(ctx.inputs) - 1)


image.register_autograd(_image_backward, setup_context=_image_setup)


@torch.library.custom_op('kgeo::jet_stokes', mutates_args=())
def jet_stokes(alpha: Tensor, beta: Tensor, r: Tensor, th: Tensor, signpr: Tensor, signpth: Tensor, neq: Tensor,
               a: float, r_o: float, th_o: float, neqmax: int = 1, model: str = 'mono', pval: float = 0.0,
               nu_parallel: float = 0.0, sigma: float = 2.0,
               specind: float = SPECIND) -> tuple[Tensor, Tensor, Tensor, Tensor]:
    from .off_eq import _stagnation_error, _supported, stokes_device
    _supported(model, pval, None, False, nu_parallel)
    _check_args(float(a), float(r_o), float(th_o))
    al, be = _pixels(alpha, beta)
    cr = dict(r=r, th=th, signpr=signpr, signpth=signpth, neq=neq)
    out = stokes_device(a, r_o, th_o, al, be, cr, neqmax=neqmax, model=model, pval=pval, nu_parallel=nu_parallel,
                        sigma=sigma, specind=specind)
    _stagnation_error(int(out['status'].item()))
    return out['I'], out['Q'], out['U'], out['evpa']


@jet_stokes.register_fake
def _(alpha, beta, r, th, signpr, signpth, neq, a, r_o, th_o, neqmax=1, model='mono', pval=0.0, nu_parallel=0.0,
      sigma=2.0, specind=SPECIND):
    n = alpha.numel()
    return tuple(alpha.new_empty((neqmax + 1, n), dtype=torch.float64) for _ in range(4))


__all__ = ['raytrace', 'coords_at_tau', 'r_equatorial', 'image', 'image_adjoint', 'jet_stokes']
