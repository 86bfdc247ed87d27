"""Differentiable equatorial image: torch.autograd.Function around kgeo_image and its
adjoint kernel kgeo_image_adjoint (include/kgeo_gb300.h).

    I = equatorial_image(params, alpha, beta, r_o=1e4, mbar_max=2,
                         emissivity='bpl', velocity='general')
    loss = ((I - target) ** 2).sum(); loss.backward()      # params.grad

params is a float64 tensor of 7 values (a, th_o, e0, e1, v0, v1, v2): e0, e1 are the
emissivity parameters ('bpl': p1, p2; 'glm' / 'ring': gamma_off, sigma) and v0..v2 the
velocity parameters ('subkep': fac_subkep; 'general': fac_subkep, beta_phi, beta_r). The
forward pass renders the (npix, mbar_max + 1) image on the GPU; the backward pass
recomputes every ray (nothing of the geodesics is stored) and returns dL/dparams from one
adjoint launch. Masks, momentum signs and crossing counts are piecewise constant and are
held fixed, as a finite difference that does not cross their boundaries sees them.
"""
import torch

from . import _lib
from . import device as _dev
from .equatorial_images import SINTHB, SPECIND, image_adjoint_device, image_device


def _model(kind_e, kind_v, p, retrograde, specind, sinthb, mu_ring, emiscut_in, emiscut_out):
    m = _lib.Emission()
    m.emissivity = _lib.EMIS[kind_e]
    m.velocity = _lib.VEL[kind_v]
    m.retrograde = int(bool(retrograde))
    m.emis_p[0], m.emis_p[1] = p[2], p[3]
    m.mu_ring = mu_ring
    m.vel_p[0], m.vel_p[1], m.vel_p[2] = p[4], p[5], p[6]
    m.emiscut_in = emiscut_in
    m.emiscut_out = emiscut_out
    m.specind = specind
    m.sinthb = sinthb
    return m


class EquatorialImageFunction(torch.autograd.Function):
    """I(params) with the adjoint kernel as the backward pass."""

    @staticmethod
    def forward(ctx, params, alpha, beta, r_o, mbar_max, kinds, opts):
        p = [float(x) for x in params.detach().cpu().tolist()]
        model = _model(kinds[0], kinds[1], p, *opts)
        n = mbar_max + 1
        I = image_device(p[0], r_o, p[1], 0, n, alpha, beta, model)['I']
        ctx.save_for_backward(alpha, beta)
        ctx.p, ctx.r_o, ctx.n, ctx.model = p, r_o, n, model
        ctx.param_device = params.device
        return I

    @staticmethod
    def backward(ctx, grad_I):
        alpha, beta = ctx.saved_tensors
        g = image_adjoint_device(ctx.p[0], ctx.r_o, ctx.p[1], 0, ctx.n, alpha, beta, ctx.model, grad_I)
        return g.to(ctx.param_device), None, None, None, None, None, None


def equatorial_image(params, alpha, beta, r_o=1.e4, mbar_max=2, emissivity='bpl', velocity='general',
                     retrograde=False, specind=SPECIND, sinthb=SINTHB, mu_ring=0.0, emiscut_in=0.0,
                     emiscut_out=1.e10):
    """Differentiable (npix, mbar_max + 1) image; see the module docstring."""
    _dev.require_cuda()
    if emissivity not in _lib.EMIS or velocity not in _lib.VEL:
        raise NotImplementedError("model (%s, %s) is not on the GPU image path" % (emissivity, velocity))
    if not isinstance(params, torch.Tensor) or params.numel() != _lib.N_IMAGE_PARAMS:
        raise ValueError("params must be a tensor of %d values" % _lib.N_IMAGE_PARAMS)
    al, be = _dev.as_device(alpha), _dev.as_device(beta)
    opts = (retrograde, float(specind), float(sinthb), float(mu_ring), float(emiscut_in), float(emiscut_out))
    return EquatorialImageFunction.apply(params, al, be, float(r_o), int(mbar_max), (emissivity, velocity), opts)


def config_params(a, th_o, p, xi, beta_r, beta_phi=1.0):
    """The 7-vector of a 'bpl' (j ~ r^-p, p2 = 0) + 'general' velocity image from the
    physical parameters (differentiable in each; any may be a tensor)."""
    def t(x):
        return x if isinstance(x, torch.Tensor) else torch.tensor(float(x), dtype=torch.float64)
    a, th_o, p, xi, beta_r, beta_phi = (t(x).to(torch.float64).reshape(()) for x in (a, th_o, p, xi, beta_r, beta_phi))
    zero = torch.zeros((), dtype=torch.float64)
    return torch.stack([a, th_o, -p, zero, xi, beta_phi, beta_r])


__all__ = ['EquatorialImageFunction', 'equatorial_image', 'config_params', 'reduce_loss_grad']


def reduce_loss_grad(loss, grad, group=None):
    """Sum a rank's image loss and its gradient over the process group: the one collective of
    a pixel-sharded image (every rank renders its own pixels; rays need no exchange). loss is a
    float, grad a sequence of floats; returns (loss, grad) summed over ranks as float64 on the
    host. Uses the default group's backend (NCCL on GPUs, gloo on CPUs)."""
    import torch.distributed as dist
    v = torch.tensor([float(loss)] + [float(g) for g in grad], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        if dist.get_backend(group) == 'nccl':
            v = v.cuda()
        dist.all_reduce(v, op=dist.ReduceOp.SUM, group=group)
    v = v.cpu()
    return float(v[0]), [float(x) for x in v[1:]]
