"""Device-side driver of the tracer: torch supplies device memory and the stream,
the work is done by the CUDA kernels behind the C ABI (kgeo_gb300/_lib.py)."""
import ctypes

import numpy as np
import torch

from . import _lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError('kgeo_gb300 needs a CUDA device (GB300); there is no CPU path')


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def as_device(x, device='cuda'):
    """float64 contiguous CUDA tensor from a numpy array / tensor / scalar."""
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64))).to(device)


class Workspace:
    """Reusable device scratch for the per-ray records (grows on demand)."""

    def __init__(self):
        self.buf = None

    def get(self, npix, device):
        need = int(_lib.load().kgeo_workspace_size(npix))
        if self.buf is None or self.buf.numel() < need or self.buf.device != device:
            self.buf = torch.empty(need, dtype=torch.uint8, device=device)
        return self.buf, need


_WS = {}


def workspace(device):
    key = (device.type, device.index)
    if key not in _WS:
        _WS[key] = Workspace()
    return _WS[key]


def trace(a, r_o, th_o, alpha, beta, ngeo=None, tau=None, maxtaufrac=1.0 - 1.0e-10, do_phi_and_t=True,
          outputs=('t', 'r', 'th', 'ph', 'sig', 'mino'), per_ray=('tau_tot', 'rclass', 'thclass'),
          stream=None):
    """Run kgeo_raytrace (tau is None: ngeo linspace samples) or kgeo_coords_at_tau.

    alpha, beta: CUDA float64 tensors (npix). tau: CUDA float64 (ntau, npix) or None.
    Returns a dict of CUDA tensors plus 'flags' (a 1-element int32 tensor).
    """
    require_cuda()
    lib = _lib.load()
    dev = alpha.device
    npix = alpha.numel()
    if tau is not None:
        nsamp = tau.shape[0]
    else:
        nsamp = int(ngeo)
    res = {}
    for k in outputs:
        res[k] = torch.empty((nsamp, npix), dtype=torch.float64, device=dev)
    if 'tau_tot' in per_ray:
        res['tau_tot'] = torch.empty(npix, dtype=torch.float64, device=dev)
    for k in ('rclass', 'thclass'):
        if k in per_ray:
            res[k] = torch.empty(npix, dtype=torch.int32, device=dev)
    res['flags'] = torch.zeros(1, dtype=torch.int32, device=dev)
    g = _lib.GeodesicsOut(*[_ptr(res.get(k)) for k in ('t', 'r', 'th', 'ph', 'sig', 'mino', 'tau_tot', 'rclass',
                                                          'thclass', 'flags')])
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    ws, need = workspace(dev).get(npix, dev)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    if tau is None:
        code = lib.kgeo_raytrace(ctypes.byref(ob), _ptr(alpha), _ptr(beta), npix, nsamp, float(maxtaufrac),
                                 ctypes.byref(g), _ptr(ws), need, ctypes.c_void_p(s.cuda_stream))
    else:
        code = lib.kgeo_coords_at_tau(ctypes.byref(ob), _ptr(alpha), _ptr(beta), npix, _ptr(tau), nsamp,
                                      1 if do_phi_and_t else 0, ctypes.byref(g), _ptr(ws), need,
                                      ctypes.c_void_p(s.cuda_stream))
    _lib.check(code)
    return res
