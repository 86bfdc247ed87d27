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


_HOST_WS = {}


def trace_host(a, r_o, th_o, alpha, beta, ngeo, maxtaufrac=1.0 - 1.0e-10, mixed=False, device=None):
    """kgeo_raytrace_host: numpy alpha, beta (npix) in, numpy outputs out.

    The outputs live in page-locked host tensors (torch's pinned allocator caches them), which
    the sample kernel stores into directly (no staging, no copies). Returns a dict of
    numpy arrays t, r, th, ph, sig, mino (ngeo, npix), tau_tot, rclass, thclass (npix) and
    the flags word (int).
    """
    require_cuda()
    lib = _lib.load()
    dev = torch.device('cuda', torch.cuda.current_device()) if device is None else device
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    npix = alpha.size
    prec = _lib.PRECISION_MIXED if mixed else _lib.PRECISION_FP64
    need = int(lib.kgeo_raytrace_host_workspace_size(npix, int(ngeo), prec))
    key = (dev.type, dev.index)
    ws = _HOST_WS.get(key)
    if ws is None or ws.numel() < need:
        ws = _HOST_WS[key] = torch.empty(max(need, 1), dtype=torch.uint8, device=dev)
    res = {}
    for k in ('t', 'r', 'th', 'ph', 'sig', 'mino'):
        res[k] = torch.empty((int(ngeo), npix), dtype=torch.float64, pin_memory=True)
    res['tau_tot'] = torch.empty(npix, dtype=torch.float64, pin_memory=True)
    res['rclass'] = torch.empty(npix, dtype=torch.int32, pin_memory=True)
    res['thclass'] = torch.empty(npix, dtype=torch.int32, pin_memory=True)
    res['flags'] = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    g = _lib.GeodesicsOut(*[_ptr(res[k]) for k in ('t', 'r', 'th', 'ph', 'sig', 'mino', 'tau_tot', 'rclass',
                                                  'thclass', 'flags')])
    ob = _lib.Observer(float(a), float(r_o), float(th_o))
    s = torch.cuda.current_stream(dev)
    _lib.check(lib.kgeo_raytrace_host(ctypes.byref(ob), ctypes.c_void_p(alpha.ctypes.data),
                                      ctypes.c_void_p(beta.ctypes.data), npix, int(ngeo), float(maxtaufrac), prec,
                                      ctypes.byref(g), _ptr(ws), need, ctypes.c_void_p(s.cuda_stream)))
    s.synchronize()
    out = {k: v.numpy() for k, v in res.items() if k != 'flags'}
    out['flags'] = int(res['flags'][0])
    return out


class PreparedRays:
    """Rays set up once on the device (kgeo_ray_setup), sampled any number of times (kgeo_ray_samples)."""

    def __init__(self, a, r_o, th_o, alpha, beta, ngeo=0, maxtaufrac=1.0 - 1.0e-10, stream=None):
        require_cuda()
        self.lib = _lib.load()
        self.dev = alpha.device
        self.npix = alpha.numel()
        self.ngeo = int(ngeo)
        self.obs = _lib.Observer(float(a), float(r_o), float(th_o))
        self.ws_bytes = int(self.lib.kgeo_workspace_size(self.npix))
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.dev)
        self.alpha, self.beta, self.maxtaufrac = alpha, beta, float(maxtaufrac)
        self.tau_tot = torch.empty(self.npix, dtype=torch.float64, device=self.dev)
        self.rclass = torch.empty(self.npix, dtype=torch.int32, device=self.dev)
        self.thclass = torch.empty(self.npix, dtype=torch.int32, device=self.dev)
        self.setup(stream)

    def _stream(self, stream):
        return ctypes.c_void_p((stream if stream is not None else torch.cuda.current_stream(self.dev)).cuda_stream)

    def setup(self, stream=None):
        per = _lib.GeodesicsOut(None, None, None, None, None, None, _ptr(self.tau_tot), _ptr(self.rclass),
                                _ptr(self.thclass), None)
        _lib.check(self.lib.kgeo_ray_setup(ctypes.byref(self.obs), _ptr(self.alpha), _ptr(self.beta), self.npix,
                                           self.ngeo, self.maxtaufrac, _ptr(self.ws), self.ws_bytes,
                                           ctypes.byref(per), self._stream(stream)))

    def alloc(self, nsamp=None, keys=('t', 'r', 'th', 'ph', 'sig', 'mino'), fill=None):
        n = self.ngeo if nsamp is None else nsamp
        if fill is None:
            return {k: torch.empty((n, self.npix), dtype=torch.float64, device=self.dev) for k in keys}
        return {k: torch.full((n, self.npix), fill, dtype=torch.float64, device=self.dev) for k in keys}

    def samples(self, out, tau=None, do_phi_and_t=True, flags=None, stream=None, chunk=-1, mixed=False):
        nsamp = tau.shape[0] if tau is not None else self.ngeo
        g = _lib.GeodesicsOut(*[_ptr(out.get(k)) for k in ('t', 'r', 'th', 'ph', 'sig', 'mino')],
                              None, None, None, _ptr(flags))
        _lib.check(self.lib.kgeo_ray_samples(ctypes.byref(self.obs), _ptr(self.ws), self.ws_bytes, self.npix,
                                             _ptr(tau), nsamp, 1 if do_phi_and_t else 0, int(chunk),
                                             _lib.PRECISION_MIXED if mixed else _lib.PRECISION_FP64, ctypes.byref(g),
                                             self._stream(stream)))
        return out


def fp64_peak_tflops():
    """Measured FP64 FMA throughput of this GPU (TFLOP/s), from the library's probe kernel."""
    require_cuda()
    v = ctypes.c_double(0.0)
    _lib.check(_lib.load().kgeo_measure_fp64_peak(ctypes.byref(v), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return v.value


def to_host(tensors):
    """Copy CUDA tensors to numpy through pinned staging buffers (one synchronisation).

    The returned arrays are views of pinned host tensors (kept alive by the arrays),
    so the device-to-host copies run at the link's full rate.
    """
    outs = []
    for t in tensors:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        outs.append(h)
    torch.cuda.current_stream().synchronize()
    return [h.numpy() for h in outs]
