"""Batched tracing of many images in one job (kgeo_batch_* of include/kgeo_gb300.h).

    plan = BatchPlan([dict(a=0.5, th_o=1.0, npix=A0.size, ngeo=128), ...], precision='mixed')
    plan.bind(alpha_all, beta_all)          # concatenated pixels, CUDA float64
    plan.autotune()                         # optional: picks the sample kernel's launch shape
    plan.graph_launch()                     # whole pipeline as one CUDA graph replay
    geo = plan.image(3)                     # views: t, r, th, ph, sig, mino (ngeo, npix); rclass ...

The reference traces one image per raytrace_ana call (kgeo/kerr_raytracing_ana.py:46); a batch
gives each image exactly the result of that call (with the same chunk length) while the GPU
runs all images' rays in one persistent launch.
"""
import ctypes

import torch

from . import _lib
from .device import require_cuda

PRECISION = {'fp64': _lib.PRECISION_FP64, 'mixed': _lib.PRECISION_MIXED}
SAMPLE_KEYS = ('t', 'r', 'th', 'ph', 'sig', 'mino')


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class BatchPlan:
    """One batch of images: the plan, its workspace and its concatenated outputs."""

    def __init__(self, images, precision='mixed', r_o=1.e4, maxtaufrac=1.0 - 1.0e-10, keys=SAMPLE_KEYS,
                 device='cuda'):
        require_cuda()
        self.lib = _lib.load()
        self.dev = torch.device(device)
        n = len(images)
        arr = (_lib.BatchImage * max(n, 1))()
        for i, im in enumerate(images):
            arr[i] = _lib.BatchImage(float(im['a']), float(im.get('r_o', r_o)), float(im['th_o']), int(im['npix']),
                                     int(im['ngeo']), 0, float(im.get('maxtaufrac', maxtaufrac)))
        self.images = [dict(im) for im in images]
        self.handle = ctypes.c_void_p(0)
        _lib.check(self.lib.kgeo_batch_create(arr, n, PRECISION[precision], ctypes.byref(self.handle)))
        nr, ns, wb = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_size_t(0)
        _lib.check(self.lib.kgeo_batch_sizes(self.handle, ctypes.byref(nr), ctypes.byref(ns), ctypes.byref(wb)))
        self.n_rays, self.n_samples, self.ws_bytes = nr.value, ns.value, wb.value
        self.ws = torch.empty(max(self.ws_bytes, 8), dtype=torch.uint8, device=self.dev)
        self.out = {k: torch.empty(self.n_samples, dtype=torch.float64, device=self.dev) for k in keys}
        self.tau_tot = torch.empty(self.n_rays, dtype=torch.float64, device=self.dev)
        self.rclass = torch.empty(self.n_rays, dtype=torch.int32, device=self.dev)
        self.thclass = torch.empty(self.n_rays, dtype=torch.int32, device=self.dev)
        self.flags = torch.zeros(max(n, 1), dtype=torch.int32, device=self.dev)  # per image, after each run
        self.pix_off, self.out_off = [], []
        po = so = 0
        for im in images:
            self.pix_off.append(po)
            self.out_off.append(so)
            po += int(im['npix'])
            so += int(im['npix']) * int(im['ngeo'])
        self.alpha = self.beta = None

    def _stream(self, stream):
        return ctypes.c_void_p((stream if stream is not None else torch.cuda.current_stream(self.dev)).cuda_stream)

    def bind(self, alpha, beta):
        """Attach the concatenated pixel coordinates (float64 CUDA tensors of n_rays values)."""
        if alpha.numel() != self.n_rays or beta.numel() != self.n_rays:
            raise Exception("alpha, beta are different lengths!")
        self.alpha = alpha.to(device=self.dev, dtype=torch.float64).contiguous()
        self.beta = beta.to(device=self.dev, dtype=torch.float64).contiguous()
        g = _lib.GeodesicsOut(*[_ptr(self.out.get(k)) for k in SAMPLE_KEYS], _ptr(self.tau_tot), _ptr(self.rclass),
                              _ptr(self.thclass), _ptr(self.flags))
        _lib.check(self.lib.kgeo_batch_bind(self.handle, _ptr(self.alpha), _ptr(self.beta), ctypes.byref(g),
                                            _ptr(self.ws), self.ws_bytes))
        return self

    @property
    def config(self):
        c, tuned = _lib.BatchConfig(), ctypes.c_int32(0)
        _lib.check(self.lib.kgeo_batch_get_config(self.handle, ctypes.byref(c), ctypes.byref(tuned)))
        return dict(block=c.block, ctas_per_sm=c.ctas_per_sm, tile=c.tile, chunk=c.chunk, tuned=bool(tuned.value))

    @config.setter
    def config(self, cfg):
        c = _lib.BatchConfig(int(cfg['block']), int(cfg['ctas_per_sm']), int(cfg['tile']), int(cfg['chunk']))
        _lib.check(self.lib.kgeo_batch_set_config(self.handle, ctypes.byref(c)))

    def autotune(self, budget_ms=2000, stream=None):
        c = _lib.BatchConfig()
        _lib.check(self.lib.kgeo_batch_autotune(self.handle, int(budget_ms), self._stream(stream), ctypes.byref(c)))
        return self.config

    def run(self, stream=None):
        _lib.check(self.lib.kgeo_batch_run(self.handle, self._stream(stream)))

    def graph_launch(self, stream=None):
        _lib.check(self.lib.kgeo_batch_graph_launch(self.handle, self._stream(stream)))

    def image(self, i):
        """Views of image i's outputs: samples (ngeo, npix), per-ray (npix)."""
        npix, ngeo = int(self.images[i]['npix']), int(self.images[i]['ngeo'])
        so, po = self.out_off[i], self.pix_off[i]
        res = {k: v[so:so + ngeo * npix].view(ngeo, npix) for k, v in self.out.items()}
        res.update(tau_tot=self.tau_tot[po:po + npix], rclass=self.rclass[po:po + npix],
                   thclass=self.thclass[po:po + npix], flags=self.flags[i:i + 1])
        return res

    def check_flags(self):
        """Host check of every image's flags word after a run (synchronises): warns when an
        iterative loop stopped at its cap (KGEO_FLAG_LOOP_CAP)."""
        from .kerr_raytracing_ana import warn_loop_cap
        f = 0
        for v in self.flags[:len(self.images)].tolist():
            f |= int(v)
        warn_loop_cap(f)
        return f

    def close(self):
        if self.handle:
            self.lib.kgeo_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
