"""kgeo_raytrace_host (host buffers in and out) gives exactly the outputs of kgeo_raytrace /
kgeo_raytrace_mixed on device buffers, on both of its paths: page-locked outputs the kernel
stores into directly, and the window pipeline (samples computed into device buffers, each window
copied while the next computes) that pageable outputs take: FP64 and mixed precision, more
windows than ring buffers, a partial last window, fewer samples than one chunk, empty inputs."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

KEYS = ('t', 'r', 'th', 'ph', 'sig', 'mino', 'tau_tot', 'rclass', 'thclass')


def _pixels(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-9, 9, n), rng.uniform(-9, 9, n)


def _device_reference(a, r_o, th_o, A, B, ngeo, mixed):
    from kgeo_gb300 import _lib
    from kgeo_gb300 import device as dev
    lib = _lib.load()
    al, be = dev.as_device(A), dev.as_device(B)
    npix = A.size
    res = {k: torch.empty((ngeo, npix), dtype=torch.float64, device='cuda') for k in KEYS[:6]}
    res['tau_tot'] = torch.empty(npix, dtype=torch.float64, device='cuda')
    res['rclass'] = torch.empty(npix, dtype=torch.int32, device='cuda')
    res['thclass'] = torch.empty(npix, dtype=torch.int32, device='cuda')
    res['flags'] = torch.zeros(1, dtype=torch.int32, device='cuda')
    g = _lib.GeodesicsOut(*[ctypes.c_void_p(res[k].data_ptr()) for k in KEYS + ('flags',)])
    ob = _lib.Observer(a, r_o, th_o)
    fn = lib.kgeo_raytrace_mixed if mixed else lib.kgeo_raytrace
    _lib.check(fn(ctypes.byref(ob), ctypes.c_void_p(al.data_ptr()), ctypes.c_void_p(be.data_ptr()), npix, ngeo,
                  1.0 - 1e-10, ctypes.byref(g), None, 0, None))
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in res.items()}


@pytest.mark.parametrize('mixed', [False, True])
@pytest.mark.parametrize('ngeo', [400, 333, 7, 1])
def test_host_pipeline_equals_device(ngeo, mixed):
    from kgeo_gb300 import device as dev
    A, B = _pixels(20000, ngeo)
    a, r_o, th_o = 0.83, 1.e4, 37 * np.pi / 180
    ref = _device_reference(a, r_o, th_o, A, B, ngeo, mixed)
    out = dev.trace_host(a, r_o, th_o, A, B, ngeo, mixed=mixed)
    for k in KEYS:
        assert out[k].shape == ref[k].shape, k
        assert np.array_equal(out[k], ref[k], equal_nan=True), k
    assert out['flags'] == int(ref['flags'][0])


def test_host_pipeline_pageable_outputs():
    """Plain numpy (pageable) outputs through the C ABI: the copies serialise but the results
    are the same."""
    from kgeo_gb300 import _lib
    lib = _lib.load()
    A, B = _pixels(5000, 3)
    a, r_o, th_o, ngeo = 0.5, 1.e4, 1.1, 240
    ref = _device_reference(a, r_o, th_o, A, B, ngeo, False)
    out = {k: np.empty((ngeo, A.size)) for k in KEYS[:6]}
    out['tau_tot'] = np.empty(A.size)
    out['rclass'] = np.empty(A.size, np.int32)
    out['thclass'] = np.empty(A.size, np.int32)
    out['flags'] = np.zeros(1, np.int32)
    g = _lib.GeodesicsOut(*[ctypes.c_void_p(out[k].ctypes.data) for k in KEYS + ('flags',)])
    ob = _lib.Observer(a, r_o, th_o)
    _lib.check(lib.kgeo_raytrace_host(ctypes.byref(ob), ctypes.c_void_p(A.ctypes.data), ctypes.c_void_p(B.ctypes.data),
                                      A.size, ngeo, 1.0 - 1e-10, _lib.PRECISION_FP64, ctypes.byref(g), None, 0, None))
    torch.cuda.synchronize()
    for k in KEYS:
        assert np.array_equal(out[k], ref[k], equal_nan=True), k


def test_host_pipeline_raytrace_ana_and_edges():
    from kgeo_gb300.kerr_raytracing_ana import raytrace_ana
    from oracle import kgeo_oracle as ko
    A, B = _pixels(3000, 11)
    g = raytrace_ana(a=0.94, observer_coords=[0, 1.e4, 0.35, 0], image_coords=[A, B], ngeo=120, plotdata=False)
    ref = ko.raytrace(0.94, 1.e4, 0.35, A, B, 120)
    assert np.allclose(g.r_s, ref['r'], rtol=1e-9, equal_nan=True)
    assert isinstance(g.r_s, np.ndarray)
    from kgeo_gb300 import device as dev
    e = dev.trace_host(0.5, 1.e4, 1.0, np.zeros(0), np.zeros(0), 50)
    assert e['r'].shape == (50, 0)
    z = dev.trace_host(0.5, 1.e4, 1.0, A[:10], B[:10], 0)
    assert z['r'].shape == (0, 10)


@pytest.mark.parametrize('mixed', [False, True])
def test_host_pipeline_windows_with_one_pageable_output(mixed):
    """One pageable sample output sends the call through the window pipeline (the other five
    page-locked); the results are the device path's."""
    from kgeo_gb300 import _lib
    lib = _lib.load()
    A, B = _pixels(12000, 5)
    a, r_o, th_o, ngeo = 0.71, 1.e4, 0.9, 333
    ref = _device_reference(a, r_o, th_o, A, B, ngeo, mixed)
    out = {k: torch.empty((ngeo, A.size), dtype=torch.float64, pin_memory=True).numpy() for k in KEYS[:5]}
    out['mino'] = np.empty((ngeo, A.size))
    out['tau_tot'] = np.empty(A.size)
    out['rclass'] = np.empty(A.size, np.int32)
    out['thclass'] = np.empty(A.size, np.int32)
    out['flags'] = np.zeros(1, np.int32)
    g = _lib.GeodesicsOut(*[ctypes.c_void_p(out[k].ctypes.data) for k in KEYS + ('flags',)])
    ob = _lib.Observer(a, r_o, th_o)
    prec = _lib.PRECISION_MIXED if mixed else _lib.PRECISION_FP64
    _lib.check(lib.kgeo_raytrace_host(ctypes.byref(ob), ctypes.c_void_p(A.ctypes.data), ctypes.c_void_p(B.ctypes.data),
                                      A.size, ngeo, 1.0 - 1e-10, prec, ctypes.byref(g), None, 0, None))
    torch.cuda.synchronize()
    for k in KEYS:
        assert np.array_equal(out[k], ref[k], equal_nan=True), k
    assert int(out['flags'][0]) == int(ref['flags'][0])
