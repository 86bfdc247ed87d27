"""kgeo_raytrace_noalloc, the allocation-free variant of kgeo_raytrace.

It serves callers that may not allocate device memory when they call in (a host
application that owns all device memory under a fixed budget, a latency-critical loop that
cannot afford an allocator call, a host with no allocator): its per-ray scratch is a fixed
array inside the library. These tests call both entry points through the C ABI and require
the same results, on two calls in a row (the shared array keeps the previous call's
contents, so the second call checks that nothing stale leaks through). This file is named
to be collected last.
"""
import ctypes

import numpy as np
import pytest

from parity import check_trace

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def env():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kgeo_gb300 import _lib, device as dev
    return torch, _lib, dev


def _run(env, fn_name, a, r_o, th_o, A, B, ngeo):
    torch, _lib, dev = env
    lib = _lib.load()
    al, be = dev.as_device(A), dev.as_device(B)
    npix = A.size
    res = {k: torch.full((ngeo, npix), np.nan, dtype=torch.float64, device='cuda')
           for k in ('t', 'r', 'th', 'ph', 'sig', 'mino')}
    res['tau_tot'] = torch.zeros(npix, dtype=torch.float64, device='cuda')
    res['rclass'] = torch.zeros(npix, dtype=torch.int32, device='cuda')
    res['thclass'] = torch.zeros(npix, dtype=torch.int32, device='cuda')
    res['flags'] = torch.zeros(1, dtype=torch.int32, device='cuda')
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    g = _lib.GeodesicsOut(*[p(res[k]) for k in ('t', 'r', 'th', 'ph', 'sig', 'mino', 'tau_tot', 'rclass',
                                                 'thclass', 'flags')])
    ob = _lib.Observer(a, r_o, th_o)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if fn_name == 'kgeo_raytrace':
        code = lib.kgeo_raytrace(ctypes.byref(ob), p(al), p(be), npix, ngeo, 1 - 1e-10, ctypes.byref(g), None, 0, s)
    else:
        code = lib.kgeo_raytrace_noalloc(ctypes.byref(ob), p(al), p(be), npix, ngeo, 1 - 1e-10, ctypes.byref(g), s)
    assert code == 0, _lib.status_string(code)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in res.items()}


def test_noalloc_matches_raytrace_on_two_calls(env):
    x = np.linspace(-8, 8, 48)
    A1, B1 = (v.flatten() for v in np.meshgrid(x, x))
    rng = np.random.default_rng(5)
    A2, B2 = rng.uniform(-10, 10, 3000), rng.uniform(-10, 10, 3000)
    for (a, r_o, th_o, A, B, ngeo) in [(0.94, 1.e4, 20 * np.pi / 180, A1, B1, 64),
                                       (0.5, 5.e3, 70 * np.pi / 180, A2, B2, 40)]:
        ref = _run(env, 'kgeo_raytrace', a, r_o, th_o, A, B, ngeo)
        got = _run(env, 'kgeo_raytrace_noalloc', a, r_o, th_o, A, B, ngeo)
        assert np.array_equal(got['rclass'], ref['rclass'])
        assert np.array_equal(got['thclass'], ref['thclass'])
        assert np.array_equal(got['flags'], ref['flags'])
        np.testing.assert_allclose(got['tau_tot'], ref['tau_tot'], rtol=1e-10, atol=0)
        np.testing.assert_allclose(got['mino'], ref['mino'], rtol=1e-10, atol=0)
        check_trace(got, ref, r_o, ref['rclass'], 'noalloc')


def test_noalloc_refuses_oversize_before_any_work(env):
    torch, _lib, dev = env
    lib = _lib.load()
    ob = _lib.Observer(0.5, 1.e4, 0.5)
    g = _lib.GeodesicsOut()
    code = lib.kgeo_raytrace_noalloc(ctypes.byref(ob), None, None, 16385, 10, 1 - 1e-10, ctypes.byref(g), None)
    assert code == 11
    assert 'KGEO_NOALLOC_MAX_PIXELS' in _lib.status_string(code)


def _default_pool_used_high(reset):
    """High-water mark of the device's default memory pool (the pool cudaMallocAsync draws
    from), through the CUDA driver API; reset=True sets it back to the current use first."""
    import ctypes
    cu = ctypes.CDLL('libcuda.so.1')
    dev = ctypes.c_int(0)
    assert cu.cuCtxGetDevice(ctypes.byref(dev)) == 0
    pool = ctypes.c_void_p(0)
    assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    used_mem_high = 8  # CU_MEMPOOL_ATTR_USED_MEM_HIGH
    v = ctypes.c_uint64(0)
    if reset:
        assert cu.cuMemPoolSetAttribute(pool, used_mem_high, ctypes.byref(v)) == 0
    assert cu.cuMemPoolGetAttribute(pool, used_mem_high, ctypes.byref(v)) == 0
    return v.value


def test_noalloc_allocates_nothing(env):
    """The defining property: a call draws nothing from the device's memory pool, where
    kgeo_raytrace without a workspace does (stream-ordered cudaMallocAsync)."""
    torch = env[0]
    x = np.linspace(-8, 8, 40)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    torch.cuda.synchronize()
    base = _default_pool_used_high(reset=True)
    _run(env, 'kgeo_raytrace_noalloc', 0.7, 1.e4, 0.6, A, B, 32)
    assert _default_pool_used_high(reset=False) == base
    _run(env, 'kgeo_raytrace', 0.7, 1.e4, 0.6, A, B, 32)
    assert _default_pool_used_high(reset=False) > base
