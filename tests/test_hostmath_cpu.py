"""CPU checks of the kernels' arithmetic: the same headers the CUDA kernels compile
(kgeo_gb300/csrc/*.cuh), built for the host by g++ (tests/hostmath), against scipy,
mpmath and the reference fixtures. The GPU tests repeat the parity checks on sm_103a."""
import ctypes
import glob
import os
import subprocess

import numpy as np
import pytest
import scipy.special as sp

from conftest import GOLDEN, ROOT
from parity import check_trace

LIBPATH = os.path.join(ROOT, 'tests', 'hostmath', 'libhostmath.so')
D = ctypes.c_double
P = ctypes.POINTER


@pytest.fixture(scope='module')
def hm():
    src = os.path.join(ROOT, 'tests', 'hostmath', 'hostmath.cpp')
    deps = [src] + glob.glob(os.path.join(ROOT, 'kgeo_gb300', 'csrc', '*.cuh'))
    if not os.path.exists(LIBPATH) or os.path.getmtime(LIBPATH) < max(os.path.getmtime(p) for p in deps):
        subprocess.run(['g++', '-O2', '-ffp-contract=off', '-std=c++17', '-shared', '-fPIC', '-o', LIBPATH, src],
                       check=True)
    L = ctypes.CDLL(LIBPATH)
    for n in ('hm_rf', 'hm_rj', 'hm_rd', 'hm_rc', 'hm_ellipf', 'hm_ellipe', 'hm_ellippi'):
        getattr(L, n).restype = D
    L.hm_rf.argtypes = [D, D, D]
    L.hm_rj.argtypes = [D, D, D, D]
    L.hm_rd.argtypes = [D, D, D]
    L.hm_rc.argtypes = [D, D]
    L.hm_ellipf.argtypes = [D, D]
    L.hm_ellipe.argtypes = [D, D]
    L.hm_ellippi.argtypes = [D, D, D]
    L.hm_setup.restype = ctypes.c_uint
    return L


def dp(a):
    return a.ctypes.data_as(P(D))


def ip(a):
    return a.ctypes.data_as(P(ctypes.c_int))


def observer(a, r_o, th_o):
    return np.array([a, a ** 2, r_o, th_o, np.sin(th_o), np.cos(th_o), np.cos(th_o) ** 2, 1 + np.sqrt(1 - a ** 2),
                     1 - np.sqrt(1 - a ** 2), float(abs(a) < 1e-4), float(r_o == np.inf)])


def host_trace(L, a, r_o, th_o, alpha, beta, ngeo, maxtaufrac=1 - 1e-10):
    n = len(alpha)
    nf = L.hm_num_fields()
    ob = observer(a, r_o, th_o)
    rec = np.zeros(nf * n)
    code, rc, tc = (np.zeros(n, np.int32) for _ in range(3))
    alpha = np.ascontiguousarray(alpha, float)
    beta = np.ascontiguousarray(beta, float)
    flags = L.hm_setup(dp(ob), dp(alpha), dp(beta), ctypes.c_long(n), D(maxtaufrac), dp(rec), ip(code), ip(rc), ip(tc), ctypes.c_long(ngeo))
    tau = np.ascontiguousarray(np.linspace(0, rec.reshape(nf, n)[2], ngeo))
    outs = [np.zeros((ngeo, n)) for _ in range(5)]
    L.hm_samples(dp(ob), dp(rec), ip(code), ctypes.c_long(n), dp(tau), ctypes.c_long(ngeo), ctypes.c_int(flags & 1),
                 *[dp(o) for o in outs])
    t, r, th, ph, sig = outs
    return dict(t=t, r=r, th=th, ph=ph, sig=sig, rclass=rc, thclass=tc)


def host_trace_stepped(L, a, r_o, th_o, alpha, beta, ngeo, chunk, maxtaufrac=1 - 1e-10):
    n = len(alpha)
    nf = L.hm_num_fields()
    ob = observer(a, r_o, th_o)
    rec = np.zeros(nf * n)
    code, rc, tc = (np.zeros(n, np.int32) for _ in range(3))
    alpha = np.ascontiguousarray(alpha, float)
    beta = np.ascontiguousarray(beta, float)
    flags = L.hm_setup(dp(ob), dp(alpha), dp(beta), ctypes.c_long(n), D(maxtaufrac), dp(rec), ip(code), ip(rc), ip(tc),
                       ctypes.c_long(ngeo))
    outs = [np.zeros((ngeo, n)) for _ in range(6)]
    L.hm_samples_stepped(dp(ob), dp(rec), ip(code), ctypes.c_long(n), ctypes.c_long(ngeo), ctypes.c_long(chunk),
                         ctypes.c_int(flags & 1), *[dp(o) for o in outs])
    t, r, th, ph, sig, mino = outs
    return dict(t=t, r=r, th=th, ph=ph, sig=sig, mino=mino)


def host_trace_rth(L, a, r_o, th_o, alpha, beta, ngeo, chunk, maxtaufrac=1 - 1e-10):
    n = len(alpha)
    nf = L.hm_num_fields()
    ob = observer(a, r_o, th_o)
    rec = np.zeros(nf * n)
    code, rc, tc = (np.zeros(n, np.int32) for _ in range(3))
    alpha = np.ascontiguousarray(alpha, float)
    beta = np.ascontiguousarray(beta, float)
    flags = L.hm_setup(dp(ob), dp(alpha), dp(beta), ctypes.c_long(n), D(maxtaufrac), dp(rec), ip(code), ip(rc), ip(tc),
                       ctypes.c_long(ngeo))
    outs = [np.zeros((ngeo, n)) for _ in range(3)]
    L.hm_samples_rth(dp(ob), dp(rec), ip(code), ctypes.c_long(n), ctypes.c_long(ngeo), ctypes.c_long(chunk),
                     ctypes.c_int(flags & 1), *[dp(o) for o in outs])
    r, th, mino = outs
    return dict(r=r, th=th, mino=mino)


def rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def test_carlson_vs_scipy(hm):
    rng = np.random.default_rng(0)
    x, y, z, p = rng.uniform(0, 3, (4, 3000))
    x[:50] = 0
    assert rel(np.array([hm.hm_rf(*v) for v in zip(x, y, z)]), sp.elliprf(x, y, z)) < 4e-15
    assert rel(np.array([hm.hm_rj(*v) for v in zip(x, y, z, p)]), sp.elliprj(x, y, z, p)) < 4e-15
    assert rel(np.array([hm.hm_rd(*v) for v in zip(x, y, z)]), sp.elliprd(x, y, z)) < 4e-15
    u, v = rng.uniform(0.01, 3, (2, 2000))
    assert rel(np.array([hm.hm_rc(*w) for w in zip(u, v)]), sp.elliprc(u, v)) < 4e-15
    assert rel(np.array([hm.hm_rc(*w) for w in zip(u, -v)]), sp.elliprc(u, -v)) < 4e-15


def test_incomplete_integrals_vs_scipy(hm):
    rng = np.random.default_rng(1)
    phi = rng.uniform(-20, 20, 4000)
    m = rng.uniform(-50, 0.999, 4000)
    assert rel(np.array([hm.hm_ellipf(*v) for v in zip(phi, m)]), sp.ellipkinc(phi, m)) < 5e-15
    assert rel(np.array([hm.hm_ellipe(*v) for v in zip(phi, m)]), sp.ellipeinc(phi, m)) < 5e-15


def test_ellip_pi_adapter_vs_reference_fixture(hm, golden):
    g = golden('ellip_pi')
    got = np.array([hm.hm_ellippi(*v) for v in zip(g['n'], g['phi'], g['m'])])
    ref = g['pi']
    assert np.array_equal(np.isfinite(got), np.isfinite(ref))
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    fin = np.isfinite(ref)
    # Pi at |phi| > pi is a sum of O(1) periodic and incomplete parts: absolute scale 1
    assert np.max(np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)) < 1e-13


def test_jacobi_vs_mpmath(hm):
    import mpmath as mpm
    rng = np.random.default_rng(2)
    out = np.zeros(3)
    mpm.mp.dps = 30
    for m in list(rng.uniform(0, 0.999, 40)) + list(1 - 10 ** rng.uniform(-12, -3, 20)):
        K = sp.ellipk(m)
        u = rng.uniform(-1, 1) * K
        hm.hm_jacobi(D(u), D(m), dp(out))
        for val, name in zip(out, ('sn', 'cn', 'dn')):
            assert abs(val - float(mpm.ellipfun(name, u, m=m))) < 2e-14


@pytest.mark.parametrize('name', sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, 'trace_*.npz'))))
def test_host_trace_vs_reference_fixture(hm, golden, name):
    g = golden(name)
    a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
    out = host_trace(hm, a, r_o, th_o, g['alpha'], g['beta'], int(g['ngeo']))
    assert np.array_equal(out['rclass'], g['rclass'])
    assert np.array_equal(out['thclass'], g['thclass'])
    if np.isfinite(r_o):
        from oracle import kgeo_oracle as ko
        rho = ko.pole_distance(a, r_o, th_o, g['alpha'], g['beta'], g['mino'])
        check_trace(out, dict(t=g['t'], r=g['r'], th=g['th'], ph=g['ph'], sig=g['sig']), r_o, g['rclass'], name, rho=rho)
        st = host_trace_stepped(hm, a, r_o, th_o, g['alpha'], g['beta'], int(g['ngeo']), 50)
        check_trace(st, dict(t=g['t'], r=g['r'], th=g['th'], ph=g['ph'], sig=g['sig']), r_o, g['rclass'],
                    name + '-recurrence', rho=rho)
        # theta and r alone (the sample kernel's path when t, phi and sigma are not requested),
        # against the same bars; the other three are taken from the fixture
        rth = host_trace_rth(hm, a, r_o, th_o, g['alpha'], g['beta'], int(g['ngeo']), 64)
        assert np.array_equal(rth['mino'], st['mino'])
        check_trace(dict(r=rth['r'], th=rth['th'], t=g['t'], ph=g['ph'], sig=g['sig']),
                    dict(t=g['t'], r=g['r'], th=g['th'], ph=g['ph'], sig=g['sig']), r_o, g['rclass'],
                    name + '-rth', rho=rho)


def test_recurrence_late_in_chunk_next_to_radial_pi_pole(hm):
    """conftest.PI_ZONE_RAYS through the host build of the FP64 recurrence (chunks of 64)
    against the oracle."""
    from conftest import PI_ZONE_RAYS
    from oracle import kgeo_oracle as ko
    a, r_o, th_o, ngeo = 0.94, 1.e4, 17 * np.pi / 180, 256
    x = np.linspace(-10, 10, 2048)
    alpha = np.array([x[j] for i, j in PI_ZONE_RAYS])
    beta = np.array([x[i] for i, j in PI_ZONE_RAYS])
    ref = ko.raytrace(a, r_o, th_o, alpha, beta, ngeo)
    rho = ko.pole_distance(a, r_o, th_o, alpha, beta, ref['mino_times'])
    assert rho[:, 0].min() < 1.5e-3
    st = host_trace_stepped(hm, a, r_o, th_o, alpha, beta, ngeo, 64)
    check_trace(st, dict(t=ref['t'], r=ref['r'], th=ref['th'], ph=ref['ph'], sig=ref['affine_times']), r_o,
                ref['rclass'], 'pi-zone-recurrence', rho=rho)


@pytest.mark.parametrize('case', ['config2', 'vortical', 'south', 'region2'])
def test_observer_states_match_direct_evaluation(hm, case):
    """The recurrence starts its first chunk from the observer's states that the setup stores
    (theta sn, cn, dn, e, pi at the amplitude -s arg or -s h nu_o; r sn, cn, dn, E, Pi at aux):
    they equal the direct evaluation at tau = 0 to rounding."""
    import bench
    if case == 'config2':
        a, th_o, A, B = bench.workload(0)
        A, B = A[::41], B[::41]
    else:
        a, th_o = {'vortical': (0.99, 2.0), 'south': (0.7, 150.0), 'region2': (0.81, 99.0)}[case]
        th_o *= np.pi / 180
        x = np.linspace(-12, 12, 61)
        A, B = (v.ravel() for v in np.meshgrid(x, x))
    A = np.ascontiguousarray(A, float)
    B = np.ascontiguousarray(B, float)
    n = A.size
    nf = hm.hm_num_fields()
    ob = observer(a, 1.e4, th_o)
    rec = np.zeros(nf * n)
    code, rc, tc = (np.zeros(n, np.int32) for _ in range(3))
    hm.hm_setup(dp(ob), dp(A), dp(B), ctypes.c_long(n), D(1 - 1e-10), dp(rec), ip(code), ip(rc), ip(tc),
                ctypes.c_long(200))
    out = np.full(n * 10, np.nan)
    hm.hm_seed_check(dp(rec), ip(code), ctypes.c_long(n), dp(out))
    out = out.reshape(n, 10)
    stepping = ((code >> 10) & 1).astype(bool)
    assert stepping.sum() > n // 2
    d = np.abs(out[stepping])
    assert np.isfinite(d[:, :9]).all()
    # sn, cn, dn, E and theta's e to a few ulps; the Pi (relative to max(1, |Pi|)) to a few ulps
    # over the pole distance, the bar of either evaluation near a pole
    assert d[:, [0, 1, 2, 3, 5, 6, 7, 8]].max() <= 2e-13, d[:, [0, 1, 2, 3, 5, 6, 7, 8]].max(axis=0)
    assert d[:, 4].max() <= 2e-14, d[:, 4].max()
    assert np.nanmax(d[:, 9]) <= 2e-14, np.nanmax(d[:, 9])
