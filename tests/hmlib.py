"""Loader of tests/hostmath (the kernels' device headers built for the host by g++) and the
image entry points of it, shared by the CPU tests. Test-only."""
import ctypes
import glob
import os
import subprocess

import numpy as np

from conftest import ROOT

LIBPATH = os.path.join(ROOT, 'tests', 'hostmath', 'libhostmath.so')
D = ctypes.c_double
P = ctypes.POINTER
_L = None

EMIS = {'bpl': 0, 'constant': 1, 'glm': 2, 'ring': 3}
VEL = {'zamo': 0, 'infall': 1, 'kep': 2, 'subkep': 3, 'general': 4}


def load():
    global _L
    if _L is None:
        src = os.path.join(ROOT, 'tests', 'hostmath', 'hostmath.cpp')
        deps = [src] + glob.glob(os.path.join(ROOT, 'kgeo_gb300', 'csrc', '*.cuh'))
        if not os.path.exists(LIBPATH) or os.path.getmtime(LIBPATH) < max(os.path.getmtime(p) for p in deps):
            subprocess.run(['g++', '-O2', '-ffp-contract=off', '-std=c++17', '-shared', '-fPIC', '-o', LIBPATH, src],
                           check=True)
        _L = ctypes.CDLL(LIBPATH)
    return _L


def dp(a):
    return a.ctypes.data_as(P(D))


def ip(a):
    return a.ctypes.data_as(P(ctypes.c_int))


def observer(a, r_o, th_o):
    return np.array([a, a ** 2, r_o, th_o, np.sin(th_o), np.cos(th_o), np.cos(th_o) ** 2, 1 + np.sqrt(1 - a ** 2),
                     1 - np.sqrt(1 - a ** 2), float(abs(a) < 1e-4), float(r_o == np.inf)])


def model_arrays(emis, vel, specind=1.0, sinthb=np.pi / 4):
    """(mi, md) of hostmath's image functions from ('bpl', kwargs), ('general', kwargs)."""
    et, ek = emis
    vt, vk = vel
    if et == 'bpl':
        ep = [ek.get('p1', -2.0), ek.get('p2', -0.5)]
    elif et == 'glm':
        ep = [ek.get('gamma_off', -1.5), ek.get('sigma', 0.5)]
    elif et == 'ring':
        ep = [ek.get('gamma_off', 0), ek.get('sigma', 0.3)]
    else:
        ep = [0.0, 0.0]
    mu = ek.get('r_ring', 4.5) if et == 'ring' else 0.0
    vp = [vk.get('fac_subkep', 1), vk.get('beta_phi', 1), vk.get('beta_r', 1)]
    mi = np.array([EMIS[et], VEL[vt], int(vk.get('retrograde', False))], np.int32)
    md = np.array(ep + [mu] + vp + [ek.get('emiscut_in', 0), ek.get('emiscut_out', 1e10), specind, sinthb], float)
    return mi, md


def image(a, r_o, th_o, alpha, beta, nord, mi, md):
    L = load()
    n = len(alpha)
    ob = observer(a, r_o, th_o)
    alpha = np.ascontiguousarray(alpha, float)
    beta = np.ascontiguousarray(beta, float)
    outs = [np.zeros((n, nord)) for _ in range(5)] + [np.zeros(n), np.zeros(n)]
    L.hm_image(dp(ob), ip(mi), dp(md), dp(alpha), dp(beta), ctypes.c_long(n), ctypes.c_int(nord),
               *[dp(o) for o in outs])
    return dict(zip(['I', 'g', 'r_s', 'Ir', 'sinthb', 'nmax', 'npol'], outs))


BFIELD = {'simple': 0, 'rad': 0, 'vert': 0, 'tor': 0, 'simple_rm1': 1, 'monopoleA': 2, 'bz_guess': 3,
          'bz_monopole': 4, 'bz_para': 5, 'power': 6, 'gen_power': 7}


def field_arrays(fieldtype, kw):
    """(field, flag, c[3]) of a Bfield(fieldtype, **kw), the kgeo_bfield encoding."""
    flag = 0
    if fieldtype in ('rad', 'vert', 'tor'):
        c = {'rad': [1, 0, 0], 'vert': [0, 1, 0], 'tor': [0, 0, 1]}[fieldtype]
    elif fieldtype in ('simple', 'simple_rm1'):
        c = [kw.get('Cr', 0), kw.get('Cvert', 0), kw.get('Cph', 0)]
    elif fieldtype == 'monopoleA':
        c = [kw.get('C', 1), kw.get('omegafac', 0.5), 0]
    elif fieldtype in ('bz_guess', 'bz_para'):
        c = [kw.get('C', 1), 0, 0]
    elif fieldtype == 'bz_monopole':
        c = [kw.get('C', 1), 0, 0]
        flag = int(bool(kw.get('secondorder_only', False)))
    elif fieldtype == 'power':
        c = [kw.get('C', 1), kw.get('p', 1), 0]
        flag = int(bool(kw.get('usemono', False)))
    else:
        c = [kw.get('n_I', 0), kw.get('p_val', 1), 0]
        flag = int(bool(kw.get('isAbove', True)))
    return BFIELD[fieldtype], flag, np.array(c, float)


def image_opts(a, r_o, th_o, alpha, beta, nord, mi, md, bfield=('rad', {}), polarization=True, pathlength=False,
               diskangle=0.1):
    L = load()
    n = len(alpha)
    ob = observer(a, r_o, th_o)
    alpha = np.ascontiguousarray(alpha, float)
    beta = np.ascontiguousarray(beta, float)
    f, flag, c = field_arrays(*bfield)
    oi = np.array([int(polarization), int(pathlength), f, flag], np.int32)
    od = np.array([diskangle, c[0], c[1], c[2]], float)
    outs = [np.zeros((n, nord)) for _ in range(7)]
    L.hm_image_opts(dp(ob), ip(mi), dp(md), ip(oi), dp(od), dp(alpha), dp(beta), ctypes.c_long(n),
                    ctypes.c_int(nord), *[dp(o) for o in outs])
    return dict(zip(['I', 'Q', 'U', 'g', 'sinthb', 'lp', 'Ie'], outs))


def bfield(a, r, fieldtype, kw):
    L = load()
    f, flag, c = field_arrays(fieldtype, kw)
    r = np.ascontiguousarray(r, float)
    out = np.zeros((len(r), 3))
    L.hm_bfield(ctypes.c_int(f), ctypes.c_int(flag), dp(c), D(a), dp(r), ctypes.c_long(len(r)), dp(out))
    return out.T


def curve_rho(a, th0, r_eq, mbar, varphi, bracket, xtol=2e-12, rtol=4 * np.finfo(float).eps, maxiter=100):
    """The curve kernel's Brent solve (host build) at each angle: (rho, status)."""
    L = load()
    ob = observer(a, np.inf, th0)
    varphi = np.ascontiguousarray(varphi, float)
    rho = np.zeros(len(varphi))
    st = np.zeros(len(varphi), np.int32)
    L.hm_curve_rho(dp(ob), D(r_eq), ctypes.c_int(mbar), D(bracket[0]), D(bracket[1]), dp(varphi),
                   ctypes.c_long(len(varphi)), D(xtol), D(rtol), ctypes.c_int(maxiter), dp(rho), ip(st))
    return rho, st


def lambert_w0(z):
    L = load()
    L.hm_lambert_w0.restype = D
    return L.hm_lambert_w0(D(z))


def re_li2(x):
    L = load()
    L.hm_re_li2.restype = D
    return L.hm_re_li2(D(x))


def image_jac(a, r_o, th_o, alpha, beta, nord, mi, md):
    L = load()
    n = len(alpha)
    ob = observer(a, r_o, th_o)
    alpha = np.ascontiguousarray(alpha, float)
    beta = np.ascontiguousarray(beta, float)
    jac = np.zeros((n, nord, 7))
    rsd = np.zeros((n, nord, 2))
    L.hm_image_jac(dp(ob), ip(mi), dp(md), dp(alpha), dp(beta), ctypes.c_long(n), ctypes.c_int(nord), dp(jac),
                   dp(rsd))
    return jac, rsd


def jet_stagnation(a, th):
    """(status, r0, Omega_F) of the stagnation solve (host build)."""
    L = load()
    out = np.zeros(2)
    st = L.hm_jet_stagnation(D(a), D(th), dp(out))
    return st, out[0], out[1]


def jet_stokes(a, r_o, th_o, field, nu, sigma, r0, specind, alpha, beta, r, th, kr, kth):
    """Per crossing (I, Q, U) of the jet emission kernel (host build); field 0 monopole, 1 power p = 0."""
    L = load()
    ob = observer(a, r_o, th_o)
    par = np.array([field, nu, sigma, r0, specind], float)
    arrs = [np.ascontiguousarray(x, float) for x in (alpha, beta, r, th, kr, kth)]
    n = len(arrs[0])
    out = np.zeros((n, 3))
    L.hm_jet_stokes(dp(ob), dp(par), *[dp(x) for x in arrs], ctypes.c_long(n), dp(out))
    return out.T
