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
