"""Failure reporting of the iterative device arithmetic, tested on the host build of the same
source (tests/hostmath): a Carlson duplication or Landen descent that stops at its iteration
cap without converging records KGEO_FLAG_LOOP_CAP (the kernels collect it into the launch's
flags word; the Python drop-ins turn it into a ConvergenceWarning), and never loops past the
cap. The forced case rebuilds the harness with both caps set to 1 and runs it in a child
process under a time limit, so a hang fails the test instead of stalling the suite."""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, 'tests', 'hostmath', 'hostmath.cpp')
FLAG_LOOP_CAP = 16


def _build(out, defines=()):
    cmd = ['g++', '-O2', '-ffp-contract=off', '-std=c++17', '-shared', '-fPIC', *defines, '-o', out, SRC]
    subprocess.run(cmd, check=True)


CHILD = textwrap.dedent('''
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, {tests!r})
    import test_hostmath_cpu as T
    L = ctypes.CDLL({lib!r})
    L.hm_setup.restype = ctypes.c_uint
    L.hm_rf.restype = ctypes.c_double
    L.hm_rf.argtypes = [ctypes.c_double] * 3
    out = {{}}
    L.hm_take_loop_cap()
    v = L.hm_rf(0.0, 1e-3, 1.0)
    out['rf'] = L.hm_take_loop_cap()
    j = np.zeros(3)
    L.hm_jacobi(ctypes.c_double(0.7), ctypes.c_double(0.999999), T.dp(j))
    out['jacobi'] = L.hm_take_loop_cap()
    x = np.linspace(-6, 6, 5)
    A, B = (g.flatten() for g in np.meshgrid(x, x))
    tr = T.host_trace(L, 0.9, 1e4, 0.5, A, B, 8)
    out['trace'] = L.hm_take_loop_cap()
    out['finite_r'] = int(np.isfinite(tr['r']).all())
    print(out)
''')


def test_loop_cap_flag_clear_on_regular_inputs(tmp_path):
    """The regular build: traces of ordinary, vortical and horizon-bound rays (a = 0 included)
    and the reference's elliptic-Pi points reach no cap."""
    sys.path.insert(0, os.path.join(ROOT, 'tests'))
    import test_hostmath_cpu as T
    lib = str(tmp_path / 'libhm.so')
    _build(lib)
    L = ctypes.CDLL(lib)
    L.hm_setup.restype = ctypes.c_uint
    L.hm_ellippi.restype = ctypes.c_double
    L.hm_ellippi.argtypes = [ctypes.c_double] * 3
    L.hm_take_loop_cap()
    x = np.linspace(-9, 9, 21)
    A, B = (g.flatten() for g in np.meshgrid(x, x))
    T.host_trace(L, 0.94, 1e4, 17 * np.pi / 180, A, B, 32)
    T.host_trace_stepped(L, 0.5, 1e4, 80 * np.pi / 180, A, B, 32, 16)
    # a = 0: r_- = r_1 = 0 makes one radial characteristic infinite (its Pi is the adapter's 0)
    T.host_trace(L, 0.0, 1e4, 45 * np.pi / 180, A, B, 16)
    T.host_trace_stepped(L, 0.0, 1e4, 45 * np.pi / 180, A, B, 16, 8)
    g = np.load(os.path.join(ROOT, 'tests', 'golden', 'ellip_pi.npz'))
    for n, phi, m in zip(g['n'], g['phi'], g['m']):
        L.hm_ellippi(n, phi, m)
    assert L.hm_take_loop_cap() == 0


def test_forced_cap_sets_flag_and_returns(tmp_path):
    """Caps forced to 1: every evaluation stops after one step, records the flag, and the
    whole trace still returns (finite, inaccurate) values."""
    lib = str(tmp_path / 'libhm_cap1.so')
    _build(lib, ['-DKG_CARLSON_MAX_IT=1', '-DKG_LANDEN_MAX=1'])
    code = CHILD.format(tests=os.path.join(ROOT, 'tests'), lib=lib)
    r = subprocess.run([sys.executable, '-c', code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = eval(r.stdout.strip().splitlines()[-1])
    assert out['rf'] == FLAG_LOOP_CAP
    assert out['jacobi'] == FLAG_LOOP_CAP
    assert out['trace'] == FLAG_LOOP_CAP
    assert out['finite_r'] == 1


def test_python_layer_warns_on_the_flag():
    from kgeo_gb300 import kerr_raytracing_ana as ka
    with pytest.warns(ka.ConvergenceWarning):
        ka._flags_check(0.5, FLAG_LOOP_CAP)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter('error')
        ka._flags_check(0.5, 1)
