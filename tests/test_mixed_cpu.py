"""CPU checks of the mixed-precision recurrence's arithmetic (the device headers built for the
host): the float-float operations against FP64, the float-float log ratio and the R_C series,
and the whole float-float recurrence against the oracle at the mixed-precision bars."""
import ctypes

import numpy as np
import pytest

import hmlib
from oracle import kgeo_oracle as ko
from parity import rel_err


def _lib():
    L = hmlib.load()
    L.hm_ff_ops.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    L.hm_ff_logratio.restype = ctypes.c_double
    L.hm_ff_logratio.argtypes = [ctypes.c_double]
    L.hm_rc_one_m1.restype = ctypes.c_double
    L.hm_rc_one_m1.argtypes = [ctypes.c_double]
    return L


def test_float_float_operations():
    L = _lib()
    rng = np.random.default_rng(4)
    out = np.zeros(9)
    worst = np.zeros(7)
    for _ in range(3000):
        a = rng.uniform(-3, 3) * 10 ** rng.uniform(-3, 3)
        b = rng.uniform(-3, 3) * 10 ** rng.uniform(-3, 3)
        L.hm_ff_ops(a, b, hmlib.dp(out))
        A, B = out[7], out[8]   # the split values (48 bits of a, b)
        assert abs(A - a) <= 4e-15 * abs(a) and abs(B - b) <= 4e-15 * abs(b)
        ref = [A + B, A - B, A * B, A / B, 1 / A, A * A, 1 - A]
        scale = [abs(A) + abs(B), abs(A) + abs(B), abs(A * B), abs(A / B), abs(1 / A), A * A, 1 + abs(A)]
        for k in range(7):
            worst[k] = max(worst[k], abs(out[k] - ref[k]) / scale[k])
    assert worst.max() <= 3e-14, worst


def test_float_float_logratio_and_series():
    L = _lib()
    for a in np.concatenate([np.linspace(-0.98, 0.98, 97), 1 / np.linspace(-0.98, 0.98, 96)[::5]]):
        ref = np.log(abs((1 + a) / (1 - a)))
        # float-float argument and leading term, FP32 series tail: ~1e-8 of the value
        assert abs(L.hm_ff_logratio(a) - ref) <= 3e-8 * max(1.0, abs(ref)), a
    for e in np.linspace(-0.25, 0.25, 51):
        if e == 0:
            continue
        ref = (np.arctan(np.sqrt(e)) / np.sqrt(e) if e > 0 else np.arctanh(np.sqrt(-e)) / np.sqrt(-e)) - 1
        assert abs(L.hm_rc_one_m1(e) - ref) <= 3e-7 * abs(ref), e


def _host_mixed(a, r_o, th_o, A, B, ngeo, chunk=256):
    L = hmlib.load()
    nf = L.hm_num_fields()
    n = len(A)
    ob = hmlib.observer(a, r_o, th_o)
    rec = np.zeros(nf * n)
    code, rc, tc = (np.zeros(n, np.int32) for _ in range(3))
    A = np.ascontiguousarray(A, float)
    B = np.ascontiguousarray(B, float)
    L.hm_setup.restype = ctypes.c_uint
    flags = L.hm_setup(hmlib.dp(ob), hmlib.dp(A), hmlib.dp(B), ctypes.c_long(n), ctypes.c_double(1 - 1e-10),
                       hmlib.dp(rec), hmlib.ip(code), hmlib.ip(rc), hmlib.ip(tc), ctypes.c_long(ngeo))
    outs = [np.zeros((ngeo, n)) for _ in range(6)]
    L.hm_samples_mixed(hmlib.dp(ob), hmlib.dp(rec), hmlib.ip(code), ctypes.c_long(n), ctypes.c_long(ngeo),
                       ctypes.c_long(chunk), ctypes.c_int(flags & 1), *[hmlib.dp(o) for o in outs])
    return dict(zip(['t', 'r', 'th', 'ph', 'sig', 'mino'], outs))


@pytest.mark.parametrize('geom', [(0.94, 17.0, 128, 10.0), (0.3, 70.0, 64, 10.0), (0.94, 17.0, 256, 2.5),
                                  (0.5, 60.0, 256, 2.5)])
def test_host_mixed_recurrence_error_bars(geom):
    # the 2.5 M boxes hold the vortical rays and the near-unit Pi characteristics of the centre
    a, th, chunk, lim = geom[0], geom[1] * np.pi / 180, geom[2], geom[3]
    x = np.linspace(-lim, lim, 20)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    ref = ko.raytrace(a, 1.e4, th, A, B, 200)
    got = _host_mixed(a, 1.e4, th, A, B, 200, chunk)
    last = np.zeros(ref['r'].shape, bool)
    last[-1] = np.isin(ref['rclass'], (2, 3, 4))
    # near an elliptic-Pi pole the float-float state's rounding is amplified by 1 / rho
    rho = ko.pole_distance(a, 1.e4, th, A, B, got['mino'])
    for k, rk, scale, bar in (('r', 'r', 1e-300, 1e-9), ('th', 'th', 1.0, 5e-7), ('ph', 'ph', 1.0, 1e-6),
                              ('t', 't', 1.e4, 1e-7), ('sig', 'affine_times', 1.e4, 1e-7)):
        e = rel_err(got[k], ref[rk], scale) / np.maximum(bar, 1e-12 / rho)
        assert e[~last].max() <= 1.0, (k, e[~last].max())
