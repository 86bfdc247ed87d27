"""GPU parity of the lensed-curve library (kgeo_rho_of_req) and the critical curve
(kgeo_critical_curve) through the drop-in equatorial_lensing functions, against the
reference's rho_of_req / make_curves2 / critical_curve fixtures (bars in
tests/test_curves_cpu.py)."""
import ctypes
import os

import numpy as np
import pytest
import torch

from oracle import kgeo_oracle as ko
from test_curves_cpu import DEG, check_roots, curve_cases

pytestmark = pytest.mark.gpu


def test_rho_of_req_fixture(golden):
    from kgeo_gb300.equatorial_lensing import rho_of_req
    g = golden('curves')
    vp = g['varphi']
    for i, a, th0, req, m in curve_cases(g):
        if 'error%d' % i in g:
            with pytest.raises(ValueError, match="f\\(a\\) and f\\(b\\) must have different signs"):
                rho_of_req(a, th0, req, mbar=m, varphis=vp)
            continue
        out = rho_of_req(a, th0, req, mbar=m, varphis=vp)
        assert np.array_equal(out[0], vp)
        check_roots(out[1], g, i, a, th0, req, m, vp)
        assert np.allclose(out[2], np.cos(vp) * out[1]) and np.allclose(out[3], np.sin(vp) * out[1])


def test_rho_of_req_batch_and_single(golden):
    """All fixture curves in one launch give the per-curve results; rho_of_req_single agrees."""
    from kgeo_gb300.equatorial_lensing import rho_of_req, rho_of_req_device, rho_of_req_single
    g = golden('curves')
    vp = g['varphi']
    cases = [c for c in curve_cases(g) if 'error%d' % c[0] not in g]
    rho, st = rho_of_req_device([(a, th0, req, m) for _, a, th0, req, m in cases], vp)
    rho, st = rho.cpu().numpy(), st.cpu().numpy()
    assert (st == 0).all()
    for k, (i, a, th0, req, m) in enumerate(cases):
        assert np.array_equal(rho[k], rho_of_req(a, th0, req, mbar=m, varphis=vp)[1]), i
    i, a, th0, req, m = cases[0]
    assert rho_of_req_single(a, th0, req, vp[5], mbar=m) == rho[0, 5]


def test_library_file(golden, tmp_path):
    """make_curves2's table and file (360 angles, orders 0..2, r_eq = 10, a = 0.5, 30 deg)."""
    from kgeo_gb300.equatorial_lensing import generate_library, make_curves2
    g = golden('curves')
    ref = g['library_a50_i30_r10']
    make_curves2(0, 'r10', 1, 0.5, 30., 2, str(tmp_path))
    fn = os.path.join(str(tmp_path), 'a50_i30_r10.txt')
    tab = np.loadtxt(fn)
    assert tab.shape == ref.shape
    assert np.array_equal(tab[:, 0], ref[:, 0])
    for m in range(3):
        assert np.all(np.abs(tab[:, m + 1] - ref[:, m + 1]) <= 1e-8 * np.abs(ref[:, m + 1])), m
    # a small library: every (spin, inc) file, existing files left alone
    before = os.path.getmtime(fn)
    out = generate_library('r10', outpath=str(tmp_path), spins=np.array([0.5, 0.9]), incs=np.array([30., 60.]),
                           mmax=2)
    assert os.path.getmtime(fn) == before
    assert set(out) == {(0.5, 60.), (0.9, 30.), (0.9, 60.)}
    for (sp, inc), t in out.items():
        assert os.path.isfile(os.path.join(str(tmp_path), 'a%02.0f_i%02.0f_r10.txt' % (100 * sp, inc)))
        assert t.shape == (360, 4) and np.isfinite(t).all()


def test_rho_of_req_errors():
    from kgeo_gb300 import _lib
    from kgeo_gb300.equatorial_lensing import rho_of_req_device
    with pytest.raises(Exception, match="th_o should be a float"):
        rho_of_req_device([(0.5, np.pi / 2, 3.0, 0)], np.zeros(4))
    with pytest.raises(Exception, match="mbar should be an integer"):
        rho_of_req_device([(0.5, 1.0, 3.0, -1)], np.zeros(4))
    lib = _lib.load()
    c = (_lib.Curve * 1)(_lib.Curve(0.5, 1.0, 3.0, 0.0, 8.0, 0, 0))
    v = torch.zeros(4, dtype=torch.float64, device='cuda')
    r = torch.zeros(4, dtype=torch.float64, device='cuda')
    p = ctypes.c_void_p
    assert lib.kgeo_rho_of_req(c, 1, p(v.data_ptr()), 4, 0.0, 1e-15, 100, p(r.data_ptr()), None, None) == 12
    assert lib.kgeo_rho_of_req(c, 1, p(v.data_ptr()), 4, 1e-12, 1e-17, 100, p(r.data_ptr()), None, None) == 12
    assert lib.kgeo_rho_of_req(c, 1, p(v.data_ptr()), 4, 1e-12, 1e-15, -1, p(r.data_ptr()), None, None) == 12


def test_critical_curve(golden):
    from kgeo_gb300 import _lib
    from kgeo_gb300.equatorial_lensing import critical_curve
    g = golden('curves')
    lib = _lib.load()
    for i in range(4):
        a, th0, n = g['crit%d' % i]
        n = int(n)
        al = torch.empty(n, dtype=torch.float64, device='cuda')
        be = torch.empty(n, dtype=torch.float64, device='cuda')
        assert lib.kgeo_critical_curve(float(a), float(th0), n, ctypes.c_void_p(al.data_ptr()),
                                       ctypes.c_void_p(be.data_ptr()), None) == 0
        al, be = al.cpu().numpy(), be.cpu().numpy()
        # the oracle's points before the mask
        rminus = 2 * (1 + np.cos(2. * np.arccos(-a) / 3.))
        rplus = 2 * (1 + np.cos(2. * np.arccos(a) / 3.))
        r = np.linspace(rminus, rplus, n)
        lam = -(r ** 3 + a ** 2 + r * (a ** 2) - 3 * r ** 2) / (a * r - a)
        eta = (r ** 2) * (3 * r ** 2 + a ** 2 - lam ** 2) / (r ** 2 - a ** 2)
        arg = eta + (a * np.cos(th0)) ** 2 - (lam / np.tan(th0)) ** 2
        assert np.all(np.abs(al + lam / np.sin(th0)) <= 1e-12 * np.max(np.abs(lam))), i
        # the masks differ at most where the square root's argument is at rounding level
        scale = np.max(np.abs(eta)) + np.max((lam / np.tan(th0)) ** 2)
        differ = np.isnan(be) != (arg < 0)
        assert np.all(np.abs(arg[differ]) <= 1e-12 * scale), i
        both = ~np.isnan(be) & (arg >= 0)
        assert np.all(np.abs(be[both] ** 2 - arg[both]) <= 1e-12 * scale), i
        A, B = critical_curve(float(a), float(th0), n)
        ra, rb = g['crit_alpha%d' % i], g['crit_beta%d' % i]
        if A.shape == ra.shape:
            # lambda cancels (a cube against lower powers), so its error is absolute: eps max|lambda|
            assert np.max(np.abs(A - ra)) <= 1e-11 * np.max(np.abs(ra)), i
            # beta = sqrt of a cancelling sum: ~sqrt(eps) near the curve's ends
            assert np.max(np.abs(B - rb)) <= 1e-6, i
        else:
            assert abs(A.size - ra.size) <= 8, i
