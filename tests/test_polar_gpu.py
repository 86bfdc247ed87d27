"""GPU parity of the polarised equatorial image (kgeo_image_ex) through the drop-in
make_image / Iobs: against the reference's polarised make_image fixtures, the oracle (incl.
the 'bz_para' field, which the reference's polarised make_image cannot run), and the ipole
EVPA profiles of the reference's tests/test_images.py on full 800 x 800 images.

Tolerances as in tests/test_polar_cpu.py: I, Q, U relative to I at 1e-9 (5e-8 for
'bz_monopole', whose f(r) the reference interpolates from a table)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import kgeo_oracle as ko
from test_polar_cpu import IPOLE, NX, check_image, evpa_kgeo, ipole_check, pol_cases, rel

pytestmark = pytest.mark.gpu

DEG = np.pi / 180
NAMES = {'I': 0, 'Q': 1, 'U': 2, 'r': 3, 't': 4, 'g': 5, 'sinthb': 6, 'n': 7, 'np': 8, 'lp': 9, 'Ie': 10}


def _objects(emis, vel, bf):
    from kgeo_gb300.bfields import Bfield
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.velocities import Velocity
    return Emissivity(emis[0], **emis[1]), Velocity(vel[0], **vel[1]), Bfield(bf[0], **bf[1])


def test_make_image_pol_fixture(golden):
    from kgeo_gb300.equatorial_images import make_image
    g = golden('image_pol')
    ps = float(g['psize'])
    for i, a, r_o, th_o, mm, emis, vel, bf, plen, spec in pol_cases(g):
        em, ve, bo = _objects(emis, vel, bf)
        res = make_image(a, r_o, th_o, mm, -8., 8., -8., 8., ps, emissivity=em, velocity=ve, bfield=bo,
                         polarization=True, pathlength=plen, specind=spec)
        assert len(res) == (11 if plen else 9)
        out = {k: res[j] for k, j in NAMES.items() if j < len(res)}
        tol = 5e-8 if bf[0] == 'bz_monopole' else 1e-9
        check_image(out, g, i, plen, tol, 5e-9 if bf[0] == 'bz_monopole' else 1e-10, {k: k for k in out})
        assert rel(out['r'], g['r%d' % i]) <= 1e-10, i
        assert rel(out['t'], g['t%d' % i]) <= 1e-12, i
        assert np.array_equal(out['n'], g['n%d' % i]), i
        assert rel(out['np'], g['np%d' % i]) <= 1e-12, i


def test_make_image_pathlength_unpolarised(golden):
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.equatorial_images import make_image
    from kgeo_gb300.velocities import Velocity
    g = golden('image_pol')
    res = make_image(0.5, 1.e4, 60 * DEG, 1, -8., 8., -8., 8., float(g['psize']), emissivity=Emissivity('bpl'),
                     velocity=Velocity('kep'), pathlength=True, diskangle=0.2)
    for k in ('I', 'Q', 'U', 'g', 'sinthb', 'lp', 'Ie'):
        assert rel(res[NAMES[k]], g['%s_unpol' % k]) <= 1e-10, k


def test_pol_random_vs_oracle():
    """Every field model on random pixels against the oracle, incl. bz_para and both
    hemispheres / both spin signs."""
    from kgeo_gb300.equatorial_images import Iobs
    rng = np.random.default_rng(7)
    fields = [('rad', {}), ('simple', {'Cr': -0.4, 'Cvert': 0.9, 'Cph': 0.3}), ('monopoleA', {}),
              ('bz_guess', {'C': 2.}), ('bz_para', {'C': 1}), ('bz_para', {'C': -0.7}), ('power', {'p': 0.5}),
              ('gen_power', {'n_I': 1.0, 'p_val': 0.6}), ('bz_monopole', {'C': -1})]
    for k, bf in enumerate(fields):
        a = float(rng.uniform(-0.95, 0.95))
        th_o = float(rng.choice([rng.uniform(5, 85), rng.uniform(95, 175)])) * DEG
        A = rng.uniform(-9, 9, 3000)
        B = rng.uniform(-9, 9, 3000)
        emis, vel = ('glm', {}), ('general', {'fac_subkep': 0.7, 'beta_phi': 0.6, 'beta_r': 0.5})
        em, ve, bo = _objects(emis, vel, bf)
        for mbar in (0, 1):
            res = Iobs(a, 1.e4, th_o, mbar, A, B, emissivity=em, velocity=ve, bfield=bo, polarization=True,
                       pathlength=True)
            o = ko.make_image_px(a, 1.e4, th_o, mbar, A, B, emis=emis, vel=vel, bfield=bf, polarization=True,
                                 pathlength=True)
            I = o['I'][:, mbar]
            assert np.array_equal(res[0] > 0, I > 0), (k, mbar)
            lit = I > 0
            assert lit.sum() > 100, (k, mbar)
            tol = 5e-9
            assert rel(res[0][lit], I[lit]) <= tol, (k, mbar, rel(res[0][lit], I[lit]))
            for j, key in ((1, 'Q'), (2, 'U')):
                e = np.max(np.abs(res[j][lit] - o[key][lit, mbar]) / I[lit])
                assert e <= tol, (k, mbar, key, e)
            assert np.max(np.abs(res[5][lit] - o['sinthb'][lit, mbar])) <= 1e-10, (k, mbar)
            assert rel(res[9][lit], o['lp'][lit, mbar]) <= tol, (k, mbar)


def test_iobs_matches_make_image_pol():
    from kgeo_gb300.equatorial_images import Iobs, image_pixels, make_image
    em, ve, bo = _objects(('ring', {}), ('kep', {}), ('bz_guess', {}))
    res = make_image(0.7, 1.e4, 40 * DEG, 2, -7., 7., -7., 7., 0.5, emissivity=em, velocity=ve, bfield=bo,
                     polarization=True)
    A, B = image_pixels(-7., 7., -7., 7., 0.5)
    for m in range(3):
        r1 = Iobs(0.7, 1.e4, 40 * DEG, m, A, B, emissivity=em, velocity=ve, bfield=bo, polarization=True)
        for j_img, j_iobs in ((0, 0), (1, 1), (2, 2), (5, 3), (3, 4), (6, 5), (4, 6)):
            assert np.array_equal(res[j_img][:, m], r1[j_iobs]), (m, j_img)


@pytest.mark.parametrize('name', sorted(IPOLE))
def test_ipole_evpa_full_image(name, golden):
    """tests/test_images.py of the reference through the drop-in make_image: 800 x 800,
    r_o = inf, n_subrings = 2, ring emissivity, general velocity, bz_guess field."""
    from kgeo_gb300.bfields import Bfield
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.equatorial_images import make_image
    from kgeo_gb300.velocities import Velocity
    a, inc, fs, br, bp, *_rest = IPOLE[name]
    res = make_image(a, np.inf, inc * np.pi / 180., 2, -10., 10., -10., 10., 20. / NX, nmax_only=False,
                     emissivity=Emissivity('ring'),
                     velocity=Velocity('general', fac_subkep=fs, beta_phi=bp, beta_r=br),
                     bfield=Bfield('bz_guess', C=1.), polarization=True, specind=1.)
    Q, U = res[1], res[2]
    ev = [evpa_kgeo(Q[:, i].reshape((NX, NX)), U[:, i].reshape((NX, NX))) for i in range(2)]
    ipole_check(name, [e[NX // 2, :] for e in ev], [e[:, NX // 2] for e in ev], golden('ipole_evpa'))


def test_image_ex_errors():
    from kgeo_gb300 import _lib
    lib = _lib.load()
    al = torch.zeros(4, dtype=torch.float64, device='cuda')
    I = torch.zeros(4, dtype=torch.float64, device='cuda')
    ob = _lib.Observer(0.5, 1.e4, 1.0)
    m = _lib.Emission()
    m.specind = 1.0
    m.sinthb = 0.7
    out = _lib.ImageOut()
    out.I = ctypes.c_void_p(I.data_ptr())
    p = ctypes.c_void_p(al.data_ptr())
    for field, c in ((8, (1, 0, 0)), (-1, (1, 0, 0)), (0, (0, 0, 0)), (3, (float('nan'), 0, 0))):
        o = _lib.ImageOptions()
        o.polarization = 1
        o.bfield.field = field
        for k in range(3):
            o.bfield.c[k] = c[k]
        st = lib.kgeo_image_ex(ctypes.byref(ob), 0, 1, p, p, 4, ctypes.byref(m), ctypes.byref(o), ctypes.byref(out),
                               None)
        assert st == 10, (field, st)
    o = _lib.ImageOptions()
    o.pathlength = 1
    o.diskangle = float('inf')
    assert lib.kgeo_image_ex(ctypes.byref(ob), 0, 1, p, p, 4, ctypes.byref(m), ctypes.byref(o), ctypes.byref(out),
                             None) == 10
    torch.cuda.synchronize()
