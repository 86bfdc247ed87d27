"""Generate the golden fixtures in this folder by running the reference kgeo itself.

Run from the repository root, in a container that has the reference checked out:

    python tests/golden/make_golden.py [path-to-kgeo-checkout]

The reference is imported unmodified. Its optional plotting / HDF5 / ehtim
imports are replaced by inert stand-ins, numpy-2 removed aliases (np.infty,
np.NaN) are restored, and the B-field data table that kgeo loads at import
time (absent from the checkout) is regenerated into a temporary folder from
the recipe in kgeo/bfields.py:7-20 (100000 nodes on [1, 100]); only the
'bz_monopole' cases of the polarised-image fixture read it.

Each fixture is a compressed .npz holding the inputs and the reference's
outputs; tests/test_oracle_golden.py pins the CPU oracle to them and the GPU
parity tests check the CUDA path against them.
"""
import contextlib
import io
import os
import sys
import tempfile
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(path):
    """Import kgeo from ``path`` with the stand-ins described in the module docstring."""
    np.infty = np.inf
    np.NaN = np.nan
    np.Inf = np.inf

    def stub(name, **attrs):
        mod = types.ModuleType(name)
        mod.__dict__.update(attrs)
        sys.modules[name] = mod
        return mod

    class Inert:
        def __getattr__(self, k):
            return Inert()

        def __call__(self, *a, **k):
            return Inert()

    mpl = stub('matplotlib')
    plt = stub('matplotlib.pyplot')
    plt.__getattr__ = lambda k: Inert()
    mpl.pyplot = plt
    stub('h5py', File=lambda *a, **k: Inert())
    stub('ehtim')
    stub('ehtim.parloop', Counter=Inert)
    stub('ehtim.observing')
    stub('ehtim.observing.obs_helpers', prog_msg=lambda *a, **k: None)

    import pkg_resources
    table = os.path.join(tempfile.mkdtemp(prefix='kgeo_bz_'), 'bz_fr_data.dat')
    orig = pkg_resources.resource_stream

    def resource_stream(pkg, name):
        if name == 'bz_fr_data.dat':
            if not os.path.exists(table):
                import mpmath

                def f(r):
                    r = r + 0j
                    out = (mpmath.polylog(2, 2. / r) - np.log(1 - 2. / r) * np.log(r / 2.)) * r * r * (2 * r - 3) / 8.
                    out += (1 + 3 * r - 6 * r * r) * np.log(r / 2.) / 12.
                    out += 11. / 72. + 1. / (3. * r) + r / 2. - r * r / 2.
                    return float(np.real(complex(out)))
                rs = np.linspace(1, 100, 100000)  # the nodes of the table's generator, kgeo/bfields.py:16-20
                np.savetxt(table, np.vstack((rs, np.array([f(r) for r in rs]))))
            return open(table, 'rb')
        return orig(pkg, name)

    pkg_resources.resource_stream = resource_stream
    sys.path.insert(0, path)
    import kgeo  # noqa: F401
    import kgeo.kerr_raytracing_ana as ana
    import kgeo.kerr_raytracing_utils as utils
    import kgeo.equatorial_lensing as lensing
    import kgeo.equatorial_images as images
    import kgeo.scipy_ellip_binding as binding
    import kgeo.velocities as vel
    import kgeo.emissivities as emis
    import kgeo.bfields as bfields
    return types.SimpleNamespace(ana=ana, utils=utils, lensing=lensing, images=images,
                                 binding=binding, vel=vel, emis=emis, bfields=bfields)


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def trace_case(ref, a, r_o, th_o, alpha, beta, ngeo):
    alpha = np.asarray(alpha, dtype=float)
    beta = np.asarray(beta, dtype=float)
    g = quiet(ref.ana.raytrace_ana, a=a, observer_coords=[0, r_o, th_o, 0],
              image_coords=[alpha, beta], ngeo=ngeo, plotdata=False)
    t, r, th, ph = g.geo_coords
    lam = -alpha * np.sin(th_o)
    eta = (alpha ** 2 - a ** 2) * np.cos(th_o) ** 2 + beta ** 2
    if abs(a) < ref.utils.MINSPIN and np.any(eta < 0):
        eta[eta < 0] = ref.utils.EP
    r1, r2, r3, r4, rclass = ref.utils.radial_roots(a, lam, eta)
    thclass = ref.utils.angular_turning(a, th_o, lam, eta)[4]
    return dict(a=a, r_o=r_o, th_o=th_o, ngeo=ngeo, alpha=alpha, beta=beta,
                mino=g.mino_times, sig=g.affine_times, t=t, r=r, th=th, ph=ph,
                rclass=rclass, thclass=thclass, tau_tot=g.tautot, nmax_eq=quiet(lambda: g.nmax_eq),
                roots=np.stack([r1, r2, r3, r4]))


def save(name, d):
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
    print('wrote', path, os.path.getsize(path), 'bytes')


def grid(lo, hi, n):
    x = np.linspace(lo, hi, n)
    A, B = np.meshgrid(x, x)
    return A.flatten(), B.flatten()


BAND_SAMPLES = np.r_[0:256:8, 255]   # samples of the ngeo = 256 band traces kept in the fixture


def band_rays(ref, a, th_o, n_angles, offsets, n_curve=100000):
    """Pixels at the given radial offsets (M) from the critical curve at n_angles screen
    angles, the construction of the 2048^2-plus-band workload's polar band; the curve is the
    reference's critical_curve (kgeo/equatorial_lensing.py:260-289)."""
    al, be = ref.lensing.critical_curve(a, th_o, n=n_curve)
    ang = np.arctan2(be, al)
    rad = np.hypot(al, be)
    order = np.argsort(ang)
    phis = np.linspace(-np.pi, np.pi, n_angles, endpoint=False)
    rc = np.interp(phis, ang[order], rad[order], period=2 * np.pi)
    R = rc[None, :] + np.asarray(offsets)[:, None]
    return (R * np.cos(phis)[None, :]).flatten(), (R * np.sin(phis)[None, :]).flatten()


def hot_path_edges(ref):
    """Rays of the rarer radial and angular classes: radial region II (four real roots, the
    ray ends on the horizon; kgeo/kerr_raytracing_utils.py:375, :485-515), the no-real-root
    case 4 with vortical theta motion, and pixels next to the critical curve."""
    deg = np.pi / 180.

    def patch(a, th, alo, ahi, blo, bhi, n=12):
        A, B = np.meshgrid(np.linspace(alo, ahi, n), np.linspace(blo, bhi, n))
        return trace_case(ref, a, 1.e4, th * deg, A.flatten(), B.flatten(), 48)
    save('trace_region2_a094_i81', patch(0.94, 81.3, -1.6, -1.1, -0.5, 0.5))
    save('trace_region2_a099_i89', patch(0.99, 89.0, -1.9, -1.0, -0.9, 0.9))
    save('trace_region2_a081_i99', patch(0.8116436987218719, 98.67750919956, -1.1, -0.95, -0.16, 0.16))
    save('trace_case4_a094_i45', patch(0.94, 45.0, -1.2, 1.2, -1.2, 1.2))
    save('trace_case4_a086_i4', patch(0.8556894680343942, 3.955530626880863, -1.6, 1.6, -1.6, 1.6))

    # the critical-curve band of the mixed-precision workload (a = 0.94, theta_o = 17 deg,
    # offsets from linspace(-0.05, 0.05, 256), the ones nearest the curve included), ngeo = 256,
    # every 8th sample and the last one stored
    offs = np.linspace(-0.05, 0.05, 256)[[0, 64, 120, 126, 127, 128, 129, 135, 191, 255]]
    A, B = band_rays(ref, 0.94, 17 * deg, 32, offs)
    d = trace_case(ref, 0.94, 1.e4, 17 * deg, A, B, 256)
    for k in ('mino', 'sig', 't', 'r', 'th', 'ph'):
        d[k] = d[k][BAND_SAMPLES]
    d.update(samples=BAND_SAMPLES, offsets=offs, n_angles=32)
    save('band_a094_i17', d)


def main(path, only=None):
    warnings.filterwarnings('ignore')
    ref = import_reference(path)
    deg = np.pi / 180.
    if only == 'edges':
        hot_path_edges(ref)
        return
    hot_path_edges(ref)

    # configuration-1 geometry on a coarser grid
    A, B = grid(-8, 8, 16)
    save('trace_a094_i20_16x16', trace_case(ref, 0.94, 1.e4, 20 * deg, A, B, 48))

    # edge rays: alpha = 0 (u_+ clamped to 1), tiny alpha, vortical, eta ~ 0, large impact
    ea = [0., 0., 1e-9, 3., -4., 0.05, 0.3, -0.2, 12., -9., 2.5, 0.0001]
    eb = [3., -3., 3., 0., 0., 0.05, -0.1, 0.15, 7., -11., 1.0, -4.0]
    save('trace_edge_a094_i20', trace_case(ref, 0.94, 1.e4, 20 * deg, ea, eb, 32))
    save('trace_edge_a050_i120', trace_case(ref, 0.5, 1.e4, 120 * deg, ea, eb, 32))
    save('trace_lowspin_a5e-5_i20', trace_case(ref, 5e-5, 1.e4, 20 * deg, [3., -4., 0.5, 6.], [2., 1., 0.3, -2.], 24))
    save('trace_spin0_i45', trace_case(ref, 0.0, 1.e4, 45 * deg, [3., -4., 0.5, 6.], [2., 1., 0.3, -2.], 24))
    save('trace_rinf_a07_i30', trace_case(ref, 0.7, np.inf, 30 * deg, [3., -4., 0.5, 6., 1.], [2., 1., 0.3, -2., -6.], 24))

    # configuration-2 draws (a ~ U[0, 0.998), th_o ~ U[1, 89] deg), coarse grids
    rng = np.random.default_rng(0)
    A, B = grid(-10, 10, 12)
    for i in range(3):
        a = float(rng.uniform(0, 0.998))
        th = float(rng.uniform(1, 89)) * deg
        save('trace_rand%d' % i, trace_case(ref, a, 1.e4, th, A, B, 24))

    # the midplane-crossing rays of tests/test_geodesics_kerr_ana.py:54-70 (r_o = 1000, ngeo = 10000)
    keys = [(0.42, 60., -17., 0.), (0.42, 60., -9., 0.), (0.42, 60., -4., 0.), (0.42, 60., 1., 0.),
            (0.42, 60., 6., 0.), (0.42, 60., 8., 0.), (0.9, 10., -12., 0.), (0.9, 10., -4., 0.),
            (0.9, 10., 1., 0.), (0.9, 10., 2., 0.), (0.73, 35., 0.0001, -10), (0.73, 35., 0.0001, -1.),
            (0.73, 35., 0.0001, 1.), (0.73, 35., 0.0001, 3.), (0.73, 35., 0.0001, 4.)]
    xs, ys, rows = [], [], []
    for (spin, inc, al, be) in keys:
        g = quiet(ref.ana.raytrace_ana, a=spin, observer_coords=[0, 1000., inc / 180. * np.pi, 0],
                  ngeo=10000, image_coords=[al, be], plotdata=False)
        t, r, h, p = np.array(g.geo_coords)[:, :, 0]
        x = r * np.sin(h) * np.cos(p)
        y = r * np.sin(h) * np.sin(p)
        z = r * np.cos(h)
        if z[0] > z[1]:
            xi, yi, zi = x[::-1], y[::-1], z[::-1]
        else:
            xi, yi, zi = x, y, z
        xs.append(np.interp(0, zi, xi))
        ys.append(np.interp(0, zi, yi))
        rows.append((spin, inc, al, be))
    save('midplane_crossings', dict(keys=np.array(rows), x0=np.array(xs), y0=np.array(ys)))

    # equatorial source radius, orders 0..2
    rng = np.random.default_rng(1)
    A, B = grid(-10, 10, 32)
    for i, (a, th) in enumerate([(float(rng.uniform(0, 0.998)), float(rng.uniform(1, 89)) * deg),
                                 (0.94, 17 * deg), (0.5, 120 * deg)]):
        out = dict(a=a, r_o=1.e4, th_o=th, alpha=A, beta=B)
        for m in range(3):
            r_s, Ir, Imax, Nmax = ref.lensing.r_equatorial(a, 1.e4, th, m, A, B)
            out.update({'r_s%d' % m: r_s, 'Ir%d' % m: Ir, 'Imax%d' % m: Imax, 'Nmax%d' % m: Nmax})
        out['outside_crit'] = ref.utils.is_outside_crit(a, th, A, B)
        save('requatorial_%d' % i, out)

    # configuration-5 image (general velocity, bpl emissivity) on a coarse grid
    em = ref.emis.Emissivity('bpl', p1=-2.0, p2=0.0)
    ve = ref.vel.Velocity('general', fac_subkep=0.8, beta_r=0.5)
    psize = 16. / 40
    res = quiet(ref.images.make_image, 0.5, 1.e4, 60 * deg, 2, -8., 8., -8., 8., psize,
                emissivity=em, velocity=ve)
    n_side = int(np.floor(8. - -8.) / psize)
    side = np.linspace(-8., -8. + n_side * psize, n_side)
    Ai, Bi = np.meshgrid(side, side)
    save('image_a05_i60', dict(a=0.5, r_o=1.e4, th_o=60 * deg, psize=psize, alpha=Ai.flatten(), beta=Bi.flatten(),
                               I=res[0], r=res[3], g=res[5], n=res[7], np_=res[8],
                               p1=-2.0, p2=0.0, fac_subkep=0.8, beta_r=0.5, beta_phi=1.0))

    # make_image across the other velocity / emissivity models, both hemispheres, cuts
    cases = [
        (0.3, 40, 1, ('constant', {}), ('zamo', {})),
        (0.9, 25, 2, ('bpl', {}), ('kep', {})),
        (0.7, 110, 1, ('glm', {}), ('kep', {'retrograde': True})),
        (0.2, 75, 1, ('ring', {'r_ring': 5.0, 'gamma_off': 0.3, 'sigma': 0.4, 'emiscut_in': 3.0}),
         ('subkep', {'fac_subkep': 0.6, 'retrograde': True})),
        (0.94, 17, 2, ('bpl', {'p1': -1.5, 'p2': -0.3}), ('infall', {})),
        (0.9375, 135, 1, ('bpl', {'p1': -2.5, 'p2': 0.1}),
         ('general', {'fac_subkep': 0.3, 'beta_phi': 0.1, 'beta_r': 0.4, 'retrograde': True})),
    ]
    psize = 18. / 20
    n_side = int(np.floor(9. - -9.) / psize)
    side = np.linspace(-9., -9. + n_side * psize, n_side)
    Ai, Bi = np.meshgrid(side, side)
    out = dict(alpha=Ai.flatten(), beta=Bi.flatten(), psize=psize, ncase=len(cases))
    for i, (a, th, mbar_max, (et, ek), (vt, vk)) in enumerate(cases):
        em = ref.emis.Emissivity(et, **ek)
        ve = ref.vel.Velocity(vt, **vk)
        res = quiet(ref.images.make_image, a, 1.e4, th * deg, mbar_max, -9., 9., -9., 9., psize,
                    emissivity=em, velocity=ve)
        out.update({'case%d' % i: repr((a, th, mbar_max, et, ek, vt, vk))})
        for k, v in zip(['I', 'Q', 'U', 'r', 't', 'g', 'sinthb', 'n', 'np'], res):
            out['%s%d' % (k, i)] = v
    save('image_models', out)

    # polarised make_image: every lab-frame B-field model, path length, r_o = inf, negative spin
    pcases = [
        (0.5, 60, 1.e4, 1, ('bpl', {}), ('kep', {}), ('rad', {}), False, 1.),
        (0.9, 25, 1.e4, 2, ('ring', {'r_ring': 4.0}), ('subkep', {'fac_subkep': 0.7}), ('vert', {}), False, 1.),
        (0.3, 130, 1.e4, 1, ('glm', {}), ('zamo', {}), ('tor', {}), False, 0.5),
        (0.7, 45, 1.e4, 1, ('bpl', {}), ('general', {'fac_subkep': 0.6, 'beta_phi': 0.7, 'beta_r': 0.8}),
         ('simple', {'Cr': 0.3, 'Cvert': -0.5, 'Cph': 0.8}), False, 1.),
        (0.6, 70, 1.e4, 1, ('constant', {}), ('infall', {}), ('simple_rm1', {'Cr': 1.0, 'Cvert': 0.4, 'Cph': -0.2}),
         False, 1.),
        (0.8, 35, 1.e4, 1, ('bpl', {}), ('kep', {'retrograde': True}), ('monopoleA', {'C': -1, 'omegafac': 0.3}),
         False, 1.),
        (0.42, 60, np.inf, 2, ('ring', {}), ('general', {}), ('bz_guess', {'C': 1.}), False, 1.),
        (-0.6, 50, 1.e4, 1, ('bpl', {}), ('subkep', {'fac_subkep': 0.8}), ('bz_guess', {'C': -1.}), False, 1.),
        (0.9, 80, 1.e4, 1, ('glm', {}), ('kep', {}), ('power', {'p': 0.75}), False, 1.),
        (0.3, 40, 1.e4, 1, ('bpl', {}), ('zamo', {}), ('power', {'p': 0.0, 'C': -1}), False, 1.),
        (0.7, 55, 1.e4, 1, ('bpl', {}), ('kep', {}), ('power', {'p': 1.2, 'usemono': True}), False, 1.),
        (0.94, 30, 1.e4, 1, ('bpl', {}), ('general', {'beta_r': 0.3}),
         ('gen_power', {'n_I': 0.5, 'p_val': 0.8, 'isAbove': False}), False, 1.),
        (0.5, 65, 1.e4, 1, ('bpl', {}), ('kep', {}), ('bz_monopole', {'C': 1}), False, 1.),
        (0.5, 65, 1.e4, 1, ('bpl', {}), ('kep', {}), ('bz_monopole', {'C': 1, 'secondorder_only': True}), False, 1.),
        (0.7, 50, 1.e4, 1, ('bpl', {}), ('general', {'fac_subkep': 0.5}), ('bz_guess', {}), True, 1.),
    ]
    psize = 16. / 20
    n_side = int(np.floor(8. - -8.) / psize)
    side = np.linspace(-8., -8. + n_side * psize, n_side)
    Ai, Bi = np.meshgrid(side, side)
    out = dict(alpha=Ai.flatten(), beta=Bi.flatten(), psize=psize, ncase=len(pcases))
    for i, (a, th, r_o, mbar_max, (et, ek), (vt, vk), (bt, bk), plen, spec) in enumerate(pcases):
        em = ref.emis.Emissivity(et, **ek)
        ve = ref.vel.Velocity(vt, **vk)
        bf = ref.bfields.Bfield(bt, **bk)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            res = quiet(ref.images.make_image, a, r_o, th * deg, mbar_max, -8., 8., -8., 8., psize,
                        emissivity=em, velocity=ve, bfield=bf, polarization=True, pathlength=plen,
                        specind=spec)
        out.update({'case%d' % i: repr((a, th, r_o, mbar_max, et, ek, vt, vk, bt, bk, plen, spec))})
        names = ['I', 'Q', 'U', 'r', 't', 'g', 'sinthb', 'n', 'np'] + (['lp', 'Ie'] if plen else [])
        for k, v in zip(names, res):
            out['%s%d' % (k, i)] = np.real(v)
    # pathlength=True without polarisation
    em = ref.emis.Emissivity('bpl')
    ve = ref.vel.Velocity('kep')
    res = quiet(ref.images.make_image, 0.5, 1.e4, 60 * deg, 1, -8., 8., -8., 8., psize,
                emissivity=em, velocity=ve, pathlength=True, diskangle=0.2)
    for k, v in zip(['I', 'Q', 'U', 'r', 't', 'g', 'sinthb', 'n', 'np', 'lp', 'Ie'], res):
        out['%s_unpol' % k] = v
    save('image_pol', out)

    # lab-frame fields of every model on a radial grid (bz_para is pinned here only: with
    # polarization=True the reference's make_image raises for it, as its complex-typed
    # Omega reaches an in-place float multiply in Emissivity.jrest)
    bout = {}
    rr = np.concatenate([np.linspace(1.05, 12., 150), np.linspace(12.5, 140., 50)])
    models = [('rad', {}), ('vert', {}), ('tor', {}), ('simple', {'Cr': 0.3, 'Cvert': -0.5, 'Cph': 0.8}),
              ('simple_rm1', {'Cr': 1.0, 'Cvert': 0.4, 'Cph': -0.2}), ('monopoleA', {'C': -1, 'omegafac': 0.3}),
              ('bz_guess', {'C': 1.}), ('bz_guess', {'C': -2.}), ('bz_para', {'C': 1}), ('bz_para', {'C': -1.5}),
              ('power', {'p': 0.75}), ('power', {'p': 0.0, 'C': -1}), ('power', {'p': 1.2, 'usemono': True}),
              ('gen_power', {'n_I': 0.5, 'p_val': 0.8, 'isAbove': False}), ('gen_power', {}),
              ('bz_monopole', {'C': 1}), ('bz_monopole', {'C': 1, 'secondorder_only': True})]
    spins = (0.3, 0.9375, -0.6)
    for i, (bt, bk) in enumerate(models):
        bf = ref.bfields.Bfield(bt, **bk)
        for j, a in enumerate(spins):
            rh = 1 + np.sqrt(1 - a * a)
            r = rr[rr > rh]
            with warnings.catch_warnings():
                warnings.simplefilter('ignore')
                B = bf.bfield_lab(a, r)
            bout['r_%d_%d' % (i, j)] = r
            bout['B_%d_%d' % (i, j)] = np.real(np.stack([np.broadcast_to(np.asarray(b), r.shape) for b in B]))
        bout['model%d' % i] = repr((bt, bk))
    bout['spins'] = np.array(spins)
    bout['nmodel'] = len(models)
    save('bfield_lab', bout)

    # lensed curves of constant equatorial radius (rho_of_req at 36 angles), incl. brackets
    # with no sign change (brentq raises), and the critical curve
    vp = np.linspace(-180, 179, 36) * np.pi / 180.
    ccases = [(0.5, 60., 'rh', 0), (0.94, 17., 5.0, 1), (0.3, 80., 'rh', 2), (0.7, 30., 10.0, 0),
              (0.99, 85., 'rh', 5), (0.01, 45., 1000., 1), (0.6, 130., 'rh', 1), (0.5, 60., 100., 2),
              (0.8, 40., 'rh', 100), (0.5, 60., 0.5, 0)]
    cout = dict(varphi=vp, ncase=len(ccases))
    for i, (a, inc, req, m) in enumerate(ccases):
        r_eq = 1 + np.sqrt(1 - a * a) if req == 'rh' else float(req)
        cout['case%d' % i] = np.array([a, inc, r_eq, m])
        try:
            with warnings.catch_warnings():
                warnings.simplefilter('ignore')
                res = quiet(ref.lensing.rho_of_req, a, inc * deg, r_eq, mbar=m, varphis=vp)
            cout['rho%d' % i] = res[1]
        except ValueError as e:
            cout['error%d' % i] = str(e)
    for i, (a, th0, n) in enumerate([(0.5, 1.0, 3000), (0.94, 0.3, 3000), (0.2, 2.5, 2000), (0.999, 1.5, 5000)]):
        al, be = ref.lensing.critical_curve(a, th0, n=n)
        cout['crit%d' % i] = np.array([a, th0, n])
        cout['crit_alpha%d' % i] = al
        cout['crit_beta%d' % i] = be
    # one file of the curve library (make_curves2: 360 angles, orders 0..2, r_eq = 10)
    lib_dir = tempfile.mkdtemp(prefix='kgeo_lib_')
    quiet(ref.lensing.make_curves2, 0, 'r10', 1, 0.5, 30., 2, lib_dir)
    fn = os.path.join(lib_dir, 'a%02.0f_i%02.0f_%s.txt' % (100 * 0.5, 30., 'r10'))
    cout['library_a50_i30_r10'] = np.loadtxt(fn)
    save('curves', cout)

    # n_angular_turnings (th_o <= pi/2 only, its check): ordinary and vortical rays, both
    # signs of beta, a MINSPIN spin, a 2-d tau and a 1-d tau
    tout = {}
    rng = np.random.default_rng(5)
    for i, (a, th) in enumerate([(0.94, 17.), (0.5, 80.), (0.99, 45.), (5e-5, 30.), (0.7, 90.)]):
        A = np.concatenate([rng.uniform(-8, 8, 300), rng.uniform(-0.3, 0.3, 100)])
        B = np.concatenate([rng.uniform(-8, 8, 300), rng.uniform(-0.3, 0.3, 100)])
        tau = np.abs(rng.uniform(0, 3, (5, A.size)))
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            nt = ref.utils.n_angular_turnings(a, th * deg, A, B, tau)
            nt1 = ref.utils.n_angular_turnings(a, th * deg, A, B, tau[2])
        tout.update({'par%d' % i: np.array([a, th]), 'alpha%d' % i: A, 'beta%d' % i: B, 'tau%d' % i: tau,
                     'n%d' % i: nt, 'n1_%d' % i: nt1})
    save('angular_turnings', tout)

    # off-equatorial jet crossings (solver.findroot on a sampled geodesic set)
    import kgeo.solver as solver
    jcases = [(0.9, 17., 'para', 1.0, 1, 1, 24, 8.), (0.5, 60., 'mono', 0.3, 1, 2, 24, 8.),
              (0.94, 163., 'power', 1.5, 0.75, 1, 24, 8.), (0.7, 3., 'para', 2.0, 1, 1, 12, 150.),
              (0.3, 40., 'power', 0.8, 0.0, 2, 20, 10.)]
    jout = dict(ncase=len(jcases))
    for i, (a, inc, model, psit, pval, neqmax, nside, lim) in enumerate(jcases):
        x = np.linspace(-lim, lim, nside)
        A, B = (v.flatten() for v in np.meshgrid(x, x))
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            geo = quiet(ref.ana.raytrace_ana, a=a, observer_coords=[0, 1.e4, inc * deg, 0], image_coords=[A, B],
                        ngeo=200, plotdata=False, savedata=False)
            res = quiet(solver.findroot, geo, psit, A, B, 1.e4, inc * deg, a, 200, model=model, neqmax=neqmax,
                        tol=1e-8, pval=pval)
        jout['case%d' % i] = repr((a, inc, model, psit, pval, neqmax, nside, lim))
        for k, v in zip(['tau', 'r', 'th', 'signpr', 'signpth', 'neq'], res[:6]):
            jout['%s%d' % (k, i)] = np.asarray(v)
        jout['shape%d' % i] = np.array(res[6])
    save('jet_crossings', jout)

    # off-equatorial jet images of the monopole field-line model (off_eq.getstokes); the
    # paraboloid and p > 0 power models of getstokes fail inside the reference with this
    # numpy / scipy (an array reaches scipy.integrate.quad's bounds), so they have no fixture
    import kgeo.off_eq as off_eq
    scases = [('mono', 0.4, 0.5, 60., 1, 0.0, 1, 2.0), ('mono', 0.3, 0.9, 17., 1, 0.3, 2, 2.0),
              ('power', 0.5, 0.7, 30., 0.0, -0.2, 1, 1.5), ('mono', 0.35, 0.7, 150., 1, 0.5, 2, 0.0)]
    sout = dict(ncase=len(scases))
    for i, (model, psit, a, inc, pval, nu, neqmax, sigma) in enumerate(scases):
        x = np.linspace(-8, 8, 16)
        A, B = np.meshgrid(x, x)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            res = quiet(off_eq.getstokes, psit, A, B, 1.e4, inc * deg, a, 200, model=model, pval=pval, neqmax=neqmax,
                        retvals=True, nu_parallel=nu, sigma=sigma)
        sout['case%d' % i] = repr((model, psit, a, inc, pval, nu, neqmax, sigma))
        for k, v in zip(['I', 'Q', 'U', 'evpa', 'r', 'th'], res):
            sout['%s%d' % (k, i)] = np.asarray(v)
    save('jet_stokes', sout)

    # EVPA of ipole images (the reference's tests/data/*.csv, from tests/test_images.py):
    # pixel location and EVPA along the middle row / column for image orders 0 and 1
    ip = {}
    for name in ('lowspin_keplerian', 'midspin_inclined_keplerian', 'midspin_inclined_subkep'):
        ip[name] = np.loadtxt(os.path.join(path, 'tests', 'data', name + '.csv'), delimiter=',', unpack=True)
    save('ipole_evpa', ip)

    # elliptic Pi adapter: random in-domain points plus every special-case mask
    rng = np.random.default_rng(2)
    n = np.concatenate([rng.uniform(-3, 0.95, 400), rng.uniform(1.05, 6, 200),
                        [1., 1., 0.5, 0.5, 2., np.inf, 0.3, 0.7]])
    phi = np.concatenate([rng.uniform(-9, 9, 400), rng.uniform(-1.4, 1.4, 200),
                          [2.0, -4.0, 1e-11, -1e-11, np.arcsin(np.sqrt(0.5)), 0.7, 3.0, 0.4]])
    m = np.concatenate([rng.uniform(-5, 0.99, 400), rng.uniform(-2, 0.9, 200),
                        [0.3, -0.2, 0.5, 0.5, 0.1, 0.4, 1.5, -2e14]])
    save('ellip_pi', dict(n=n, phi=phi, m=m, pi=ref.binding.ellip_pi_arr(n, phi, m)))

    # general velocity on a radial grid and at the ipole-checked points of tests/test_velocities.py
    rr = np.linspace(1.2, 30., 200)
    vout = {}
    for i, (a, xi, bp, br, retro) in enumerate([(0.5, 0.8, 1.0, 0.5, False), (0.9375, 0.3, 0.1, 0.4, False),
                                                (0.42, 0.24, 0.42, 0.24, True)]):
        rh = 1 + np.sqrt(1 - a * a)
        r = rr[rr > rh]
        u0, u1, u2, u3 = ref.vel.u_general(a, r, fac_subkep=xi, beta_phi=bp, beta_r=br, retrograde=retro)
        vout.update({'r%d' % i: r, 'u%d' % i: np.stack([u0, u1, u3]),
                     'par%d' % i: np.array([a, xi, bp, br, float(retro)])})
    save('velocity_general', vout)


if __name__ == '__main__':
    # python tests/golden/make_golden.py [path-to-kgeo-checkout] [edges]
    # ('edges' regenerates only the fixtures of hot_path_edges)
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference', sys.argv[2] if len(sys.argv) > 2 else None)
