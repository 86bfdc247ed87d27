"""GPU parity of raytrace_ana / coords_at_tau (CUDA path through the C ABI) against
reference fixtures and the CPU oracle. Tolerances: tests/parity.py."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from parity import check_trace, lambda_eta_sensitivity

pytestmark = pytest.mark.gpu

TRACES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, 'trace_*.npz')))


@pytest.fixture(scope='module')
def kg():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kgeo_gb300 import kerr_raytracing_ana
    return kerr_raytracing_ana


def _run(kg, a, r_o, th_o, alpha, beta, ngeo):
    g = kg.raytrace_ana(a=a, observer_coords=[0, r_o, th_o, 0], image_coords=[alpha, beta], ngeo=ngeo,
                        plotdata=False)
    t, r, th, ph = g.geo_coords
    return dict(t=t, r=r, th=th, ph=ph, sig=g.affine_times, mino=g.mino_times)


@pytest.mark.parametrize('name', TRACES)
def test_trace_vs_reference_fixture(kg, golden, name):
    g = golden(name)
    a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
    got = _run(kg, a, r_o, th_o, g['alpha'], g['beta'], int(g['ngeo']))
    np.testing.assert_allclose(got['mino'], g['mino'], rtol=1e-12, atol=0)
    ref = dict(t=g['t'], r=g['r'], th=g['th'], ph=g['ph'], sig=g['sig'])
    if not np.isfinite(r_o):
        # r_o = inf: the reference's t and sigma are inf - inf garbage, and r at tau = 0 divides
        # by a rounding-level denominator; parity is checked on r, theta, phi from sample 1 on.
        # The last sample of every ray is 1e-10 tau_tot from the horizon or from r = infinity
        # (r ~ 1/(tau_tot - tau)), condition number ~1e10: held to 1e-4 there.
        for k in ('r', 'th', 'ph'):
            for sl, tol in ((slice(1, -1), 1e-9), (slice(-1, None), 1e-4)):
                x, y = got[k][sl], ref[k][sl]
                assert np.array_equal(np.isfinite(x), np.isfinite(y))
                fin = np.isfinite(y)
                assert np.all(np.abs(x[fin] - y[fin]) <= tol * np.maximum(np.abs(y[fin]), 1.0))
        return
    from oracle import kgeo_oracle as ko
    rho = ko.pole_distance(a, r_o, th_o, g['alpha'], g['beta'], g['mino'])
    check_trace(got, ref, r_o, g['rclass'], name, rho=rho)


@pytest.mark.parametrize('name', TRACES)
def test_theta_r_only_trace_vs_reference_fixture(kg, golden, name):
    """kgeo_raytrace with t, phi and sigma not requested runs the sample kernel's theta / r
    path (the Jacobi recurrence without E and Pi): r and theta against the reference's within
    the same bars, the Mino times identical to the full trace's."""
    import torch
    from kgeo_gb300 import device as dev
    g = golden(name)
    a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
    if not np.isfinite(r_o):
        pytest.skip('r_o = inf: covered by the full trace test')
    al, be = dev.as_device(g['alpha']), dev.as_device(g['beta'])
    res = dev.trace(a, r_o, th_o, al, be, ngeo=int(g['ngeo']), outputs=('r', 'th', 'mino'), per_ray=())
    torch.cuda.synchronize()
    full = _run(kg, a, r_o, th_o, g['alpha'], g['beta'], int(g['ngeo']))
    assert np.array_equal(res['mino'].cpu().numpy(), full['mino'])
    from oracle import kgeo_oracle as ko
    rho = ko.pole_distance(a, r_o, th_o, g['alpha'], g['beta'], g['mino'])
    ref = dict(t=g['t'], r=g['r'], th=g['th'], ph=g['ph'], sig=g['sig'])
    got = dict(ref, r=res['r'].cpu().numpy(), th=res['th'].cpu().numpy())
    check_trace(got, ref, r_o, g['rclass'], name + '-rth', rho=rho)


def test_config1_full_vs_oracle(kg):
    """a = 0.94, r_o = 1e4, theta_o = 20 deg, 64x64 over [-8, 8], ngeo = 100 (the reference's CPU case)."""
    from oracle import kgeo_oracle as ko
    x = np.linspace(-8, 8, 64)
    A, B = np.meshgrid(x, x)
    A, B = A.flatten(), B.flatten()
    a, r_o, th_o = 0.94, 1.e4, 20 * np.pi / 180
    ref = ko.raytrace(a, r_o, th_o, A, B, 100)
    got = _run(kg, a, r_o, th_o, A, B, 100)
    refd = dict(t=ref['t'], r=ref['r'], th=ref['th'], ph=ref['ph'], sig=ref['affine_times'])
    rho = ko.pole_distance(a, r_o, th_o, A, B, ref['mino_times'])
    check_trace(got, refd, r_o, ref['rclass'], 'config1', rho=rho)


def test_classes_bit_exact_config2_grids(kg):
    """rclass / thclass on full 512x512 grids for configuration-2 draws (a ~ U[0, 0.998), th_o ~ U[1, 89] deg)."""
    import torch
    from oracle import kgeo_oracle as ko
    from kgeo_gb300 import device as dev
    x = np.linspace(-10, 10, 512)
    A, B = np.meshgrid(x, x)
    A, B = A.flatten(), B.flatten()
    rng = np.random.default_rng(0)
    for _ in range(4):
        a = float(rng.uniform(0, 0.998))
        th_o = float(rng.uniform(1, 89)) * np.pi / 180
        lam, eta = ko.conserved(a, th_o, A, B)
        _, _, _, _, rc = ko.quartic_roots(a, lam, eta)
        tc = ko.theta_turning(a, th_o, lam, eta)[4]
        res = dev.trace(a, 1.e4, th_o, dev.as_device(A), dev.as_device(B), ngeo=2, outputs=())
        torch.cuda.synchronize()
        assert np.array_equal(res['rclass'].cpu().numpy(), rc)
        assert np.array_equal(res['thclass'].cpu().numpy(), tc)


def test_coords_at_tau_vs_oracle(kg):
    from oracle import kgeo_oracle as ko
    rng = np.random.default_rng(3)
    A = rng.uniform(-9, 9, 300)
    B = rng.uniform(-9, 9, 300)
    a, r_o, th_o = 0.7, 5.e3, 40 * np.pi / 180
    lam, eta = ko.conserved(a, th_o, A, B)
    r1, r2, r3, r4, rc = ko.quartic_roots(a, lam, eta)
    tt = ko.mino_total(a, r_o, eta, r1, r2, r3, r4)
    tau = rng.uniform(0, 0.999, (7, 300)) * tt
    sig, (t, r, th, ph) = ko.coords_at_tau(a, r_o, th_o, A, B, tau)
    gs, (gt, gr, gth, gph) = kg.coords_at_tau(a, [0, r_o, th_o, 0], [A, B], tau)
    check_trace(dict(t=gt, r=gr, th=gth, ph=gph, sig=gs), dict(t=t, r=r, th=th, ph=ph, sig=sig), r_o,
                np.zeros(300, int), 'coords_at_tau', rho=ko.pole_distance(a, r_o, th_o, A, B, tau))
    gs0, (gt0, gr0, gth0, gph0) = kg.coords_at_tau(a, [0, r_o, th_o, 0], [A, B], tau, do_phi_and_t=False)
    s0, (t0, r0, th0, ph0) = ko.coords_at_tau(a, r_o, th_o, A, B, tau, do_phi_and_t=False)
    assert np.allclose(gr0, r0, rtol=1e-10, atol=0) and np.allclose(gth0, th0, rtol=1e-10, atol=1e-10)
    assert np.array_equal(gt0, t0) and np.array_equal(gph0, ph0) and np.array_equal(gs0, s0)


def test_midplane_crossings_known_answers(kg, golden):
    """The ipole-checked first midplane crossings of the reference's tests/test_geodesics_kerr_ana.py:54-70."""
    g = golden('midplane_crossings')
    want = np.array([(-0.0522336, -16.0342), (-0.103693, -8.09784), (-0.308159, -3.20445), (-0.327624, 1.67648),
                     (877.845, -13.6213), (0.129720, 6.94829), (-0.164094, -11.0082), (-0.655582, -2.99558),
                     (-0.518830, -0.632352), (-0.691096, -1.15767), (11.8258, -0.0858775), (1.02201, 1.13478),
                     (0.0148225, 0.0165869), (-1.20034, -1.08604), (-2.11221, 1.02322)])
    for i, (spin, inc, al, be) in enumerate(g['keys']):
        out = _run(kg, float(spin), 1000., float(inc) / 180. * np.pi, np.array([al]), np.array([be]), 10000)
        r, h, p = out['r'][:, 0], out['th'][:, 0], out['ph'][:, 0]
        x, y, z = r * np.sin(h) * np.cos(p), r * np.sin(h) * np.sin(p), r * np.cos(h)
        if z[0] > z[1]:
            x, y, z = x[::-1], y[::-1], z[::-1]
        x0, y0 = np.interp(0, z, x), np.interp(0, z, y)
        assert np.allclose([x0, y0], want[i], rtol=1e-3)
        # a crossing interpolated from the final sample of a horizon-bound ray inherits that
        # sample's ~1e-6 conditioning noise (tests/parity.py); every other crossing is held to 1e-9
        # (np.interp clamps to the end value when the ray never reaches z = 0)
        rev = out['r'].shape[0] > 1 and (out['r'][0, 0] * np.cos(out['th'][0, 0]) >
                                         out['r'][1, 0] * np.cos(out['th'][1, 0]))
        last = 0 if rev else z.size - 1
        j = int(np.searchsorted(z, 0.0))
        used = {max(j - 1, 0), min(j, z.size - 1)}
        tol = 1e-4 if last in used else 1e-9
        assert np.allclose([x0, y0], [g['x0'][i], g['y0'][i]], rtol=tol, atol=tol)


def test_argument_errors_match_reference(kg):
    A = np.array([1.0, 2.0])
    with pytest.raises(Exception, match=r'\|a\| should be a float in range \[0,1\)'):
        kg.raytrace_ana(a=1, observer_coords=[0, 1e4, 0.3, 0], image_coords=[A, A], ngeo=3)
    with pytest.raises(Exception, match='r_o should be a float > 100'):
        kg.raytrace_ana(a=0.5, observer_coords=[0, 50., 0.3, 0], image_coords=[A, A], ngeo=3)
    with pytest.raises(Exception, match=r'th_o should be a float in range'):
        kg.raytrace_ana(a=0.5, observer_coords=[0, 1e4, np.pi / 2, 0], image_coords=[A, A], ngeo=3)
    with pytest.raises(Exception, match='alpha, beta are different lengths!'):
        kg.raytrace_ana(a=0.5, observer_coords=[0, 1e4, 0.3, 0], image_coords=[A, A[:1]], ngeo=3)


def test_empty_and_single_sample(kg):
    from oracle import kgeo_oracle as ko
    g = kg.raytrace_ana(a=0.5, observer_coords=[0, 1e4, 0.3, 0], image_coords=[np.zeros(0), np.zeros(0)], ngeo=5)
    assert g.geo_coords[1].shape == (5, 0)
    A, B = np.array([3.0, -2.0]), np.array([1.0, 4.0])
    g = kg.raytrace_ana(a=0.5, observer_coords=[0, 1e4, 0.3, 0], image_coords=[A, B], ngeo=1)
    ref = ko.raytrace(0.5, 1e4, 0.3, A, B, 1)
    assert g.mino_times.shape == (1, 2) and np.array_equal(g.mino_times, ref['mino_times'])
    assert np.allclose(g.geo_coords[1], ref['r'], rtol=1e-10)


@pytest.mark.parametrize('idx', [0, 1, 2])
def test_r_equatorial_vs_reference_fixture(kg, golden, idx):
    from kgeo_gb300 import equatorial_lensing as el
    g = golden('requatorial_%d' % idx)
    a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
    for m in range(3):
        r_s, Ir, Imax, Nmax = el.r_equatorial(a, r_o, th_o, m, g['alpha'], g['beta'])
        assert np.array_equal(Nmax, g['Nmax%d' % m])
        assert np.array_equal(r_s == 0, g['r_s%d' % m] == 0) and np.array_equal(r_s < 0, g['r_s%d' % m] < 0)
        np.testing.assert_allclose(r_s, g['r_s%d' % m], rtol=1e-10, atol=0)
        np.testing.assert_allclose(Ir, g['Ir%d' % m], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(Imax, g['Imax%d' % m], rtol=1e-10, atol=1e-12)
    assert np.array_equal(el.is_outside_crit(a, th_o, g['alpha'], g['beta']), g['outside_crit'])


def test_crossing_counts_bit_exact(kg, golden):
    from oracle import kgeo_oracle as ko
    for name in TRACES:
        g = golden(name)
        a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
        got = kg.raytrace_ana(a=a, observer_coords=[0, r_o, th_o, 0], image_coords=[g['alpha'], g['beta']],
                              ngeo=int(g['ngeo']), plotdata=False)
        assert np.array_equal(got.nmax_eq, g['nmax_eq']), name
        npol = ko.n_poloidal_orbits(a, th_o, g['alpha'], g['beta'], g['mino'])
        np.testing.assert_allclose(got.n_poloidal, npol, rtol=1e-10, atol=1e-12)


def test_r_equatorial_config2_grid_vs_oracle(kg):
    """Full 512x512 grid of configuration 2 (seeded a, theta_o), orders 0..2, against the oracle."""
    from oracle import kgeo_oracle as ko
    from kgeo_gb300 import equatorial_lensing as el
    from kgeo_gb300 import device as dev
    rng = np.random.default_rng(0)
    a = float(rng.uniform(0, 0.998))
    th_o = float(rng.uniform(1, 89)) * np.pi / 180
    x = np.linspace(-10, 10, 512)
    A, B = np.meshgrid(x, x)
    A, B = A.flatten(), B.flatten()
    r_s, Ir, Imax, Nmax = (t.cpu().numpy() for t in el.r_equatorial_device(a, 1.e4, th_o, [0, 1, 2],
                                                                           dev.as_device(A), dev.as_device(B)))
    for m in range(3):
        rr, ir, imax, nmax = ko.r_equatorial(a, 1.e4, th_o, m, A, B)
        assert np.array_equal(Nmax, nmax)
        assert np.array_equal(r_s[m] == 0, rr == 0)
        np.testing.assert_allclose(r_s[m], rr, rtol=1e-10, atol=0)
        np.testing.assert_allclose(Ir[m], ir, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize('seed', [11, 12, 13])
def test_config2_draws_vs_oracle(kg, seed):
    """Seeded configuration-2 geometries (a ~ U[0, 0.998), theta_o ~ U[1, 89] deg, one mirrored
    below the equator), 40x40 over [-10, 10], ngeo = 400, through the default (recurrence) path."""
    from oracle import kgeo_oracle as ko
    rng = np.random.default_rng(seed)
    a = float(rng.uniform(0, 0.998))
    th_o = float(rng.uniform(1, 89)) * np.pi / 180
    if seed == 13:
        th_o = np.pi - th_o
    x = np.linspace(-10, 10, 40)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    ref = ko.raytrace(a, 1.e4, th_o, A, B, 400)
    got = _run(kg, a, 1.e4, th_o, A, B, 400)
    rho = ko.pole_distance(a, 1.e4, th_o, A, B, ref['mino_times'])
    refd = dict(t=ref['t'], r=ref['r'], th=ref['th'], ph=ref['ph'], sig=ref['affine_times'])
    check_trace(got, refd, 1.e4, ref['rclass'], 'config2-%d' % seed, rho=rho)
    # the theta / r only path on the same draws
    from kgeo_gb300 import device as dev
    res = dev.trace(a, 1.e4, th_o, dev.as_device(A), dev.as_device(B), ngeo=400, outputs=('r', 'th', 'mino'),
                    per_ray=())
    check_trace(dict(refd, r=res['r'].cpu().numpy(), th=res['th'].cpu().numpy()), refd, 1.e4, ref['rclass'],
                'config2-rth-%d' % seed, rho=rho)


@pytest.mark.parametrize('chunk', [1, 7, 50, 64])
def test_recurrence_matches_independent_samples(kg, chunk):
    """The addition-theorem recurrence (chunk > 1) against independent per-sample evaluation
    (chunk 0) on the same prepared rays: same classes, agreement within the parity bars."""
    import torch
    from oracle import kgeo_oracle as ko
    from kgeo_gb300 import device as dev
    x = np.linspace(-9, 9, 48)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    a, th_o = 0.8, 35 * np.pi / 180
    prep = dev.PreparedRays(a, 1.e4, th_o, dev.as_device(A), dev.as_device(B), ngeo=200)
    o0 = prep.samples(prep.alloc(fill=float('nan')), chunk=0)
    o1 = prep.samples(prep.alloc(fill=float('nan')), chunk=chunk)
    torch.cuda.synchronize()
    h0 = {k: v.cpu().numpy() for k, v in o0.items()}
    h1 = {k: v.cpu().numpy() for k, v in o1.items()}
    assert np.array_equal(h0['mino'], h1['mino'])
    rho = ko.pole_distance(a, 1.e4, th_o, A, B, h0['mino'])
    check_trace(h1, h0, 1.e4, prep.rclass.cpu().numpy(), 'chunk%d' % chunk, rho=rho)


@pytest.mark.parametrize('geom', [(0.94, 17.0), (0.3, 70.0), (0.7, 5.0), 'band'])
def test_mixed_precision_error_bars(kg, geom):
    """Mixed-precision (float-float) recurrence against the FP64 oracle: r 1e-8, theta 5e-7,
    phi 1e-6 (relative, floor 1), t and sigma 1e-7 of r_o, on 40x40 grids and on rays of the
    critical-curve band (0.94, 17 deg: 256 angles x the 16 offsets nearest the curve). Only the
    FP64 path's pole rule widens a bar (10 eps / rho, rho = |1 - n sn^2| the distance to an
    elliptic-Pi pole): within 1e-5 of a pole the mixed kernel re-seeds from the FP64 direct
    evaluation, so no sample is left to the float-float state's pole-amplified rounding."""
    import torch
    from oracle import kgeo_oracle as ko
    from kgeo_gb300 import device as dev
    from parity import rel_err, EPS
    if geom == 'band':
        from kgeo_gb300.equatorial_lensing import critical_band
        a, th = 0.94, 17 * np.pi / 180
        A, B = critical_band(a, th, n_angles=256, n_radii=256)
        A, B = (v.reshape(256, 256)[120:136].flatten() for v in (A, B))
    else:
        a, th = geom[0], geom[1] * np.pi / 180
        x = np.linspace(-10, 10, 40)
        A, B = (v.flatten() for v in np.meshgrid(x, x))
    ref = ko.raytrace(a, 1.e4, th, A, B, 256)
    prep = dev.PreparedRays(a, 1.e4, th, dev.as_device(A), dev.as_device(B), ngeo=256)
    out = prep.samples(prep.alloc(fill=float('nan')), mixed=True)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items()}
    assert np.array_equal(np.isfinite(got['ph']), np.isfinite(ref['ph']))
    rho = ko.pole_distance(a, 1.e4, th, A, B, ref['mino_times'])
    for k, rk, scale, bar in (('r', 'r', 1e-300, 1e-8), ('th', 'th', 1.0, 5e-7), ('ph', 'ph', 1.0, 1e-6),
                              ('t', 't', 1.e4, 1e-7), ('sig', 'affine_times', 1.e4, 1e-7)):
        e = rel_err(got[k], ref[rk], scale) / np.maximum(bar, 10 * EPS / rho)
        assert e.max() <= 1.0, (k, e.max())


def test_band_fixture_vs_reference(kg, golden):
    """Rays 2e-4 to 5e-2 M from the critical curve (a = 0.94, theta_o = 17 deg, ngeo = 256),
    against the reference's samples kept in the fixture (every 8th and the last)."""
    from oracle import kgeo_oracle as ko
    g = golden('band_a094_i17')
    a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
    got = _run(kg, a, r_o, th_o, g['alpha'], g['beta'], int(g['ngeo']))
    idx = g['samples']
    np.testing.assert_allclose(got['mino'][idx], g['mino'], rtol=1e-12, atol=0)
    full_tau = got['mino']
    rho = ko.pole_distance(a, r_o, th_o, g['alpha'], g['beta'], full_tau)[idx]
    sens = lambda_eta_sensitivity(a, r_o, th_o, g['alpha'], g['beta'], ngeo=int(g['ngeo']))
    sub = lambda cols: {k: v[idx] for k, v in sens(cols).items()}  # noqa: E731
    check_trace({k: got[k][idx] for k in ('t', 'r', 'th', 'ph', 'sig')},
                dict(t=g['t'], r=g['r'], th=g['th'], ph=g['ph'], sig=g['sig']), r_o, g['rclass'], 'band-fixture',
                rho=rho, sens=sub)


def test_band_vs_oracle(kg):
    """The critical-curve band of the 2048^2-plus-band workload (a = 0.94, theta_o = 17 deg,
    ngeo = 256) at 256 screen angles and the 16 radial offsets of linspace(-0.05, 0.05, 256)
    nearest the curve (|offset| 2e-4 to 3e-3 M), FP64 recurrence against the oracle."""
    import torch
    from oracle import kgeo_oracle as ko
    from kgeo_gb300.equatorial_lensing import critical_band
    A, B = critical_band(0.94, 17 * np.pi / 180, n_angles=256, n_radii=256)
    A, B = (v.reshape(256, 256)[120:136].flatten() for v in (A, B))
    a, r_o, th_o = 0.94, 1.e4, 17 * np.pi / 180
    ref = ko.raytrace(a, r_o, th_o, A, B, 256)
    got = _run(kg, a, r_o, th_o, A, B, 256)
    torch.cuda.synchronize()
    refd = dict(t=ref['t'], r=ref['r'], th=ref['th'], ph=ref['ph'], sig=ref['affine_times'])
    rho = ko.pole_distance(a, r_o, th_o, A, B, ref['mino_times'])
    check_trace(got, refd, r_o, ref['rclass'], 'band', rho=rho,
                sens=lambda_eta_sensitivity(a, r_o, th_o, A, B, ngeo=256))


@pytest.mark.parametrize('name', ['trace_region2_a094_i81', 'trace_region2_a099_i89', 'trace_region2_a081_i99'])
def test_region2_r_equatorial_vs_oracle(kg, golden, name):
    """Radial region II rays (four real roots, the ray ends on the horizon): r_s, Ir, Imax and
    Nmax of orders 0..2 against the oracle on the fixture's pixels."""
    from oracle import kgeo_oracle as ko
    from kgeo_gb300 import equatorial_lensing as el
    g = golden(name)
    a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
    assert (g['rclass'] == 2).sum() >= 20
    for m in range(3):
        r_s, Ir, Imax, Nmax = el.r_equatorial(a, r_o, th_o, m, g['alpha'], g['beta'])
        rr, ir, imax, nmax = ko.r_equatorial(a, r_o, th_o, m, g['alpha'], g['beta'])
        assert np.array_equal(Nmax, nmax)
        assert np.array_equal(r_s == 0, rr == 0)
        np.testing.assert_allclose(r_s, rr, rtol=1e-10, atol=0)
        np.testing.assert_allclose(Ir, ir, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(Imax, imax, rtol=1e-10, atol=1e-12)
    # the fixture's Mino totals are the reference's Imax of these rays
    got = kg.raytrace_ana(a=a, observer_coords=[0, r_o, th_o, 0], image_coords=[g['alpha'], g['beta']],
                          ngeo=int(g['ngeo']), plotdata=False)
    np.testing.assert_allclose(got.tautot, g['tau_tot'], rtol=1e-12, atol=0)


def test_no_loop_cap_on_fixture_traces(kg, golden):
    """No Carlson duplication or Landen descent stops at its iteration cap on any fixture's rays
    (setup and FP64 recurrence, and the mixed kernel): KGEO_FLAG_LOOP_CAP stays clear."""
    import torch
    from kgeo_gb300 import _lib, device as dev
    for name in TRACES + ['band_a094_i17']:
        g = golden(name)
        a, r_o, th_o = float(g['a']), float(g['r_o']), float(g['th_o'])
        res = dev.trace(a, r_o, th_o, dev.as_device(g['alpha']), dev.as_device(g['beta']), ngeo=int(g['ngeo']))
        torch.cuda.synchronize()
        assert not (int(res['flags'].item()) & _lib.FLAG_LOOP_CAP), name
        if not np.isfinite(r_o):
            continue
        prep = dev.PreparedRays(a, r_o, th_o, dev.as_device(g['alpha']), dev.as_device(g['beta']), ngeo=int(g['ngeo']))
        fl = torch.zeros(1, dtype=torch.int32, device='cuda')
        prep.samples(prep.alloc(), mixed=True, flags=fl)
        torch.cuda.synchronize()
        assert not (int(fl.item()) & _lib.FLAG_LOOP_CAP), name + '-mixed'


def test_recurrence_late_in_chunk_next_to_radial_pi_pole(kg):
    """Rays of the 2048^2 grid at a = 0.94, theta_o = 17 deg (ngeo = 256) whose radial Pi passes
    within rho ~ 1.0e-3 of its pole late in a 64-sample recurrence chunk, where the re-seed zone
    widens with the steps since the last direct Jacobi evaluation (phi was 1.21x the 1e-10 bar
    with a flat zone), FP64 path against the oracle."""
    import torch
    from oracle import kgeo_oracle as ko
    from conftest import PI_ZONE_RAYS
    a, r_o, th_o, ngeo = 0.94, 1.e4, 17 * np.pi / 180, 256
    x = np.linspace(-10, 10, 2048)
    A = np.array([x[j] for i, j in PI_ZONE_RAYS])
    B = np.array([x[i] for i, j in PI_ZONE_RAYS])
    ref = ko.raytrace(a, r_o, th_o, A, B, ngeo)
    got = _run(kg, a, r_o, th_o, A, B, ngeo)
    torch.cuda.synchronize()
    refd = dict(t=ref['t'], r=ref['r'], th=ref['th'], ph=ref['ph'], sig=ref['affine_times'])
    rho = ko.pole_distance(a, r_o, th_o, A, B, ref['mino_times'])
    check_trace(got, refd, r_o, ref['rclass'], 'pi-zone', rho=rho)


@pytest.mark.parametrize('part', ['grid', 'band'])
def test_config3_random_rays_vs_oracle(kg, part):
    """A seeded random 3,000 rays of the 2048^2-plus-band workload (a = 0.94, theta_o = 17 deg,
    ngeo = 256), grid or band, through the FP64 recurrence (chunks of 64) and the mixed kernel
    (chunks of 256) against the oracle, with the parity bars of oracle/parity.py: FP64 1e-10,
    mixed 1e-6, both widened by the pole rule and the input-conditioning allowance."""
    import torch
    from oracle import kgeo_oracle as ko
    from oracle.parity import parity_ratios
    from kgeo_gb300 import device as dev
    from kgeo_gb300.equatorial_lensing import critical_band
    a, th = 0.94, 17 * np.pi / 180
    rng = np.random.default_rng(17)
    if part == 'grid':
        x = np.linspace(-10, 10, 2048)
        i, j = rng.integers(0, 2048, 3000), rng.integers(0, 2048, 3000)
        A, B = x[j], x[i]
    else:
        bA, bB = critical_band(a, th, n_angles=4096, n_radii=256)
        k = rng.choice(bA.size, 3000, replace=False)
        A, B = bA[k], bB[k]
    ref = ko.raytrace(a, 1.e4, th, A, B, 256)
    refd = dict(t=ref['t'], r=ref['r'], th=ref['th'], ph=ref['ph'], sig=ref['affine_times'])
    rho = ko.pole_distance(a, 1.e4, th, A, B, ref['mino_times'])
    sens = lambda_eta_sensitivity(a, 1.e4, th, A, B, ngeo=256)
    prep = dev.PreparedRays(a, 1.e4, th, dev.as_device(A), dev.as_device(B), ngeo=256)
    for mixed, tol in ((False, 1e-10), (True, 1e-6)):
        out = prep.samples(prep.alloc(fill=float('nan')), mixed=mixed)
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in out.items()}
        for k in refd:
            assert np.array_equal(np.isfinite(got[k]), np.isfinite(refd[k])), (mixed, k)
        ratio = parity_ratios(got, refd, 1.e4, tol, rho, sens)
        worst = {k: float(v.max()) / tol for k, v in ratio.items()}
        assert max(worst.values()) <= 1.0, (mixed, worst)
