"""GPU checks of the Geodesics-side extras: n_angular_turnings against the reference's
fixture, the calc_t_equatorial consistency check (crossing coordinates of raytrace vs
r_equatorial) with the reference script's bounds, the crossing counts re-exported from
kerr_raytracing_utils, and the HDF5 round trip when h5py is present."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEG = np.pi / 180


def test_n_angular_turnings_fixture(golden):
    from kgeo_gb300.kerr_raytracing_utils import n_angular_turnings
    g = golden('angular_turnings')
    for i in range(5):
        a, th = g['par%d' % i]
        A, B, tau = g['alpha%d' % i], g['beta%d' % i], g['tau%d' % i]
        n = n_angular_turnings(float(a), float(th) * DEG, A, B, tau)
        n1 = n_angular_turnings(float(a), float(th) * DEG, A, B, tau[2])
        ref = g['n%d' % i]
        assert n.shape == ref.shape and n1.shape == g['n1_%d' % i].shape
        assert np.array_equal(np.isnan(n), np.isnan(ref)), i
        scale = np.maximum(np.abs(ref), 1.0)
        assert np.nanmax(np.abs(n - ref) / scale) <= 1e-11, (i, np.nanmax(np.abs(n - ref) / scale))
        assert np.nanmax(np.abs(n1 - g['n1_%d' % i]) / scale[2]) <= 1e-11, i
    with pytest.raises(Exception, match=r"th_o should be a float in range \(0,pi/2\]"):
        n_angular_turnings(0.5, 100 * DEG, A, B, tau)


@pytest.mark.parametrize('spin,inc', [(0.99, 60.), (0.5, 17.), (0.3, 120.)])
def test_equatorial_consistency(spin, inc):
    """scripts/calc_t_equatorial.py: theta = pi/2 to 1e-14 and r = r_s to
    max(1e-12, 32 eps tau r_s) at the crossing Mino times of orders 0..2 (r_o = 1e6 as the
    script); the flat 1e-12 holds at the 99.9th percentile (measured <= 2.6e-13)."""
    from kgeo_gb300.equatorial_images import image_pixels
    from kgeo_gb300.equatorial_lensing import equatorial_consistency
    A, B = image_pixels(-7., 7., -7., 7., 0.05)
    out = equatorial_consistency(spin, 1.e6, inc * DEG, A, B, mbar_max=2)
    for m, (dth, dr, q) in out.items():
        assert dth <= 1e-14 and q <= 1, (m, dth, dr, q)
        if m == 0:
            assert dr <= 1e-12, (m, dr)


def test_crossing_reexports():
    from kgeo_gb300 import kerr_raytracing_utils as ku
    from oracle import kgeo_oracle as ko
    rng = np.random.default_rng(1)
    A, B = rng.uniform(-8, 8, 500), rng.uniform(-8, 8, 500)
    tau = rng.uniform(0, 2, (3, 500))
    assert np.array_equal(ku.n_equatorial_crossings(0.7, 0.5, A, B, tau), ko.n_equatorial_crossings(0.7, 0.5, A, B, tau))
    assert np.array_equal(ku.is_outside_crit(0.7, 0.5, A, B), ko.outside_critical(0.7, 0.5, A, B))
    assert np.allclose(ku.n_poloidal_orbits(0.7, 0.5, A, B, tau), ko.n_poloidal_orbits(0.7, 0.5, A, B, tau),
                       rtol=1e-12, atol=0)


def test_savegeos_roundtrip(tmp_path):
    pytest.importorskip('h5py')
    from kgeo_gb300.kerr_raytracing_ana import raytrace_ana
    from kgeo_gb300.kerr_raytracing_utils import loadgeos
    A = np.linspace(-5, 5, 40)
    g = raytrace_ana(a=0.5, observer_coords=[0, 1.e4, 1.0, 0], image_coords=[A, 0 * A], ngeo=20, plotdata=False)
    fn = str(tmp_path / 'geo.h5')
    g.savegeos(outfile=fn)
    h = loadgeos(fn)
    for k in ('t_s', 'r_s', 'th_s', 'ph_s', 'sig_s', 'tausteps'):
        assert np.array_equal(getattr(g, k), getattr(h, k)), k
    assert h.a == g.a and h.th_o == g.th_o and h.r_o == g.r_o
