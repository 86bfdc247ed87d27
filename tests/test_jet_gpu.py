"""GPU parity of the jet field-line crossing solver (kgeo_jet_guesses / kgeo_jet_findroot)
through the drop-in kgeo_gb300.solver.findroot, on geodesics traced by the drop-in
raytrace_ana, against findroot of the reference (tests/golden/jet_crossings.npz).

Bars: the guess layout (shape) and the counts (signs of p_r, p_theta, neq) exactly; tau, r,
theta within 1e-9 relative (the secant stops on a 1e-8 step, converging superlinearly; both
sides then sit at the root to a few ulps, moved by the tracer's own 1e-10-level parity)."""
import numpy as np
import pytest

from test_jet_cpu import jet_cases

pytestmark = pytest.mark.gpu


def test_findroot_fixture(golden):
    from kgeo_gb300.kerr_raytracing_ana import raytrace_ana
    from kgeo_gb300.solver import findroot
    g = golden('jet_crossings')
    for i, a, th_o, model, psit, pval, neqmax, A, B in jet_cases(g):
        geo = raytrace_ana(a=a, observer_coords=[0, 1.e4, th_o, 0], image_coords=[A, B], ngeo=200, plotdata=False)
        res = findroot(geo, psit, A, B, 1.e4, th_o, a, 200, model=model, neqmax=neqmax, tol=1e-8, pval=pval)
        assert tuple(res[6]) == tuple(g['shape%d' % i]), (i, res[6])
        for k, j in (('signpr', 3), ('signpth', 4), ('neq', 5)):
            ref = g['%s%d' % (k, i)]
            bad = ~((res[j] == ref) | (np.isnan(res[j]) & np.isnan(ref)))
            assert not bad.any(), (i, k, int(bad.sum()))
        for k, j in (('tau', 0), ('r', 1), ('th', 2)):
            ref = g['%s%d' % (k, i)]
            assert np.allclose(res[j], ref, rtol=1e-9, atol=1e-12, equal_nan=True), \
                (i, k, np.nanmax(np.abs(res[j] - ref) / np.maximum(np.abs(ref), 1e-12)))


def test_guesses_and_taumax_vs_oracle():
    from kgeo_gb300.kerr_raytracing_ana import raytrace_ana
    from kgeo_gb300.solver import get_maxtau_forwardjet, getguesses
    from oracle import kgeo_oracle as ko
    x = np.linspace(-9, 9, 30)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    for a, th, neqmax in ((0.8, 30 * np.pi / 180, 1), (0.4, 100 * np.pi / 180, 2), (0.6, 1.0, None)):
        t = get_maxtau_forwardjet(a, 1.e4, th, A, B, neqmax=neqmax)
        to = ko.get_maxtau_forwardjet(a, 1.e4, th, A, B, neqmax=neqmax)
        assert np.allclose(t, to, rtol=1e-12, atol=0, equal_nan=True)
        geo = raytrace_ana(a=a, observer_coords=[0, 1.e4, th, 0], image_coords=[A, B], ngeo=150, plotdata=False)
        gg = getguesses(geo, a, 1.e4, th, A, B, 1.2, 150, neqmax=neqmax or 1, model='para')
        ref = ko.getguesses(dict(r=geo.r_s, th=geo.th_s, mino_times=geo.mino_times), a, 1.e4, th, A, B, 1.2, 150,
                            neqmax=neqmax or 1, model='para')
        assert gg.shape == ref.shape
        assert np.array_equal(gg == -1, ref == -1)
        assert np.allclose(gg, ref, rtol=1e-15, atol=0)


def test_findroot_errors():
    from kgeo_gb300.solver import findroot_device
    with pytest.raises(NotImplementedError):
        findroot_device(0.5, 1.e4, 1.0, np.zeros(2), np.zeros(2), -np.ones((1, 2)), 1.0, model='other')
