"""GPU parity of the jet field-line crossing solver (kgeo_jet_guesses / kgeo_jet_findroot)
through the drop-in kgeo_gb300.solver.findroot, on geodesics traced by the drop-in
raytrace_ana, against findroot of the reference (tests/golden/jet_crossings.npz).

Bars: the guess layout (shape) and, on the guesses that converge, the counts (signs of p_r,
p_theta, neq) exactly and tau, r, theta within 1e-9 relative (the secant stops on a 1e-8 step,
converging superlinearly; both sides then sit at the root to a few ulps, moved by the tracer's
own 1e-10-level parity)."""
import numpy as np
import pytest

from test_jet_cpu import jet_cases

pytestmark = pytest.mark.gpu


def test_findroot_fixture(golden):
    """The drop-in findroot against the reference's. scipy's array newton steps every guess
    until all have converged; a guess that does not converge (the reference warns) wanders for
    500 steps, and a converged one keeps stepping meanwhile: in the nearly face-on case with the
    flat-space guesses (case 3) a quarter of the guesses never converge and the reference's
    converged ones partly end on other roots of the same objective (39 at negative Mino times).
    So: every guess this solver reports converged is a root of the oracle's objective; where
    the reference reached the same root (always but case 3), tau, r, theta agree to 1e-9 and
    the signs and neq exactly."""
    from kgeo_gb300 import solver
    from kgeo_gb300.kerr_raytracing_ana import raytrace_ana
    from oracle import kgeo_oracle as ko
    g = golden('jet_crossings')
    for i, a, th_o, model, psit, pval, neqmax, A, B in jet_cases(g):
        geo = raytrace_ana(a=a, observer_coords=[0, 1.e4, th_o, 0], image_coords=[A, B], ngeo=200, plotdata=False)
        res = solver.findroot(geo, psit, A, B, 1.e4, th_o, a, 200, model=model, neqmax=neqmax, tol=1e-8, pval=pval)
        assert tuple(res[6]) == tuple(g['shape%d' % i]), (i, res[6])
        guesses = solver.getguesses(geo, a, 1.e4, th_o, A, B, psit, 200, neqmax=neqmax, model=model, pval=pval)
        st = solver.findroot_device(a, 1.e4, th_o, A, B, guesses, psit, model=model, pval=pval)['status']
        ours = (st == 0).cpu().numpy().reshape(-1)
        theirs = ko.findroot(dict(r=geo.r_s, th=geo.th_s, mino_times=geo.mino_times), psit, A, B, 1.e4, th_o, a,
                             200, model=model, neqmax=neqmax, tol=1e-8, pval=pval, converged=True)[7]
        live = guesses.reshape(-1) != -1
        # no-crossing entries: zeros, and neq at the secant's flat-pair end point
        for k, j in (('tau', 0), ('r', 1), ('th', 2), ('signpr', 3), ('signpth', 4)):
            assert np.all(res[j][~live] == 0), (i, k)
        assert np.array_equal(res[5][~live], g['neq%d' % i][~live]), i
        # every converged solve is a root of the reference's objective
        G = res[6][0]
        At, Bt = np.tile(A, G), np.tile(B, G)
        _, (_, r0, th0, _) = ko.coords_at_tau(a, 1.e4, th_o, At, Bt, res[0].reshape(1, -1))
        fval = ko.psifunc(r0[0], th0[0], a, model=model, pval=pval) - psit
        mine = ours & live
        assert np.all(np.abs(fval[mine]) <= 1e-6 * max(1.0, abs(psit))), (i, np.nanmax(np.abs(fval[mine])))
        tref = g['tau%d' % i]
        same = mine & theirs & (np.abs(res[0] - tref) <= 1e-6 * np.maximum(np.abs(tref), 1e-12))
        if i != 3:
            assert np.array_equal(ours[live], theirs[live]), (i, int((ours != theirs)[live].sum()))
            assert np.array_equal(same, mine), (i, int((same != mine).sum()))
        else:
            assert same.sum() >= 0.5 * (mine & theirs).sum(), (i, int(same.sum()), int((mine & theirs).sum()))
        for k, j in (('signpr', 3), ('signpth', 4), ('neq', 5)):
            ref = g['%s%d' % (k, i)][same]
            got = res[j][same]
            bad = ~((got == ref) | (np.isnan(got) & np.isnan(ref)))
            assert not bad.any(), (i, k, int(bad.sum()))
        for k, j in (('tau', 0), ('r', 1), ('th', 2)):
            ref = g['%s%d' % (k, i)][same]
            got = res[j][same]
            assert np.allclose(got, ref, rtol=1e-9, atol=1e-12, equal_nan=True), \
                (i, k, np.nanmax(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)))


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
