"""CPU checks of the jet field-line crossing solver: the oracle restatement of
kgeo/solver.py (getguesses, findroot with scipy.optimize.newton, getneq) against findroot of the
reference itself on sampled geodesic sets (para / mono / power field lines, neqmax 1 and 2, both
hemispheres, the nearly face-on flat-space guesses)."""
import warnings

import numpy as np

from oracle import kgeo_oracle as ko

DEG = np.pi / 180


def jet_cases(g):
    for i in range(int(g['ncase'])):
        a, inc, model, psit, pval, neqmax, nside, lim = eval(str(g['case%d' % i]))
        x = np.linspace(-lim, lim, nside)
        A, B = (v.flatten() for v in np.meshgrid(x, x))
        yield i, a, inc * DEG, model, psit, pval, neqmax, A, B


def test_oracle_findroot(golden):
    g = golden('jet_crossings')
    for i, a, th_o, model, psit, pval, neqmax, A, B in jet_cases(g):
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            geo = ko.raytrace(a, 1.e4, th_o, A, B, 200)
            res = ko.findroot(geo, psit, A, B, 1.e4, th_o, a, 200, model=model, neqmax=neqmax, tol=1e-8, pval=pval)
        assert tuple(res[6]) == tuple(g['shape%d' % i]), i
        for k, j in (('signpr', 3), ('signpth', 4), ('neq', 5)):
            assert np.array_equal(res[j], g['%s%d' % (k, i)], equal_nan=True), (i, k)
        for k, j in (('tau', 0), ('r', 1), ('th', 2)):
            ref = g['%s%d' % (k, i)]
            assert np.allclose(res[j], ref, rtol=1e-12, atol=1e-12, equal_nan=True), (i, k)
