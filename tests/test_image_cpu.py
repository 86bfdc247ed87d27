"""CPU checks of the equatorial image and its adjoint: the oracle against the reference's
make_image fixtures, the image kernel's arithmetic (the device headers built for the host)
against the same fixtures, its dual-number Jacobian against central finite differences,
and against the pure-torch FP64 autograd restatement."""
import numpy as np
import pytest
import torch

import hmlib
from oracle import kgeo_oracle as ko
from oracle import kgeo_torch_ref as tr

DEG = np.pi / 180
CFG5 = dict(a=0.5, th_o=60 * DEG, r_o=1.e4, p=2.0, xi=0.8, beta_r=0.5)


def rel(x, ref, floor=1e-300):
    d = np.abs(x - ref) / np.maximum(np.abs(ref), floor)
    return np.nanmax(d) if np.isfinite(d).any() else 0.0


def cases(g):
    for i in range(int(g['ncase'])):
        a, th, mm, et, ek, vt, vk = eval(str(g['case%d' % i]))
        yield i, a, th * DEG, mm, (et, ek), (vt, vk)


def test_oracle_make_image_models(golden):
    g = golden('image_models')
    for i, a, th_o, mm, emis, vel in cases(g):
        o = ko.make_image_px(a, 1.e4, th_o, mm, g['alpha'], g['beta'], emis=emis, vel=vel)
        for k in ('I', 'Q', 'U', 'r', 't', 'g', 'sinthb', 'n', 'np'):
            ref = g['%s%d' % (k, i)]
            assert np.array_equal(np.isnan(o[k]), np.isnan(ref)), (i, k)
            assert rel(o[k], ref) <= 1e-14, (i, k, rel(o[k], ref))


def test_host_image_models(golden):
    """The image kernel's arithmetic (host build) against make_image of the reference."""
    g = golden('image_models')
    for i, a, th_o, mm, emis, vel in cases(g):
        mi, md = hmlib.model_arrays(emis, vel)
        h = hmlib.image(a, 1.e4, th_o, g['alpha'], g['beta'], mm + 1, mi, md)
        for k, hk, tol in (('I', 'I', 1e-10), ('r', 'r_s', 1e-10), ('t', 'Ir', 1e-12), ('g', 'g', 1e-10),
                           ('sinthb', 'sinthb', 0), ('n', 'nmax', 0), ('np', 'npol', 1e-12)):
            ref = g['%s%d' % (k, i)]
            assert np.array_equal(np.isnan(h[hk]), np.isnan(ref)), (i, k)
            assert np.array_equal(h[hk] > 0, ref > 0) or k in ('t', 'np', 'r'), (i, k)
            assert rel(h[hk], ref) <= tol, (i, k, rel(h[hk], ref))


def test_host_image_config5_fixture(golden):
    g = golden('image_a05_i60')
    emis = ('bpl', {'p1': float(g['p1']), 'p2': float(g['p2'])})
    vel = ('general', {'fac_subkep': float(g['fac_subkep']), 'beta_r': float(g['beta_r'])})
    mi, md = hmlib.model_arrays(emis, vel)
    h = hmlib.image(float(g['a']), float(g['r_o']), float(g['th_o']), g['alpha'], g['beta'], 3, mi, md)
    assert rel(h['I'], g['I']) <= 1e-10
    assert rel(h['g'], g['g']) <= 1e-10
    assert np.array_equal(h['nmax'], g['n'])


def _grid(n, lim=8.0):
    x = np.linspace(-lim, lim, n)
    A, B = np.meshgrid(x, x)
    return A.flatten(), B.flatten()


def test_host_jacobian_vs_central_differences():
    """dI/dq of the dual-number chain against central differences (step 1e-6) of the same
    FP64 image, per pixel and order, at the configuration-5 parameters."""
    c = CFG5
    A, B = _grid(40)
    emis = ('bpl', {'p1': -c['p'], 'p2': 0.0})
    vel = ('general', {'fac_subkep': c['xi'], 'beta_r': c['beta_r'], 'beta_phi': 0.9})
    mi, md = hmlib.model_arrays(emis, vel)
    jac, _ = hmlib.image_jac(c['a'], c['r_o'], c['th_o'], A, B, 3, mi, md)
    h = 1e-6

    def img(a, th, md_):
        return hmlib.image(a, c['r_o'], th, A, B, 3, mi, md_)['I']
    slots = {2: 0, 3: 1, 4: 3, 5: 4, 6: 5}
    for q in range(7):
        if q == 0:
            fd = (img(c['a'] + h, c['th_o'], md) - img(c['a'] - h, c['th_o'], md)) / (2 * h)
        elif q == 1:
            fd = (img(c['a'], c['th_o'] + h, md) - img(c['a'], c['th_o'] - h, md)) / (2 * h)
        else:
            mp, mm_ = md.copy(), md.copy()
            mp[slots[q]] += h
            mm_[slots[q]] -= h
            fd = (img(c['a'], c['th_o'], mp) - img(c['a'], c['th_o'], mm_)) / (2 * h)
        J = jac[:, :, q]
        scale = np.abs(J).max()
        assert scale > 0
        err = np.abs(fd - J)
        # pixels whose mask or momentum sign flips inside the step are not differentiable
        ok = err <= 1e-5 * np.abs(J) + 1e-7 * scale
        assert ok.mean() > 0.999, (q, ok.mean())
        assert abs(fd[ok].sum() - J[ok].sum()) <= 1e-6 * np.abs(J[ok]).sum(), q


def test_torch_autograd_matches_host_jacobian():
    """The pure-torch FP64 restatement, differentiated by torch.autograd, against the dual
    Jacobian the adjoint kernel uses, contracted with a random upstream gradient."""
    c = CFG5
    A, B = _grid(36)
    emis = ('bpl', {'p1': -c['p'], 'p2': 0.0})
    vel = ('general', {'fac_subkep': c['xi'], 'beta_r': c['beta_r']})
    geo, o = tr.geometry(ko, c['a'], c['r_o'], c['th_o'], A, B, 2, emis, vel)
    params = torch.tensor([c['a'], c['th_o'], -c['p'], 0.0, c['xi'], 1.0, c['beta_r']], dtype=torch.float64,
                          requires_grad=True)
    I = tr.image(params, c['r_o'], A, B, 2, geo=geo)
    assert rel(I.detach().numpy(), o['I']) <= 1e-10
    w = torch.from_numpy(np.random.default_rng(3).standard_normal(tuple(I.shape)))
    (w * I).sum().backward()
    mi, md = hmlib.model_arrays(emis, vel)
    jac, _ = hmlib.image_jac(c['a'], c['r_o'], c['th_o'], A, B, 3, mi, md)
    gh = np.einsum('pm,pmq->q', w.numpy(), jac)
    np.testing.assert_allclose(params.grad.numpy(), gh, rtol=1e-9, atol=0)
