"""GPU parity of the equatorial image (kgeo_image) and its adjoint (kgeo_image_adjoint)
through the drop-in make_image / Iobs and the autograd Function: against the reference's
make_image fixtures, the oracle, central finite differences and the pure-torch FP64
autograd restatement."""
import numpy as np
import pytest
import torch

from oracle import kgeo_oracle as ko
from oracle import kgeo_torch_ref as tr

pytestmark = pytest.mark.gpu

DEG = np.pi / 180
CFG5 = dict(a=0.5, th_o=60 * DEG, r_o=1.e4, p=2.0, xi=0.8, beta_r=0.5)


def rel(x, ref, floor=1e-300):
    d = np.abs(x - ref) / np.maximum(np.abs(ref), floor)
    return np.nanmax(d) if np.isfinite(d).any() else 0.0


def _objects(emis, vel):
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.velocities import Velocity
    return Emissivity(emis[0], **emis[1]), Velocity(vel[0], **vel[1])


def test_make_image_models_fixture(golden):
    from kgeo_gb300.equatorial_images import make_image
    g = golden('image_models')
    for i in range(int(g['ncase'])):
        a, th, mm, et, ek, vt, vk = eval(str(g['case%d' % i]))
        em, ve = _objects((et, ek), (vt, vk))
        res = make_image(a, 1.e4, th * DEG, mm, -9., 9., -9., 9., float(g['psize']), emissivity=em, velocity=ve)
        for k, v, tol in zip(['I', 'Q', 'U', 'r', 't', 'g', 'sinthb', 'n', 'np'], res,
                             [1e-10, 0, 0, 1e-10, 1e-12, 1e-10, 0, 0, 1e-12]):
            ref = g['%s%d' % (k, i)]
            assert v.shape == ref.shape, (i, k)
            assert np.array_equal(np.isnan(v), np.isnan(ref)), (i, k)
            assert rel(v, ref) <= tol, (i, k, rel(v, ref))
        assert np.array_equal(res[0] > 0, g['I%d' % i] > 0), i


def test_make_image_config5_fixture(golden):
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.equatorial_images import make_image
    from kgeo_gb300.velocities import Velocity
    g = golden('image_a05_i60')
    res = make_image(float(g['a']), float(g['r_o']), float(g['th_o']), 2, -8., 8., -8., 8., float(g['psize']),
                     emissivity=Emissivity('bpl', p1=-2.0, p2=0.0),
                     velocity=Velocity('general', fac_subkep=0.8, beta_r=0.5))
    assert rel(res[0], g['I']) <= 1e-10
    assert rel(res[3], g['r']) <= 1e-10
    assert rel(res[5], g['g']) <= 1e-10
    assert np.array_equal(res[7], g['n'])
    assert rel(res[8], g['np_']) <= 1e-12


def test_iobs_matches_oracle():
    from kgeo_gb300.equatorial_images import Iobs
    c = CFG5
    x = np.linspace(-8, 8, 64)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    em, ve = _objects(('bpl', {'p1': -2.0, 'p2': 0.0}), ('general', {'fac_subkep': 0.8, 'beta_r': 0.5}))
    for m in (0, 1, 2):
        got = Iobs(c['a'], c['r_o'], c['th_o'], m, A, B, emissivity=em, velocity=ve)
        I, gg, r_s, Ir, Imax, Nmax = ko.image_order(c['a'], c['r_o'], c['th_o'], m, A, B, p1=-2.0, p2=0.0,
                                                    fac_subkep=0.8, beta_r=0.5)
        assert rel(got[0], I) <= 1e-10 and rel(got[3], gg) <= 1e-10 and rel(got[4], r_s) <= 1e-10
        assert rel(got[6], Ir) <= 1e-12 and rel(got[7], Imax) <= 1e-12
        assert np.array_equal(got[8], Nmax)
        assert np.array_equal(got[5] > 0, I > 0)


def test_image_config5_vs_oracle_subgrid():
    """The configuration-5 image (512 x 512 over [-8, 8] M) against the oracle on every 4th
    pixel of each axis."""
    from kgeo_gb300.equatorial_images import emission_model, image_device
    c = CFG5
    x = np.linspace(-8, 8, 512)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    em, ve = _objects(('bpl', {'p1': -2.0, 'p2': 0.0}), ('general', {'fac_subkep': 0.8, 'beta_r': 0.5}))
    model = emission_model(em, ve)
    res = image_device(c['a'], c['r_o'], c['th_o'], 0, 3, torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(),
                       model, outputs=('I', 'g', 'nmax'))
    I = res['I'].cpu().numpy()
    sub = (np.arange(512)[:, None] % 4 == 0) & (np.arange(512)[None, :] % 4 == 0)
    sub = sub.flatten()
    o = ko.make_image_px(c['a'], c['r_o'], c['th_o'], 2, A[sub], B[sub], emis=('bpl', {'p1': -2.0, 'p2': 0.0}),
                         vel=('general', {'fac_subkep': 0.8, 'beta_r': 0.5}))
    assert np.array_equal(I[sub] > 0, o['I'] > 0)
    assert rel(I[sub], o['I']) <= 1e-10
    assert np.array_equal(res['nmax'].cpu().numpy()[sub], o['n'])


def test_model_errors():
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.equatorial_images import make_image
    from kgeo_gb300.velocities import Velocity
    with pytest.raises(Exception, match=r"fac_subkep should be in the range \[0,1\]"):
        make_image(0.5, 1.e4, 1.0, 1, -4., 4., -4., 4., 1.0, velocity=Velocity('subkep', fac_subkep=1.5))
    with pytest.raises(Exception, match=r"beta_r should be in the range \[0,1\]"):
        make_image(0.5, 1.e4, 1.0, 1, -4., 4., -4., 4., 1.0, velocity=Velocity('general', beta_r=-0.1))
    with pytest.raises(Exception, match="mbar_max should be an integer >=0!"):
        make_image(0.5, 1.e4, 1.0, -1, -4., 4., -4., 4., 1.0)
    from kgeo_gb300.bfields import Bfield
    with pytest.raises(NotImplementedError):
        make_image(0.5, 1.e4, 1.0, 1, -4., 4., -4., 4., 1.0, polarization=True,
                   bfield=Bfield('const_comoving', Cr=1.))
    with pytest.raises(Exception, match="all field coefficients are 0!"):
        Bfield('simple')
    with pytest.raises(NotImplementedError):
        make_image(0.5, 1.e4, 1.0, 1, -4., 4., -4., 4., 1.0, velocity=Velocity('gelles'))
    with pytest.raises(Exception, match="th_o should be a float"):
        make_image(0.5, 1.e4, np.pi / 2, 1, -4., 4., -4., 4., 1.0, emissivity=Emissivity('constant'))


def _cfg5_pixels(n=512):
    x = np.linspace(-8, 8, n)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    return torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()


def _loss_setup(n=512):
    """L = sum (I - I_target)^2 with the target rendered at the parameters perturbed by
    2 % with signs from default_rng(0)."""
    from kgeo_gb300.image_grad import config_params, equatorial_image
    c = CFG5
    al, be = _cfg5_pixels(n)
    phys = np.array([c['a'], c['th_o'], c['p'], c['xi'], c['beta_r']])
    eps = np.random.default_rng(0).choice([-1.0, 1.0], size=5)
    with torch.no_grad():
        target = equatorial_image(config_params(*(phys * (1 + 0.02 * eps))), al, be)

    def loss(x):
        I = equatorial_image(config_params(*x), al, be)
        return ((I - target) ** 2).sum()
    return phys, loss


def test_adjoint_gradient_vs_central_differences():
    """Configuration 5 at full size: the adjoint gradient of L with respect to (a, th_o, p,
    xi, beta_r) against FP64 central differences (step 1e-6) of the GPU image."""
    phys, loss = _loss_setup()
    x = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in phys]
    L = loss(x)
    L.backward()
    grad = np.array([float(v.grad) for v in x])
    h = 1e-6
    for k in range(5):
        xp = list(phys)
        xm = list(phys)
        xp[k] += h
        xm[k] -= h
        with torch.no_grad():
            fd = (float(loss(xp)) - float(loss(xm))) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-4 * abs(fd), (k, fd, grad[k])


def test_adjoint_vs_oracle_central_differences():
    """The adjoint gradient against central differences (step 1e-6) of the numpy oracle's
    image, on a 96 x 96 grid."""
    from kgeo_gb300.image_grad import config_params, equatorial_image
    c = CFG5
    n = 96
    x = np.linspace(-8, 8, n)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    al, be = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    phys = np.array([c['a'], c['th_o'], c['p'], c['xi'], c['beta_r']])
    eps = np.random.default_rng(0).choice([-1.0, 1.0], size=5)

    def oracle_I(ph):
        o = ko.make_image_px(float(ph[0]), c['r_o'], float(ph[1]), 2, A, B, emis=('bpl', {'p1': -ph[2], 'p2': 0.0}),
                             vel=('general', {'fac_subkep': ph[3], 'beta_r': ph[4]}))
        return o['I']
    target = oracle_I(phys * (1 + 0.02 * eps))
    xs = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in phys]
    I = equatorial_image(config_params(*xs), al, be)
    L = ((I - torch.from_numpy(target).cuda()) ** 2).sum()
    L.backward()
    grad = np.array([float(v.grad) for v in xs])
    h = 1e-6
    for k in range(5):
        xp = phys.copy()
        xm = phys.copy()
        xp[k] += h
        xm[k] -= h
        fd = (((oracle_I(xp) - target) ** 2).sum() - ((oracle_I(xm) - target) ** 2).sum()) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-4 * abs(fd), (k, fd, grad[k])


def test_adjoint_vs_torch_autograd():
    """The adjoint kernel against the pure-torch FP64 restatement differentiated by autograd."""
    from kgeo_gb300.image_grad import equatorial_image
    c = CFG5
    x = np.linspace(-8, 8, 40)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    emis = ('bpl', {'p1': -c['p'], 'p2': 0.0})
    vel = ('general', {'fac_subkep': c['xi'], 'beta_r': c['beta_r']})
    geo, _ = tr.geometry(ko, c['a'], c['r_o'], c['th_o'], A, B, 2, emis, vel)
    p0 = [c['a'], c['th_o'], -c['p'], 0.0, c['xi'], 1.0, c['beta_r']]
    w = torch.from_numpy(np.random.default_rng(5).standard_normal((A.size, 3)))
    pt = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    (w * tr.image(pt, c['r_o'], A, B, 2, geo=geo)).sum().backward()
    pg = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    (w.cuda() * equatorial_image(pg, A, B)).sum().backward()
    np.testing.assert_allclose(pg.grad.numpy(), pt.grad.numpy(), rtol=1e-8, atol=0)


def test_adjoint_deterministic_and_model_variants():
    """Two adjoint launches give identical sums; other velocity / emissivity models agree
    with central differences of the GPU forward."""
    from kgeo_gb300.image_grad import equatorial_image
    al, be = _cfg5_pixels(128)
    w = torch.from_numpy(np.random.default_rng(9).standard_normal((al.numel(), 2))).cuda()
    for emis, vel, p0, th in (('bpl', 'general', [0.5, 1.0, -2.0, -0.2, 0.8, 0.7, 0.5], 1.0),
                              ('glm', 'subkep', [0.9, 2.0, -1.5, 0.5, 0.6, 1.0, 1.0], 2.0),
                              ('ring', 'kep', [0.3, 0.6, 0.2, 0.4, 1.0, 1.0, 1.0], 0.6)):
        kw = dict(mbar_max=1, emissivity=emis, velocity=vel, mu_ring=4.0 if emis == 'ring' else 0.0)
        grads = []
        for _ in range(2):
            p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
            (w * equatorial_image(p, al, be, **kw)).sum().backward()
            grads.append(p.grad.clone())
        assert torch.equal(grads[0], grads[1])
        g = grads[0].numpy()
        h = 1e-6
        for q in range(7):
            if g[q] == 0 and q >= 2:
                continue
            pp, pm = list(p0), list(p0)
            pp[q] += h
            pm[q] -= h
            with torch.no_grad():
                fd = (float((w * equatorial_image(torch.tensor(pp, dtype=torch.float64), al, be, **kw)).sum()) -
                      float((w * equatorial_image(torch.tensor(pm, dtype=torch.float64), al, be, **kw)).sum())) / (2 * h)
            assert abs(fd - g[q]) <= 1e-4 * max(abs(fd), 1e-8), (emis, vel, q, fd, g[q])
