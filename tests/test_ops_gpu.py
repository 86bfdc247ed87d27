"""The kgeo torch operators on the GPU: the same kernels as the drop-in functions (identical
outputs), the reference's exceptions, the image operator's autograd through the adjoint
kernel, and torch.library.opcheck's schema and fake-tensor checks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A, R_O, TH_O = 0.6, 1.e4, 0.5


def pixels(n=24):
    import torch
    x = np.linspace(-8, 8, n)
    a, b = (v.flatten() for v in np.meshgrid(x, x))
    return torch.tensor(a, device='cuda'), torch.tensor(b, device='cuda')


def test_raytrace_and_coords_ops_equal_dropins():
    import torch
    from kgeo_gb300 import ops  # noqa: F401
    from kgeo_gb300.kerr_raytracing_ana import coords_at_tau, raytrace_ana
    al, be = pixels()
    mino, sig, t, r, th, ph = torch.ops.kgeo.raytrace(al, be, A, R_O, TH_O, 50, 1 - 1e-10)
    g = raytrace_ana(a=A, observer_coords=[0, R_O, TH_O, 0], image_coords=[al, be], ngeo=50, plotdata=False,
                     device_arrays=True)
    for x, y in ((mino, g.mino_times), (sig, g.affine_times), (t, g.geo_coords[0]), (r, g.geo_coords[1]),
                 (th, g.geo_coords[2]), (ph, g.geo_coords[3])):
        assert torch.equal(torch.nan_to_num(x), torch.nan_to_num(y))
    tau = mino[10:13].contiguous()
    out = torch.ops.kgeo.coords_at_tau(al, be, tau, A, R_O, TH_O, True)
    sig2, coords = coords_at_tau(A, [0, R_O, TH_O, 0], [al, be], tau, device_arrays=True)
    for x, y in zip(out, [sig2] + list(coords)):
        assert torch.equal(torch.nan_to_num(x), torch.nan_to_num(torch.as_tensor(y, device='cuda')))


def test_r_equatorial_op_equals_device_function():
    import torch
    from kgeo_gb300 import ops  # noqa: F401
    from kgeo_gb300.equatorial_lensing import r_equatorial_device
    al, be = pixels()
    got = torch.ops.kgeo.r_equatorial(al, be, A, R_O, TH_O, 0, 3)
    ref = r_equatorial_device(A, R_O, TH_O, range(3), al, be)
    for x, y in zip(got, ref):
        assert torch.equal(x, y)


def test_image_op_forward_backward_equal_image_grad():
    import torch
    from kgeo_gb300 import ops  # noqa: F401
    from kgeo_gb300.image_grad import equatorial_image
    al, be = pixels(20)
    p0 = torch.tensor([A, TH_O, -2.0, -0.5, 0.7, 0.8, 0.6], dtype=torch.float64, requires_grad=True)
    I = torch.ops.kgeo.image(p0, al, be, R_O, 2, 'bpl', 'general')
    w = torch.linspace(0, 1, I.numel(), dtype=torch.float64, device='cuda').reshape(I.shape)
    (I * w).sum().backward()
    p1 = p0.detach().clone().requires_grad_(True)
    I1 = equatorial_image(p1, al, be, r_o=R_O, mbar_max=2, emissivity='bpl', velocity='general')
    (I1 * w).sum().backward()
    assert torch.equal(I, I1)
    assert torch.equal(p0.grad, p1.grad)


def test_jet_stokes_op_equals_stokes_device():
    import torch
    from kgeo_gb300 import off_eq, ops  # noqa: F401
    from kgeo_gb300 import device as dev
    from kgeo_gb300 import solver
    al, be = pixels(32)
    geo = dev.trace(0.5, R_O, 1.0, al, be, ngeo=200, outputs=('r', 'th', 'mino'), per_ray=())
    cr, _ = solver.crossings_device(0.5, R_O, 1.0, al, be, geo['r'], geo['th'], geo['mino'], 0.4, model='mono')
    got = torch.ops.kgeo.jet_stokes(al, be, cr['r'], cr['th'], cr['signpr'], cr['signpth'], cr['neq'], 0.5, R_O, 1.0,
                                    1, 'mono', 0.0, 0.0, 2.0, 1.0)
    ref = off_eq.stokes_device(0.5, R_O, 1.0, al, be, cr, neqmax=1, model='mono')
    for x, k in zip(got, ('I', 'Q', 'U', 'evpa')):
        assert torch.equal(x, ref[k])


def test_ops_raise_reference_errors():
    import torch
    from kgeo_gb300 import ops  # noqa: F401
    al, be = pixels(4)
    with pytest.raises(Exception, match=r"\|a\| should be a float in range \[0,1\)"):
        torch.ops.kgeo.raytrace(al, be, 1.2, R_O, TH_O, 5, 1 - 1e-10)
    with pytest.raises(Exception, match="th_o should be a float"):
        torch.ops.kgeo.r_equatorial(al, be, A, R_O, np.pi / 2, 0, 1)
    with pytest.raises(Exception, match="alpha, beta are different lengths!"):
        torch.ops.kgeo.raytrace(al, be[:3], A, R_O, TH_O, 5, 1 - 1e-10)


def test_opcheck_schema_and_fake():
    import torch
    from kgeo_gb300 import ops  # noqa: F401
    al, be = pixels(8)
    utils = ('test_schema', 'test_faketensor')
    torch.library.opcheck(torch.ops.kgeo.raytrace.default, (al, be, A, R_O, TH_O, 12, 1 - 1e-10), test_utils=utils)
    torch.library.opcheck(torch.ops.kgeo.r_equatorial.default, (al, be, A, R_O, TH_O, 0, 2), test_utils=utils)
