"""The kgeo torch operators are registered and their fake implementations give the CUDA
kernels' output shapes (meta tensors, FakeTensorMode); no compute."""
import pytest
import torch

from kgeo_gb300 import ops  # noqa: F401

F64 = torch.float64


def meta(*shape):
    return torch.empty(*shape, device='meta', dtype=F64)


def test_ops_registered():
    for name in ('raytrace', 'coords_at_tau', 'r_equatorial', 'image', 'image_adjoint', 'jet_stokes'):
        assert hasattr(torch.ops.kgeo, name), name


def test_fake_shapes():
    out = torch.ops.kgeo.raytrace(meta(10), meta(10), 0.5, 1e4, 0.3, 7, 1 - 1e-10)
    assert [tuple(x.shape) for x in out] == [(7, 10)] * 6
    out = torch.ops.kgeo.coords_at_tau(meta(10), meta(10), meta(3, 10), 0.5, 1e4, 0.3, True)
    assert [tuple(x.shape) for x in out] == [(3, 10)] * 5
    out = torch.ops.kgeo.r_equatorial(meta(10), meta(10), 0.5, 1e4, 0.3, 0, 3)
    assert [tuple(x.shape) for x in out] == [(3, 10), (3, 10), (10,), (10,)]
    assert tuple(torch.ops.kgeo.image(meta(7), meta(10), meta(10), 1e4, 2).shape) == (10, 3)
    assert tuple(torch.ops.kgeo.image_adjoint(meta(10, 3), meta(7), meta(10), meta(10)).shape) == (7,)
    out = torch.ops.kgeo.jet_stokes(meta(10), meta(10), *[meta(2, 10)] * 5, 0.5, 1e4, 0.3, 2)
    assert [tuple(x.shape) for x in out] == [(3, 10)] * 4


def test_fake_tensor_mode():
    from torch._subclasses.fake_tensor import FakeTensorMode
    with FakeTensorMode():
        a = torch.empty(12, dtype=F64)
        out = torch.ops.kgeo.raytrace(a, a, 0.5, 1e4, 0.3, 5)
        assert [tuple(x.shape) for x in out] == [(5, 12)] * 6


def test_cuda_required_on_real_tensors():
    """On real CPU tensors the operators do not fall back to a CPU path."""
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    a = torch.zeros(4, dtype=F64)
    with pytest.raises(RuntimeError):
        torch.ops.kgeo.raytrace(a, a, 0.5, 1e4, 0.3, 5)
