"""Drop-in for kgeo.scipy_ellip_binding (kgeo/scipy_ellip_binding.py): the elliptic
integral of the third kind Pi(n; phi | m) in Abramowitz & Stegun's convention, with the
reference adapter's special cases and periodic continuation, evaluated by the library's
CUDA Carlson arithmetic (kgeo_ellip_pi), the same code the tracer's kernels run."""
import ctypes

import numpy as np
import torch

from . import _lib
from . import device as _dev

FORMS = {'setup': 0, 'samples': 1, 'adapter': 2}


def ellip_pi_arr(n, phi, m, form='samples'):
    """Pi(n; phi | m); kgeo/scipy_ellip_binding.py:87-237.

    Same argument handling as the reference: scalars become 1-element arrays, the three
    inputs must share their last dimension, and 1-d n or m against a 2-d phi are repeated
    along phi's first axis. Returns a numpy float64 array of phi's shape. ``form`` picks which
    compiled copy of the kernels' arithmetic evaluates it: 'setup' (the per-ray setup, FMA
    contraction off), 'samples' (the direct sample evaluators) or 'adapter' (the standalone
    adapter)."""
    if not isinstance(n, np.ndarray):
        n = np.array([n]).flatten()
    if not isinstance(phi, np.ndarray):
        phi = np.array([phi]).flatten()
    if not isinstance(m, np.ndarray):
        m = np.array([m]).flatten()
    if not (n.shape[-1] == phi.shape[-1] == m.shape[-1]):
        raise Exception("inputs to ellip_pi_arr do not have same last dimension!")
    if len(n.shape) != len(phi.shape):
        n = np.outer(np.ones(phi.shape[0]), n)
    if len(m.shape) != len(phi.shape):
        m = np.outer(np.ones(phi.shape[0]), m)
    shape = phi.shape
    n, phi, m = (np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), shape)).ravel()
                 for v in (n, phi, m))
    _dev.require_cuda()
    lib = _lib.load()
    dn, dphi, dm = (_dev.as_device(v) for v in (n, phi, m))
    out = torch.empty(dphi.shape, dtype=torch.float64, device=dphi.device)
    s = torch.cuda.current_stream(dphi.device)
    _lib.check(lib.kgeo_ellip_pi(_dev._ptr(dn), _dev._ptr(dphi), _dev._ptr(dm), dphi.numel(), FORMS[form],
                                 _dev._ptr(out), ctypes.c_void_p(s.cuda_stream)))
    return out.cpu().numpy().reshape(shape)
