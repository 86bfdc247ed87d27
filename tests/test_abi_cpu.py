"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports every
function include/kgeo_gb300.h declares (no compute calls: there is no GPU here)."""
import os
import re
import shutil

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, 'include', 'kgeo_gb300.h')


def declared():
    text = open(HEADER).read()
    return re.findall(r'^\w[\w\s\*]*?\b(kgeo_\w+)\s*\(', text, re.M)


@pytest.fixture(scope='module')
def lib():
    from kgeo_gb300 import build, _lib
    if not os.path.exists(build.LIB):
        if not (shutil.which('nvcc') or os.path.exists('/usr/local/cuda/bin/nvcc')):
            pytest.skip('nvcc not available to build the library')
        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared()
    for n in ('kgeo_raytrace', 'kgeo_coords_at_tau', 'kgeo_ray_setup', 'kgeo_ray_samples', 'kgeo_r_equatorial',
              'kgeo_equatorial_crossings', 'kgeo_workspace_size'):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(lib):
    from kgeo_gb300 import _lib
    assert set(declared()) == set(_lib.SIGNATURES)


def test_host_only_calls(lib):
    assert lib.kgeo_abi_version() == 2
    assert lib.kgeo_workspace_size(1000) >= 1000 * 8 * 50
    assert lib.kgeo_status_string(1) == b'|a| should be a float in range [0,1)'
    assert lib.kgeo_status_string(2) == b'r_o should be a float > 100'


def test_argument_errors_return_codes_without_gpu(lib):
    """Argument checks happen on the host before any CUDA call, as the reference raises before computing."""
    import ctypes
    from kgeo_gb300 import _lib
    g = _lib.GeodesicsOut()
    for (a, r_o, th_o), code in [((1.0, 1e4, 0.3), 1), ((-1.5, 1e4, 0.3), 1), ((0.5, 99.0, 0.3), 2),
                                 ((0.5, float('nan'), 0.3), 2), ((0.5, 1e4, 0.0), 3), ((0.5, 1e4, 1.5707963267948966), 3),
                                 ((0.5, 1e4, 3.2), 3)]:
        ob = _lib.Observer(a, r_o, th_o)
        assert lib.kgeo_raytrace(ctypes.byref(ob), None, None, 10, 5, 1.0, ctypes.byref(g), None, 0, None) == code
    ob = _lib.Observer(0.5, 1e4, 0.3)
    assert lib.kgeo_r_equatorial(ctypes.byref(ob), -1, 3, None, None, 10, None, None, None, None, None) == 6
    assert lib.kgeo_raytrace(ctypes.byref(ob), None, None, -1, 5, 1.0, ctypes.byref(g), None, 0, None) == 4
    assert lib.kgeo_raytrace(ctypes.byref(ob), None, None, 10, -5, 1.0, ctypes.byref(g), None, 0, None) == 5
    assert lib.kgeo_raytrace(ctypes.byref(ob), None, None, 10, 5, 1.0, ctypes.byref(g), None, 0, None) == 8


def test_kernel_stacks_within_default_limit(lib):
    """Every kernel's per-thread stack (its whole call chain) stays under CUDA's default
    1024-byte limit with the build's margin; the build refuses a unit otherwise, and this
    re-reads the ptxas report it keeps (kgeo_gb300/_build/ptxas.log)."""
    from kgeo_gb300 import build
    path = os.path.join(build.BUILD, 'ptxas.log')
    if not os.path.exists(path):
        pytest.skip('library built without its ptxas report')
    res = build.check_resources(open(path).read())
    names = ' '.join(res)
    for k in ('stepped_kernel', 'ray_setup_kernel', 'samples_kernel', 'batch_samples_kernel', 'image_kernel'):
        assert k in names
    over = {k: v for k, v in res.items() if v[1] > build.STACK_BUDGET}
    assert not over, over
