"""ctypes binding of libkgeo_gb300.so (the C ABI declared in include/kgeo_gb300.h).

There is no CPU fallback: every call needs the CUDA library and a CUDA device, and
fails loudly without them.
"""
import ctypes
import os

from . import build as _build

c_double = ctypes.c_double
c_int = ctypes.c_int
c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_size_t = ctypes.c_size_t
c_void_p = ctypes.c_void_p


class Observer(ctypes.Structure):
    _fields_ = [('a', c_double), ('r_o', c_double), ('th_o', c_double)]


class GeodesicsOut(ctypes.Structure):
    _fields_ = [('t', c_void_p), ('r', c_void_p), ('th', c_void_p), ('ph', c_void_p), ('sig', c_void_p),
                ('mino', c_void_p), ('tau_tot', c_void_p), ('rclass', c_void_p), ('thclass', c_void_p),
                ('flags', c_void_p)]


class Emission(ctypes.Structure):
    """kgeo_emission."""
    _fields_ = [('emissivity', c_int32), ('velocity', c_int32), ('retrograde', c_int32), ('reserved', c_int32),
                ('emis_p', c_double * 2), ('mu_ring', c_double), ('vel_p', c_double * 3),
                ('emiscut_in', c_double), ('emiscut_out', c_double), ('specind', c_double), ('sinthb', c_double)]


class ImageOut(ctypes.Structure):
    """kgeo_image_out."""
    _fields_ = [('I', c_void_p), ('g', c_void_p), ('r_s', c_void_p), ('Ir', c_void_p), ('sinthb', c_void_p),
                ('imax', c_void_p), ('nmax', c_void_p), ('npol', c_void_p), ('Q', c_void_p), ('U', c_void_p),
                ('lp', c_void_p), ('Ie', c_void_p)]


class BField(ctypes.Structure):
    """kgeo_bfield."""
    _fields_ = [('field', c_int32), ('flag', c_int32), ('c', c_double * 3)]


class ImageOptions(ctypes.Structure):
    """kgeo_image_options."""
    _fields_ = [('polarization', c_int32), ('pathlength', c_int32), ('diskangle', c_double), ('bfield', BField)]


class Curve(ctypes.Structure):
    """kgeo_curve."""
    _fields_ = [('a', c_double), ('th_o', c_double), ('r_eq', c_double), ('rho_min', c_double),
                ('rho_max', c_double), ('mbar', c_int32), ('reserved', c_int32)]


class JetField(ctypes.Structure):
    """kgeo_jet_field."""
    _fields_ = [('model', c_int32), ('reserved', c_int32), ('psitarget', c_double), ('pval', c_double)]


class JetEmission(ctypes.Structure):
    """kgeo_jet_emission."""
    _fields_ = [('model', c_int32), ('neqmax', c_int32), ('pval', c_double), ('nu_parallel', c_double),
                ('sigma', c_double), ('specind', c_double)]


class BatchImage(ctypes.Structure):
    """kgeo_batch_image."""
    _fields_ = [('a', c_double), ('r_o', c_double), ('th_o', c_double), ('npix', c_int64), ('ngeo', c_int32),
                ('reserved', c_int32), ('maxtaufrac', c_double)]


class BatchConfig(ctypes.Structure):
    """kgeo_batch_config."""
    _fields_ = [('block', c_int32), ('ctas_per_sm', c_int32), ('tile', c_int32), ('chunk', c_int32)]


EMIS = {'bpl': 0, 'constant': 1, 'glm': 2, 'ring': 3}
VEL = {'zamo': 0, 'infall': 1, 'kep': 2, 'cunningham': 2, 'subkep': 3, 'cunningham_subkep': 3, 'general': 4}
JET = {'para': 0, 'mono': 1, 'power': 2}
BFIELD = {'simple': 0, 'rad': 0, 'vert': 0, 'tor': 0, 'simple_rm1': 1, 'monopoleA': 2, 'bz_guess': 3,
          'bz_monopole': 4, 'bz_para': 5, 'power': 6, 'gen_power': 7}
N_IMAGE_PARAMS = 7  # a, th_o, emis_p[0..1], vel_p[0..2]

# name -> (restype, argtypes); kept in step with include/kgeo_gb300.h
SIGNATURES = {
    'kgeo_workspace_size': (c_size_t, [c_int64]),
    'kgeo_raytrace': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_int32, c_double,
                              ctypes.POINTER(GeodesicsOut), c_void_p, c_size_t, c_void_p]),
    'kgeo_coords_at_tau': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_void_p, c_int32,
                                   c_int32, ctypes.POINTER(GeodesicsOut), c_void_p, c_size_t, c_void_p]),
    'kgeo_ray_setup': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_int32, c_double, c_void_p,
                               c_size_t, ctypes.POINTER(GeodesicsOut), c_void_p]),
    'kgeo_ray_samples': (c_int, [ctypes.POINTER(Observer), c_void_p, c_size_t, c_int64, c_void_p, c_int32, c_int32,
                                 c_int32, c_int32, ctypes.POINTER(GeodesicsOut), c_void_p]),
    'kgeo_raytrace_host_workspace_size': (c_size_t, [c_int64, c_int32, c_int32]),
    'kgeo_raytrace_host': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_int32, c_double, c_int32,
                                   ctypes.POINTER(GeodesicsOut), c_void_p, c_size_t, c_void_p]),
    'kgeo_raytrace_mixed': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_int32, c_double,
                                    ctypes.POINTER(GeodesicsOut), c_void_p, c_size_t, c_void_p]),
    'kgeo_raytrace_noalloc': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_int32, c_double,
                                      ctypes.POINTER(GeodesicsOut), c_void_p]),
    'kgeo_measure_fp64_peak': (c_int, [ctypes.POINTER(c_double), c_void_p]),
    'kgeo_r_equatorial': (c_int, [ctypes.POINTER(Observer), c_int32, c_int32, c_void_p, c_void_p, c_int64,
                                  c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    'kgeo_equatorial_crossings': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_void_p, c_int32,
                                          c_void_p, c_void_p, c_void_p, c_void_p]),
    'kgeo_image': (c_int, [ctypes.POINTER(Observer), c_int32, c_int32, c_void_p, c_void_p, c_int64,
                           ctypes.POINTER(Emission), ctypes.POINTER(ImageOut), c_void_p]),
    'kgeo_image_ex': (c_int, [ctypes.POINTER(Observer), c_int32, c_int32, c_void_p, c_void_p, c_int64,
                              ctypes.POINTER(Emission), ctypes.POINTER(ImageOptions), ctypes.POINTER(ImageOut),
                              c_void_p]),
    'kgeo_angular_turnings': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_void_p, c_int32,
                                      c_void_p, c_void_p]),
    'kgeo_jet_guesses': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p,
                                 c_int32, ctypes.POINTER(JetField), c_int32, c_void_p, c_void_p, c_void_p, c_int32,
                                 c_void_p]),
    'kgeo_jet_findroot': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_void_p, c_int32,
                                  ctypes.POINTER(JetField), c_double, c_int32, c_void_p, c_size_t, c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    'kgeo_jet_stokes': (c_int, [ctypes.POINTER(Observer), c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_void_p, c_int32, ctypes.POINTER(JetEmission), c_void_p, c_void_p, c_void_p,
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    'kgeo_rho_of_req': (c_int, [ctypes.POINTER(Curve), c_int32, c_void_p, c_int32, c_double, c_double, c_int32,
                                c_void_p, c_void_p, c_void_p]),
    'kgeo_critical_curve': (c_int, [c_double, c_double, c_int64, c_void_p, c_void_p, c_void_p]),
    'kgeo_image_adjoint_workspace_size': (c_size_t, [c_int64]),
    'kgeo_image_adjoint': (c_int, [ctypes.POINTER(Observer), c_int32, c_int32, c_void_p, c_void_p, c_int64,
                                   ctypes.POINTER(Emission), c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'kgeo_batch_create': (c_int, [ctypes.POINTER(BatchImage), c_int32, c_int32, ctypes.POINTER(c_void_p)]),
    'kgeo_batch_destroy': (None, [c_void_p]),
    'kgeo_batch_sizes': (c_int, [c_void_p, ctypes.POINTER(c_int64), ctypes.POINTER(c_int64),
                                 ctypes.POINTER(c_size_t)]),
    'kgeo_batch_bind': (c_int, [c_void_p, c_void_p, c_void_p, ctypes.POINTER(GeodesicsOut), c_void_p, c_size_t]),
    'kgeo_batch_get_config': (c_int, [c_void_p, ctypes.POINTER(BatchConfig), ctypes.POINTER(c_int32)]),
    'kgeo_batch_set_config': (c_int, [c_void_p, ctypes.POINTER(BatchConfig)]),
    'kgeo_batch_autotune': (c_int, [c_void_p, c_int32, c_void_p, ctypes.POINTER(BatchConfig)]),
    'kgeo_batch_run': (c_int, [c_void_p, c_void_p]),
    'kgeo_batch_graph_launch': (c_int, [c_void_p, c_void_p]),
    'kgeo_ellip_pi': (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p]),
    'kgeo_status_string': (ctypes.c_char_p, [c_int]),
    'kgeo_abi_version': (c_int, []),
}

PRECISION_FP64 = 0
PRECISION_MIXED = 1
FLAG_ANY_ETA_POS = 1
FLAG_ANY_ETA_NONPOS = 2
FLAG_ANY_STEP_ZERO = 4
FLAG_MINSPIN_VORTICAL = 8
FLAG_LOOP_CAP = 16

_lib = None


def library_path():
    return _build.LIB


def load():
    """Load libkgeo_gb300.so (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise RuntimeError('kgeo_gb300: CUDA library %s is not built; run python kgeo_gb300/build.py '
                               '(or __graft_entry__.build())' % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def status_string(code):
    return load().kgeo_status_string(code).decode()


class KgeoError(Exception):
    """A non-zero kgeo_status from the C ABI."""

    def __init__(self, code):
        self.code = code
        super().__init__(status_string(code))


def check(code):
    if code != 0:
        raise KgeoError(code)
