"""Drop-in for kgeo.kerr_raytracing_utils: the Geodesics container and the constants.

kgeo/kerr_raytracing_utils.py:9-93. The per-pixel helpers of that module
(radial roots, Mino totals, crossing counts) run on the GPU inside the tracing
kernels; nmax_eq / n_poloidal evaluate on the GPU through the C ABI.
"""
import numpy as np

MINSPIN = 1.e-4   # kgeo/kerr_raytracing_utils.py:9
EP = 1.e-12       # kgeo/kerr_raytracing_utils.py:12


class Geodesics(object):
    """Result of raytrace_ana (kgeo/kerr_raytracing_utils.py:15-93).

    mino_times, affine_times and the entries of geo_coords = [t, r, th, ph] are
    (ngeo, npix) arrays: numpy float64 by default, or CUDA tensors when the trace
    was run with device_arrays=True.
    """

    def __init__(self, a, observer_coords, image_coords, mino_times, affine_times, geo_coords):
        self.a = a
        self.observer_coords = observer_coords
        self.image_coords = image_coords
        self.mino_times = mino_times
        self.affine_times = affine_times
        self.geo_coords = geo_coords

    # observer
    @property
    def t_o(self):
        return self.observer_coords[0]

    @property
    def r_o(self):
        return self.observer_coords[1]

    @property
    def th_o(self):
        return self.observer_coords[2]

    @property
    def ph_o(self):
        return self.observer_coords[3]

    # image
    @property
    def alpha(self):
        return self.image_coords[0]

    @property
    def beta(self):
        return self.image_coords[1]

    @property
    def npix(self):
        return len(self.alpha)

    @property
    def lam(self):
        return -self.alpha * np.sin(self.th_o)

    @property
    def eta(self):
        return (self.alpha ** 2 - self.a ** 2) * np.cos(self.th_o) ** 2 + self.beta ** 2

    @property
    def n_poloidal(self):
        from .equatorial_lensing import n_poloidal_orbits
        return n_poloidal_orbits(self.a, self.th_o, self.alpha, self.beta, self.tausteps)

    @property
    def nmax_eq(self):
        from .equatorial_lensing import n_equatorial_crossings
        return n_equatorial_crossings(self.a, self.th_o, self.alpha, self.beta, self.tautot)

    # geodesics
    @property
    def tausteps(self):
        return self.mino_times

    @property
    def tautot(self):
        return self.mino_times[-1]

    @property
    def affinesteps(self):
        return self.affine_times

    @property
    def t_s(self):
        return self.geo_coords[0]

    @property
    def r_s(self):
        return self.geo_coords[1]

    @property
    def th_s(self):
        return self.geo_coords[2]

    @property
    def ph_s(self):
        return self.geo_coords[3]

    @property
    def sig_s(self):
        return self.affine_times
