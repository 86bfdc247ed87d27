"""Drop-in for kgeo.kerr_raytracing_utils: the Geodesics container, its HDF5 save / load,
the constants and the per-pixel crossing counts.

kgeo/kerr_raytracing_utils.py:9-240 and :551-826. The per-pixel helpers of that module
(radial roots, Mino totals) run on the GPU inside the tracing kernels; the crossing counts
(n_equatorial_crossings, n_poloidal_orbits, n_angular_turnings, is_outside_crit) evaluate on
the GPU through the C ABI. savegeos / loadgeos keep the reference's HDF5 layout and need h5py.
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

    def savegeos(self, outfile=None, path='./'):
        """HDF5 file with the reference's datasets (kgeo/kerr_raytracing_utils.py:201-222):
        spin, inc, r_o, alpha, beta, t, r, theta, phi, affine, mino."""
        import h5py
        if outfile is None:
            fname = path + 'a%0.2f_th%0.2f_geo.h5' % (self.a, self.th_o * 180 / np.pi)
        else:
            fname = outfile

        def host(x):
            return x.detach().cpu().numpy() if hasattr(x, 'detach') else x
        with h5py.File(fname, 'w') as hf:
            hf.create_dataset('spin', data=self.a)
            hf.create_dataset('inc', data=self.th_o)
            hf.create_dataset('r_o', data=self.r_o)
            hf.create_dataset('alpha', data=host(self.alpha))
            hf.create_dataset('beta', data=host(self.beta))
            hf.create_dataset('t', data=host(self.t_s))
            hf.create_dataset('r', data=host(self.r_s))
            hf.create_dataset('theta', data=host(self.th_s))
            hf.create_dataset('phi', data=host(self.ph_s))
            hf.create_dataset('affine', data=host(self.sig_s))
            hf.create_dataset('mino', data=host(self.tausteps))


def loadgeos(infile):
    """Geodesics from a savegeos file (kgeo/kerr_raytracing_utils.py:224-240)."""
    import h5py
    with h5py.File(infile, 'r') as hf:
        a = hf['spin'][()]
        r_o = hf['r_o'][()]
        th_o = hf['inc'][()]
        alpha = hf['alpha'][()]
        beta = hf['beta'][()]
        mino_times = hf['mino'][()]
        affine_times = hf['affine'][()]
        t_s = hf['t'][()]
        r_s = hf['r'][()]
        th_s = hf['theta'][()]
        ph_s = hf['phi'][()]
    return Geodesics(a, [0, r_o, th_o, 0], [alpha, beta], mino_times, affine_times, [t_s, r_s, th_s, ph_s])


def n_equatorial_crossings(a, th_o, alpha, beta, tau):
    """kgeo/kerr_raytracing_utils.py:605-684 (GPU)."""
    from .equatorial_lensing import n_equatorial_crossings as f
    return f(a, th_o, alpha, beta, tau)


def n_poloidal_orbits(a, th_o, alpha, beta, tau):
    """kgeo/kerr_raytracing_utils.py:551-603 (GPU)."""
    from .equatorial_lensing import n_poloidal_orbits as f
    return f(a, th_o, alpha, beta, tau)


def n_angular_turnings(a, th_o, alpha, beta, tau):
    """kgeo/kerr_raytracing_utils.py:686-792 (GPU)."""
    from .equatorial_lensing import n_angular_turnings as f
    return f(a, th_o, alpha, beta, tau)


def is_outside_crit(a, th_o, alpha, beta):
    """kgeo/kerr_raytracing_utils.py:794-826 (GPU)."""
    from .equatorial_lensing import is_outside_crit as f
    return f(a, th_o, alpha, beta)
