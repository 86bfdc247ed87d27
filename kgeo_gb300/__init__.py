"""kgeo_gb300: the analytic Kerr null-geodesic tracer of kgeo and its consumers, GB300-native.

Drop-in modules (same names, signatures and outputs as kgeo's):
  kerr_raytracing_ana   raytrace_ana, coords_at_tau
  kerr_raytracing_utils Geodesics (savegeos / loadgeos), n_equatorial_crossings,
                        n_poloidal_orbits, n_angular_turnings, is_outside_crit
  equatorial_lensing    r_equatorial, nmax_equatorial, nmax_poloidal, rho_of_req,
                        critical_curve, make_curves2, generate_library
  equatorial_images     make_image, Iobs (unpolarised, polarised, with path length)
  emissivities, velocities, bfields   the emission, velocity and B-field models
  solver                jet field-line crossings (getguesses, findroot)
  off_eq                getstokes: Stokes images of the monopole jet field line
The same functions as torch operators on CUDA tensors (torch.ops.kgeo.*, with fake
implementations and the image's autograd): import kgeo_gb300.ops.
Beyond kgeo: image_grad (an adjoint-backed torch.autograd.Function) and batch (many images in
one persistent launch, CUDA graph replay, autotuned shape). The compute path is the CUDA
library libkgeo_gb300.so (C ABI: include/kgeo_gb300.h); there is no CPU path.
"""
from .kerr_raytracing_utils import Geodesics, MINSPIN, EP  # noqa: F401

__all__ = ['Geodesics', 'MINSPIN', 'EP']
