"""kgeo_gb300: the analytic Kerr null-geodesic tracer of kgeo, GB300-native.

Drop-ins: kgeo_gb300.kerr_raytracing_ana.raytrace_ana / coords_at_tau and the
Geodesics container (kgeo_gb300.kerr_raytracing_utils). The compute path is the
CUDA library libkgeo_gb300.so (C ABI: include/kgeo_gb300.h).
"""
from .kerr_raytracing_utils import Geodesics, MINSPIN, EP  # noqa: F401

__all__ = ['Geodesics', 'MINSPIN', 'EP']
