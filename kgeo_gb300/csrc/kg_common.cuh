// Common definitions for the kgeo GB300 kernels.
//
// Every routine here is written once and compiled both for the device (nvcc,
// sm_103a) and, for host-side unit checks of the same arithmetic, by g++.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define KG_HD __host__ __device__ __forceinline__
#else
#define KG_HD inline
#endif

namespace kg {

// Constants of the reference (kgeo/kerr_raytracing_utils.py:9-12, kgeo/scipy_ellip_binding.py:7).
constexpr double MINSPIN = 1.0e-4;
constexpr double EP = 1.0e-12;
constexpr double PI = 3.141592653589793;       // np.pi
constexpr double HALFPI = 1.5707963267948966;  // 0.5 * np.pi
constexpr double PHI_ZERO = 1.0e-10;           // ellip_pi's phi -> 0 cut-off
constexpr double M_NEG_INF = -1.0e14;          // ellip_pi's m -> -inf cut-off

KG_HD double kg_inf() { return __builtin_huge_val(); }
KG_HD double kg_nan() { return __builtin_nan(""); }

KG_HD double sq(double x) { return x * x; }

// 1/x to FP64 working accuracy (not correctly rounded): the hardware reciprocal
// approximation refined by two Newton steps. For the recurrence's normalisations, where the
// last-bit rounding of an IEEE divide carries no meaning; |x| must be a normal number.
KG_HD double rcp_fast(double x) {
#if defined(__CUDA_ARCH__)
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
#else
  return 1.0 / x;
#endif
}

KG_HD float rsqrt_f(float x) {
#if defined(__CUDA_ARCH__)
  return rsqrtf(x);
#else
  return 1.0f / sqrtf(x);
#endif
}

// x**3 as numpy evaluates it (a correctly rounded pow): product of a double-double
// square with x, rounded once.
KG_HD double cube_rn(double x) {
  double hi = x * x;
  double lo = std::fma(x, x, -hi);
  double c = hi * x;
  double ce = std::fma(hi, x, -c);
  return c + (ce + lo * x);
}

// Python / numpy sign conventions.
KG_HD double sign_of(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0); }

}  // namespace kg
