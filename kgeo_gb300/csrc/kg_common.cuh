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

// ---- iteration caps ---------------------------------------------------------
// Every iterative loop of the elliptic arithmetic stops at a hard cap (Carlson duplication
// KG_CARLSON_MAX_IT steps, descending Landen KG_LANDEN_MAX levels; both are far above what
// FP64 convergence takes, 4-12 steps and 3-6 levels). A loop that reaches its cap without
// meeting its convergence test calls note_loop_cap(). On the device the tracer's kernels keep
// one shared word per block (loop_cap_begin at block start, loop_cap_end OR-s it into the
// launch's flags word as FLAG_LOOP_CAP); kernels that do not collect it leave the word
// unread. The host build keeps one process-wide word (host_loop_cap()).
#ifndef KG_CARLSON_MAX_IT
#define KG_CARLSON_MAX_IT 40
#endif
#ifndef KG_LANDEN_MAX
#define KG_LANDEN_MAX 12
#endif

constexpr unsigned FLAG_LOOP_CAP = 16u;

#if defined(__CUDACC__)
static __shared__ unsigned kg_loop_cap_word;
#endif

inline unsigned& host_loop_cap() {
  static unsigned word = 0;
  return word;
}

KG_HD void note_loop_cap() {
#if defined(__CUDA_ARCH__)
  atomicOr_block(&kg_loop_cap_word, FLAG_LOOP_CAP);
#else
  host_loop_cap() |= FLAG_LOOP_CAP;
#endif
}

#if defined(__CUDACC__)
// Clear the block's word; every thread of the block must call it (it synchronises).
__device__ __forceinline__ void loop_cap_begin() {
  if (threadIdx.x == 0) kg_loop_cap_word = 0u;
  __syncthreads();
}

// OR the block's word into *flags; every thread of the block must call it (it synchronises).
__device__ __forceinline__ void loop_cap_end(uint32_t* flags) {
  __syncthreads();
  if (threadIdx.x == 0 && kg_loop_cap_word && flags) atomicOr(flags, kg_loop_cap_word);
}
#endif

}  // namespace kg
