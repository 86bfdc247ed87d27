// FP32 pieces of the mixed-precision recurrence (kg_mixed2.cuh): the Pi increment of one step
// in FP32 (used where the float-float series form does not apply) and the pole distances
// within which the recurrence keeps FP64.
#pragma once

#include "kg_elliptic_f32.cuh"
#include "kg_ray.cuh"

namespace kg {

KG_HD float rcp_rn_f(float x) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}

// Pi increment of one step in FP32 (see pi_add_term for the formula); X is formed in
// float-float by the caller (it cancels near a pole) and handed over rounded.
KG_HD float pi_add_term_f(float n, float c, float X, float S3) {
  float iX = rcp_rn_f(X);
  float t = S3 * iX;
  float z2 = c * (t * t);
  if (X > 0.0f && fabsf(z2) < 2.0e-2f) return n * t * rc_one_f(-z2);
  if (c > 0.0f) {
    float sc = sqrtf(c);
    float q = sc * S3;
    return n / (2.0f * sc) * logf(fabsf((X + q) / (X - q)));
  }
  if (c < 0.0f) {
    float sc = sqrtf(-c);
    return n / sc * atan2f(sc * S3, X);
  }
  return n * t;
}

// Below this distance rho = |1 - n sn^2| to a Pi pole a characteristic's increment, where the
// float-float R_C series does not apply, is kept in FP64 (the FP32 atan2 / log form would lose
// ~eps32 / rho). The R1 / S1 log terms have their own, narrower zone (MIXED_LOG_RHO).
constexpr double MIXED_RHO = 0.1;

template <class FV>
KG_HD bool theta_near_pole(const FV& f, double sn) {
  return near_pi_pole(f[T_N], sn);
}

template <class FV>
KG_HD bool radial_near_pole(const FV& f, double sn) {
  return near_pi_pole(f[R_N0], sn) || near_pi_pole(f[R_N1], sn) || near_pi_pole(f[R_N2], sn);
}

}  // namespace kg
