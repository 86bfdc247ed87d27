// Float-float ("double-single") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi) / 2), about 48 significant bits carried entirely on the FP32
// pipe. GB300 issues FP32 at 64x its FP64 rate, so a float-float operation (3-11 FP32
// instructions) costs a fraction of one FP64 instruction. Error-free transformations:
// two-sum (Knuth) and two-product by fused multiply-add (Dekker / Ogita-Rump-Oishi).
//
// Device code uses the _rn intrinsics for every add / multiply whose rounding the algorithms
// rely on, so the compiler can neither contract nor reassociate them.
#pragma once

#include "kg_common.cuh"

namespace kg {

#if defined(__CUDA_ARCH__)
KG_HD float f_add(float a, float b) { return __fadd_rn(a, b); }
KG_HD float f_sub(float a, float b) { return __fsub_rn(a, b); }
KG_HD float f_mul(float a, float b) { return __fmul_rn(a, b); }
KG_HD float f_rcp(float a) { return __frcp_rn(a); }
#else
KG_HD float f_add(float a, float b) { return a + b; }
KG_HD float f_sub(float a, float b) { return a - b; }
KG_HD float f_mul(float a, float b) { return a * b; }
KG_HD float f_rcp(float a) { return 1.0f / a; }
#endif

struct ff {
  float hi, lo;
};

KG_HD ff ff_c(float x) { return ff{x, 0.0f}; }

// Split of a double (FP64 operations: used for constants and chunk starts only).
KG_HD ff ff_from(double x) {
  const float hi = (float)x;
  return ff{hi, (float)(x - (double)hi)};
}

// float -> double without a conversion instruction for normal floats and zeros: the IEEE
// fields moved by integer operations (exponent rebiased by 1023 - 127, mantissa shifted by
// 52 - 23); denormals, infinities and NaNs take the conversion instruction. GB300 executes
// float / double conversions on its FP64 pipe, at 1/64 of the FP32 rate. Exact either way.
KG_HD double f2d_exact(float x) {
#if defined(__CUDA_ARCH__)
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) {
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)x;
  }
  const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
#else
  return (double)x;
#endif
}

// hi + lo in double: exact (the two FP32 words together carry at most ~49 significant bits).
KG_HD double ff_to_double(ff a) { return f2d_exact(a.hi) + f2d_exact(a.lo); }

// s + e = a + b exactly, |b| <= |a| or a == 0
KG_HD ff quick_two_sum(float a, float b) {
  const float s = f_add(a, b);
  return ff{s, f_sub(b, f_sub(s, a))};
}

KG_HD ff ff_add(ff a, ff b) {
  const float s = f_add(a.hi, b.hi);
  const float bb = f_sub(s, a.hi);
  float e = f_add(f_sub(a.hi, f_sub(s, bb)), f_sub(b.hi, bb));
  e = f_add(e, f_add(a.lo, b.lo));
  return quick_two_sum(s, e);
}

KG_HD ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
KG_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

KG_HD ff ff_add_f(ff a, float b) {
  const float s = f_add(a.hi, b);
  const float bb = f_sub(s, a.hi);
  float e = f_add(f_sub(a.hi, f_sub(s, bb)), f_sub(b, bb));
  e = f_add(e, a.lo);
  return quick_two_sum(s, e);
}

KG_HD ff ff_mul(ff a, ff b) {
  const float p = f_mul(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}

KG_HD ff ff_mul_f(ff a, float b) {
  const float p = f_mul(a.hi, b);
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return quick_two_sum(p, e);
}

KG_HD ff ff_sqr(ff a) {
  const float p = f_mul(a.hi, a.hi);
  float e = fmaf(a.hi, a.hi, -p);
  e = fmaf(f_add(a.hi, a.hi), a.lo, e);
  return quick_two_sum(p, e);
}

// 1 / a: FP32 reciprocal and one Newton step carried in float-float.
KG_HD ff ff_rcp(ff a) {
  const float x = f_rcp(a.hi);
  float d = fmaf(-a.hi, x, 1.0f);  // 1 - a.hi x, exact to FP32 rounding of a ~1e-7 residual
  d = fmaf(-a.lo, x, d);
  return quick_two_sum(x, f_mul(x, d));
}

KG_HD ff ff_div(ff a, ff b) { return ff_mul(a, ff_rcp(b)); }

// 1 - a for a float-float a (the Jacobi denominators).
KG_HD ff ff_one_minus(ff a) { return ff_add_f(ff_neg(a), 1.0f); }

}  // namespace kg
