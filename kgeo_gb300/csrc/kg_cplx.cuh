// Complex arithmetic with numpy's rounding and signed-zero conventions.
//
// The radial-root classification of the reference (kgeo/kerr_raytracing_utils.py:345-378)
// is decided by exact tests `imag(r) != 0` on numpy complex128 results, and the signs of
// the imaginary parts feed the region-IV constants. These helpers reproduce numpy's
// operation sequence: real operands are promoted to (x, +0); products use
// (ar*br - ai*bi, ar*bi + ai*br); quotients use Smith's method with the scaled
// reciprocal that numpy's complex `divide` loop uses; square roots follow C99 csqrt's
// branch and signed-zero rules. This translation unit is compiled without FMA
// contraction so each product and sum is rounded once, as in numpy.
#pragma once

#include "kg_common.cuh"

namespace kg {

struct cplx {
  double re, im;
};

KG_HD cplx cx(double re, double im) { return cplx{re, im}; }
KG_HD cplx cx_real(double x) { return cplx{x, 0.0}; }

KG_HD cplx operator+(cplx a, cplx b) { return cplx{a.re + b.re, a.im + b.im}; }
KG_HD cplx operator-(cplx a, cplx b) { return cplx{a.re - b.re, a.im - b.im}; }
KG_HD cplx operator-(cplx a) { return cplx{-a.re, -a.im}; }

KG_HD cplx operator*(cplx a, cplx b) {
  return cplx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// numpy complex division (Smith's method, scaled reciprocal).
KG_HD cplx operator/(cplx a, cplx b) {
  double abr = fabs(b.re), abi = fabs(b.im);
  if (abr >= abi) {
    if (abr == 0.0 && abi == 0.0) return cplx{a.re / abr, a.im / abr};
    double rat = b.im / b.re;
    double scl = 1.0 / (b.re + b.im * rat);
    return cplx{(a.re + a.im * rat) * scl, (a.im - a.re * rat) * scl};
  }
  double rat = b.re / b.im;
  double scl = 1.0 / (b.im + b.re * rat);
  return cplx{(a.re * rat + a.im) * scl, (a.im * rat - a.re) * scl};
}

// C99 csqrt semantics: principal branch, sign of the imaginary part follows im
// (including signed zeros); exact for inputs on the real axis.
KG_HD cplx csqrt(cplx z) {
  double x = z.re, y = z.im;
  if (y == 0.0) {
    if (x < 0.0) return cplx{0.0, copysign(sqrt(-x), y)};
    return cplx{sqrt(x), y};
  }
  if (x == 0.0) {
    double r = sqrt(0.5 * fabs(y));
    return cplx{r, copysign(r, y)};
  }
  double d = hypot(x, y);
  if (x > 0.0) {
    double r = sqrt(0.5 * d + 0.5 * x);
    return cplx{r, 0.5 * (y / r)};
  }
  double s = sqrt(0.5 * d - 0.5 * x);
  return cplx{fabs(0.5 * (y / s)), copysign(s, y)};
}

KG_HD double cabs(cplx z) { return hypot(z.re, z.im); }

// Cube root with the largest real part; real inputs keep their sign
// (kgeo/kerr_raytracing_utils.py:828-855).
KG_HD cplx cbrt_max_real(cplx x) {
  double r = cabs(x);
  if (x.im == 0.0) {
    // numpy 2: sign(z) = z / |z| (here +-1 or 0 on the real axis), times cbrt(|z|)
    double s = (r == 0.0) ? 0.0 : x.re / r;
    double c = cbrt(r);
    return cplx{s * c, 0.0 * c + 0.0};
  }
  double th = atan2(x.im, x.re);
  double c = cbrt(r);
  const double third = 1.0 / 3.0;
  // 1j*th/3. : complex division by (3+0j) multiplies by the rounded reciprocal
  double a0 = th * third;
  // 2j*np.pi/3. is a Python complex constant: 2*pi/3 correctly rounded
  const double two_pi_3 = (2.0 * PI) / 3.0;
  double a1 = a0 + two_pi_3;
  double a2 = a0 - two_pi_3;
  double s0, c0, s1, c1, s2, c2;
  s0 = sin(a0); c0 = cos(a0);
  s1 = sin(a1); c1 = cos(a1);
  s2 = sin(a2); c2 = cos(a2);
  cplx z0{c * c0, c * s0}, z1{c * c1, c * s1}, z2{c * c2, c * s2};
  if (z0.re > z1.re && z0.re > z2.re) return z0;
  if (z1.re > z0.re && z1.re > z2.re) return z1;
  if (z2.re > z0.re && z2.re > z1.re) return z2;
  return cplx{kg_nan(), kg_nan()};  // exact ties leave the reference's output undefined
}

}  // namespace kg
