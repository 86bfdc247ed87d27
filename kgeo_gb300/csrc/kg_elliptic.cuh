// Elliptic integrals and Jacobi elliptic functions, FP64.
//
// Written from the published algorithms:
//  * Carlson symmetric integrals R_F, R_J (and R_D = R_J(x,y,z,z)) by duplication with
//    the fifth-order Taylor tail, B. C. Carlson, "Numerical computation of real or
//    complex elliptic integrals", Numer. Algorithms 10 (1995) 13-26; DLMF 19.36(i).
//  * R_C from its closed forms, DLMF 19.2.17-19.2.20.
//  * Jacobi sn, cn, dn by the descending Landen (Gauss) transformation,
//    DLMF 22.7.1-22.7.3, with the small-parameter expansion DLMF 22.10.4-22.10.6.
//  * Incomplete F, E, Pi from R_F/R_D/R_J, DLMF 19.25.5, 19.25.7, 19.25.14, with
//    the periodic continuation of the amplitude (DLMF 19.2.10 for F and E; the same
//    half-period shift for Pi).
//
// The shared-duplication form `rj_multi` evaluates R_F(x,y,z) and R_J(x,y,z,p_i) for
// several p_i at once: the x, y, z duplication sequence and its lambda_m are common to
// all of them, only the p-dependent terms differ.
#pragma once

#include "kg_common.cuh"

namespace kg {

// (3 r)^(-1/6) and (r/4)^(-1/6) for r = 1e-16 (Carlson 1995, eqs. 2.2 and 2.16).
constexpr double RF_Q = 386.0;
constexpr double RJ_Q = 585.0;
constexpr int CARLSON_MAX_IT = KG_CARLSON_MAX_IT;  // hard cap; convergence takes 4-12 steps in FP64

// R_C(1, 1 + e) for e > -1 (DLMF 19.2.18-19 in well-conditioned arctan / log form,
// and the series sum_k (-e)^k / (2k + 1) near e = 0).
KG_HD double rc_one(double e) {
  if (fabs(e) < 2.0e-3) {
    return 1.0 + e * (-1.0 / 3.0 + e * (1.0 / 5.0 + e * (-1.0 / 7.0 + e * (1.0 / 9.0 + e * (-1.0 / 11.0 + e * (1.0 / 13.0))))));
  }
  if (e > 0.0) {
    double s = sqrt(e);
    return atan(s) / s;
  }
  double s = sqrt(-e);
  return (log1p(s) - 0.5 * log1p(e)) / s;
}

// General R_C(x, y), x >= 0, y != 0 (Cauchy principal value for y < 0), DLMF 19.2.17-20.
// The principal value is R_C(x, y) = sqrt(x / (x - y)) R_C(x - y, -y) (DLMF 19.2.20), written
// without a recursive call so that every kernel's stack is known at compile time.
KG_HD double carlson_rc(double x, double y) {
  double scale = 1.0;
  if (y < 0.0) {
    scale = sqrt(x / (x - y));
    const double x1 = x - y;
    y = -y;
    x = x1;
  }
  double d = y - x;
  if (fabs(d) < 2.0e-3 * x) return scale * (rc_one(d / x) / sqrt(x));
  if (d > 0.0) {
    if (x == 0.0) return scale * (HALFPI / sqrt(y));
    return scale * (atan(sqrt(d / x)) / sqrt(d));
  }
  double xd = -d;
  return scale * (log((sqrt(x) + sqrt(xd)) / sqrt(y)) / sqrt(xd));
}

KG_HD double carlson_rf(double x, double y, double z) {
  const double x0 = x, y0 = y;
  const double A0 = (x + y + z) / 3.0;
  const double Q = RF_Q * fmax(fmax(fabs(A0 - x), fabs(A0 - y)), fabs(A0 - z));
  double A = A0, f = 1.0;
  int it = 0;
  for (; it < CARLSON_MAX_IT && f * Q >= fabs(A); ++it) {
    double sx = sqrt(x), sy = sqrt(y), sz = sqrt(z);
    double lam = sx * sy + sx * sz + sy * sz;
    x = 0.25 * (x + lam);
    y = 0.25 * (y + lam);
    z = 0.25 * (z + lam);
    A = 0.25 * (A + lam);
    f *= 0.25;
  }
  if (it == CARLSON_MAX_IT && f * Q >= fabs(A)) note_loop_cap();
  double X = (A0 - x0) * f / A;
  double Y = (A0 - y0) * f / A;
  double Z = -(X + Y);
  double E2 = X * Y - Z * Z;
  double E3 = X * Y * Z;
  return (1.0 - E2 / 10.0 + E3 / 14.0 + E2 * E2 / 24.0 - 3.0 * E2 * E3 / 44.0) / sqrt(A);
}

// R_F(x,y,z) and R_J(x,y,z,p[i]) for NP values p[i] > 0, sharing the x,y,z duplication.
template <int NP>
KG_HD void rj_multi(double x, double y, double z, const double* p_in, double* rj, double* rf) {
  const double x0 = x, y0 = y, z0 = z;
  const double Af0 = (x + y + z) / 3.0;
  const double Qf = RF_Q * fmax(fmax(fabs(Af0 - x), fabs(Af0 - y)), fabs(Af0 - z));
  double Af = Af0;
  double p[NP], A0[NP], A[NP], Q[NP], delta[NP], sum[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    p[i] = p_in[i];
    A0[i] = (x + y + z + 2.0 * p[i]) / 5.0;
    A[i] = A0[i];
    delta[i] = (p[i] - x) * (p[i] - y) * (p[i] - z);
    sum[i] = 0.0;
    Q[i] = RJ_Q * fmax(fmax(fabs(A0[i] - x), fabs(A0[i] - y)), fmax(fabs(A0[i] - z), fabs(A0[i] - p[i])));
  }
  double f = 1.0;   // 4^-m
  double f3 = 1.0;  // 4^-3m
  for (int it = 0;; ++it) {
    // Carlson's stopping rule 4^-m Q < |A_m|, required of every integral in the set (written
    // as "not >=" so that NaN arguments stop at once: their result is NaN, not a capped loop)
    bool done = !(f * Qf >= fabs(Af));
#pragma unroll
    for (int i = 0; i < NP; ++i) done = done && !(f * Q[i] >= fabs(A[i]));
    if (done) break;
    if (it == CARLSON_MAX_IT) {
      note_loop_cap();
      break;
    }
    double sx = sqrt(x), sy = sqrt(y), sz = sqrt(z);
    double lam = sx * sy + sx * sz + sy * sz;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      double sp = sqrt(p[i]);
      double d = (sp + sx) * (sp + sy) * (sp + sz);
      double e = f3 * delta[i] / (d * d);
      double term;
      if (fabs(e) < 2.0e-3) {
        term = rc_one(e) / d;  // R_C(1, 1 + e_m) / d_m, series
      } else {
        // the same term as R_C(alpha_m, beta_m) / 2 (Carlson's earlier form), which keeps
        // full precision when 1 + e_m is small (p much smaller than x, y, z)
        double al = p[i] * (sx + sy + sz) + sx * sy * sz;
        double pl = p[i] + lam;
        term = 0.5 * carlson_rc(al * al, p[i] * pl * pl);
      }
      sum[i] += f * term;
      p[i] = 0.25 * (p[i] + lam);
      A[i] = 0.25 * (A[i] + lam);
    }
    x = 0.25 * (x + lam);
    y = 0.25 * (y + lam);
    z = 0.25 * (z + lam);
    Af = 0.25 * (Af + lam);
    f *= 0.25;
    f3 *= 0.015625;
  }
  {
    double X = (Af0 - x0) * f / Af;
    double Y = (Af0 - y0) * f / Af;
    double Z = -(X + Y);
    double E2 = X * Y - Z * Z;
    double E3 = X * Y * Z;
    *rf = (1.0 - E2 / 10.0 + E3 / 14.0 + E2 * E2 / 24.0 - 3.0 * E2 * E3 / 44.0) / sqrt(Af);
  }
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double inv = f / A[i];
    double X = (A0[i] - x0) * inv;
    double Y = (A0[i] - y0) * inv;
    double Z = (A0[i] - z0) * inv;
    double P = -0.5 * (X + Y + Z);
    double XYZ = X * Y * Z;
    double P2 = P * P;
    double E2 = X * Y + X * Z + Y * Z - 3.0 * P2;
    double E3 = XYZ + 2.0 * E2 * P + 4.0 * P2 * P;
    double E4 = (2.0 * XYZ + E2 * P + 3.0 * P2 * P) * P;
    double E5 = XYZ * P2;
    double tail = 1.0 - 3.0 * E2 / 14.0 + E3 / 6.0 + 9.0 * E2 * E2 / 88.0 - 3.0 * E4 / 22.0
                  - 9.0 * E2 * E3 / 52.0 + 3.0 * E5 / 26.0;
    rj[i] = f * tail / (A[i] * sqrt(A[i])) + 6.0 * sum[i];
  }
}

KG_HD double carlson_rj(double x, double y, double z, double p) {
  double rj, rf;
  rj_multi<1>(x, y, z, &p, &rj, &rf);
  return rj;
}

KG_HD double carlson_rd(double x, double y, double z) { return carlson_rj(x, y, z, z); }

// R_J(x,y,z,rho) for any rho != 0, as the reference's Pi adapter evaluates it:
// directly for rho > 0, through DLMF 19.20.14 for rho < 0
// (kgeo/scipy_ellip_binding.py:207-230). rf must be R_F(x,y,z).
KG_HD double rj_any(double x, double y, double z, double rho, double rf) {
  if (rho > 0.0) return carlson_rj(x, y, z, rho);
  double q = -rho;
  double p = (z * (x + y + q) - x * y) / (z + q);
  double rj0 = carlson_rj(x, y, z, p);
  double rc = carlson_rc(x * y + p * q, p * q);
  return ((p - z) * rj0 - 3.0 * rf + 3.0 * sqrt((x * y * z) / (x * y + p * q)) * rc) / (q + z);
}

// ---------------------------------------------------------------------------
// Complete integrals
// ---------------------------------------------------------------------------

KG_HD double ellip_k(double m) { return carlson_rf(0.0, 1.0 - m, 1.0); }

KG_HD double ellip_e(double m) {
  return carlson_rf(0.0, 1.0 - m, 1.0) - (m / 3.0) * carlson_rd(0.0, 1.0 - m, 1.0);
}

// ---------------------------------------------------------------------------
// Incomplete integrals at an arbitrary real amplitude phi.
// Reduction phi = n*pi + phi0, |phi0| <= pi/2 (ties to even).
// ---------------------------------------------------------------------------

KG_HD double ellip_f(double phi, double m) {
  double n = rint(phi / PI);
  double p0 = phi - n * PI;
  double s = sin(p0), c = cos(p0);
  double inc = s * carlson_rf(c * c, 1.0 - m * s * s, 1.0);
  return n == 0.0 ? inc : inc + 2.0 * n * ellip_k(m);
}

KG_HD double ellip_e_inc(double phi, double m) {
  double n = rint(phi / PI);
  double p0 = phi - n * PI;
  double s = sin(p0), c = cos(p0);
  double x = c * c, y = 1.0 - m * s * s;
  double inc = s * carlson_rf(x, y, 1.0) - (m / 3.0) * s * s * s * carlson_rd(x, y, 1.0);
  return n == 0.0 ? inc : inc + 2.0 * n * ellip_e(m);
}

// Pi(n; phi | m) for |phi| <= pi/2 from R_F and R_J (with the rho < 0 transform).
KG_HD double ellip_pi_core(double n, double phi, double m) {
  double s = sin(phi), c = cos(phi);
  double x = c * c, y = 1.0 - m * s * s, rho = 1.0 - n * s * s;
  double rf = carlson_rf(x, y, 1.0);
  double rj = rj_any(x, y, 1.0, rho, rf);
  return s * rf + (n / 3.0) * (s * s * s) * rj;
}

// Pi(n; phi | m) with the special-case rules of kgeo/scipy_ellip_binding.py:87-237,
// for any real phi.
KG_HD double ellip_pi_ref(double n, double phi, double m) {
  double s = sin(phi);
  double y = 1.0 - m * s * s;
  double rho = 1.0 - n * s * s;
  double aphi = fabs(phi);
  if (aphi <= PHI_ZERO) return phi;
  if (m < M_NEG_INF) return 0.0;
  if (y < 0.0) return kg_nan();
  if (aphi > HALFPI && m >= 1.0) return kg_nan();
  if (aphi > HALFPI && n == 1.0) return kg_inf();
  if (rho == 0.0) return kg_inf();
  if (std::isinf(n)) return 0.0;
  if (aphi > HALFPI) {
    // reference: k = sign*floor(|phi|/pi), then pi/2 < |phi2| <= pi folds once more;
    // both reduce to 2 n Pi(n|m) + Pi(phi0) with phi = n pi + phi0.
    double nr = rint(phi / PI);
    double p0 = phi - nr * PI;
    double comp = ellip_pi_core(n, HALFPI, m);
    double inc = fabs(p0) <= PHI_ZERO ? p0 : ellip_pi_core(n, p0, m);
    return 2.0 * nr * comp + inc;
  }
  return ellip_pi_core(n, phi, m);
}

// ---------------------------------------------------------------------------
// Jacobi elliptic functions
// ---------------------------------------------------------------------------

constexpr int LANDEN_MAX = KG_LANDEN_MAX;

struct Jacobi {
  double sn, cn, dn;
};

// sn, cn, dn(u | m) for 0 <= m < 1 and |u| <= K(m) (any real u works; accuracy is best
// on the reduced range). Descending Landen transformation, DLMF 22.7.1-3.
KG_HD Jacobi jacobi_landen(double u, double m) {
  double k1s[LANDEN_MAX], c1s[LANDEN_MAX];
  int nl = 0;
  double mm = m;
  double w = u;
  // descend until the parameter is small enough for the first-order expansion
  while (mm > 1.0e-9 && nl < LANDEN_MAX) {
    double kp = sqrt(1.0 - mm);
    double k1 = (1.0 - kp) / (1.0 + kp);
    k1s[nl] = k1;
    c1s[nl] = 2.0 * kp / (1.0 + kp);  // 1 - k1 without cancellation
    ++nl;
    w = w / (1.0 + k1);
    mm = k1 * k1;
  }
  if (mm > 1.0e-9) note_loop_cap();
  // DLMF 22.10.4-6 to first order in m
  double s = sin(w), c = cos(w);
  double t = 0.25 * mm * (w - s * c);
  double sn = s - t * c;
  double cn = c + t * s;
  double dn = 1.0 - 0.5 * mm * s * s;
  for (int i = nl - 1; i >= 0; --i) {
    double k1 = k1s[i];
    double den = 1.0 + k1 * sn * sn;
    double sn_u = (1.0 + k1) * sn / den;
    double cn_u = cn * dn / den;
    double dn_u = (c1s[i] + k1 * (cn * cn)) / den;  // (1 - k1 sn^2) / (1 + k1 sn^2)
    sn = sn_u;
    cn = cn_u;
    dn = dn_u;
  }
  return Jacobi{sn, cn, dn};
}

// Reduce u = 2 n K + v with |v| <= K; returns n (as a double) and v.
KG_HD double reduce_half_period(double u, double K2, double* v) {
  double n = rint(u / K2);
  *v = u - n * K2;
  return n;
}

}  // namespace kg
