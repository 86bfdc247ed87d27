// Per-ray setup and per-sample evaluation of the analytic Kerr null geodesic
// (Gralla & Lupsasca 2019a/b), FP64.
//
// ray_setup() follows kgeo's per-pixel chain: conserved quantities
// (kgeo/kerr_raytracing_ana.py:76-82), u_+/u_- with their clamps
// (kgeo/kerr_raytracing_utils.py:276-328), the radial quartic roots and rclass
// (:330-380), the total Mino time (:382-548) and every ray-constant term of the theta
// (kgeo/kerr_raytracing_ana.py:216-363) and r (:404-624) antiderivatives. It is
// compiled without FMA contraction so that its roundings follow numpy's one-op-at-a-time
// evaluation, which keeps the exact-zero classification tests faithful.
//
// sample_*() evaluate r, theta, G_phi, G_t, I_phi, I_t, I_sigma at one Mino time from
// that record. The elliptic work is reorganised for the GPU: the Jacobi argument is
// reduced by its half period (am(u + 2K) = am(u) + pi) and sn, cn, dn come from one
// Landen evaluation; F, E and every Pi at the same amplitude share one Carlson
// duplication loop (rj_multi), and the periodic parts are ray constants.
#pragma once

#include "kg_common.cuh"
#include "kg_cplx.cuh"
#include "kg_elliptic.cuh"

namespace kg {

// Per-image constants, evaluated once on the host with the host libm (as numpy does).
struct Observer {
  double a, a2;           // spin, a**2
  double r_o;             // observer radius (may be +inf)
  double th_o;            // inclination
  double sin_th, cos_th;  // np.sin(th_o), np.cos(th_o)
  double cos2;            // np.cos(th_o)**2
  double rplus, rminus;   // 1 +- sqrt(1 - a**2)
  int minspin;            // |a| < MINSPIN
  int r_o_inf;            // r_o == inf
};

// Status bits shared by all rays of a launch (atomicOr).
enum : unsigned {
  FLAG_ANY_ETA_POS = 1u,     // some pixel has eta > 0 (ordinary branch runs, eta == 0 joins it)
  FLAG_ANY_ETA_NONPOS = 2u,  // some pixel has eta <= 0
  FLAG_ANY_STEP_ZERO = 4u,   // some pixel has a zero Mino step (numpy linspace's denormal path)
  FLAG_MINSPIN_VORTICAL = 8u // |a| < MINSPIN with eta <= 0: the reference raises
};

// Radial integration case (kgeo/kerr_raytracing_ana.py:404, 473, 554).
enum : int { RCASE_NONE = 0, RCASE_2 = 2, RCASE_3 = 3, RCASE_4 = 4 };
// Theta branch (kgeo/kerr_raytracing_ana.py:216, 298).
enum : int { TH_ZERO = 0, TH_ORD = 1, TH_VORT = 2 };

// Field indices of the per-ray record (structure of arrays: rec[field * npix + ray]).
enum RecField : int {
  F_LAM = 0, F_S, F_TAUMAX, F_TAUTOT,
  // theta
  T_SCALE, T_GTH, T_M, T_S1M, T_K2, T_N, T_KK, T_PIC, T_EC, T_KC, T_PREF, T_GPH, T_GT,
  T_UP, T_UM, T_PREFC, T_H,
  // radial, common
  R_XS, R_IRO, R_M, R_K2, R_KC, R_EC, R_N0, R_N1, R_N2, R_PIC0, R_PIC1, R_PIC2,
  // radial, case-specific
  R_C0, R_C1, R_C2, R_C3, R_C4, R_C5, R_C6, R_C7, R_C8, R_C9, R_C10, R_C11, R_C12, R_C13,
  R_C14, R_C15, R_C16, R_C17, R_C18, R_C19,
  // per-ray factors the sample kernels would otherwise recompute at every sample
  R_C20, R_C21, R_C22, R_C23, R_C24,
  // one step of the even Mino grid: theta Jacobi values / integrals at the step, r ditto
  S_TSN, S_TCN, S_TDN, S_TE, S_TPI, S_TC,
  S_RSN, S_RCN, S_RDN, S_RE, S_RP0, S_RP1, S_RP2, S_RC0, S_RC1, S_RC2,
  // observer constants the gain estimate needs
  G_A, G_RP, G_RM, G_RO,
  // constants of the Pi increments' atan2 / log forms: sqrt|c| and n / (2 sqrt c) (c > 0) or
  // n / sqrt(-c) (c < 0), theta then r
  S_TQ, S_TQN, S_RQ0, S_RQ1, S_RQ2, S_RQN0, S_RQN1, S_RQN2,
  // reciprocals and quotients of ray constants that the radial assembly would divide by at
  // every sample (case 3: 1/(1 - al_i^2), al0^2/jd, 1/(al0^2 - 1), (2k - n0)/jd, 1/C16,
  // 1/C17; case 4: 1/(1 + g_i^2))
  R_D0, R_D1, R_D2, R_D3, R_D4, R_D5, R_D6, R_D7,
  // coefficients of I_phi and I_t in I_+ and I_- (kgeo/kerr_raytracing_ana.py:626-633)
  F_CP, F_CM, F_TP, F_TM,
  // theta assembly: G_t = T_GTC (E - F) (ordinary motion), cos(theta) = T_NSQUP sn
  T_GTC, T_NSQUP,
  // products of the step's Jacobi values for the addition theorem (jacobi_add_q), theta then r:
  // m sn_v^2, cn_v dn_v, sn_v dn_v, m sn_v cn_v with sn_v = -S_TSN (-S_RSN), the step's sign
  S_TJ0, S_TJ1, S_TJ2, S_TJ3, S_RJ0, S_RJ1, S_RJ2, S_RJ3,
  // the recurrence states at tau = 0 (the observer), from the setup's integrals at the
  // observer's amplitudes: theta sn, cn, dn, e, pi; r sn, cn, dn, E, Pi_0..2
  T_SN0, T_CN0, T_DN0, T_E0, T_PI0, R_SN0, R_CN0, R_DN0, R_E0, R_PA0, R_PA1, R_PA2,
  NUM_FIELDS
};

// code bit: the ray's samples may be produced by the addition-theorem recurrence
constexpr int CODE_STEP = 1 << 10;
// code bits 11..15: the mixed-precision recurrence keeps the increments of this integral in
// FP64 (theta Pi, r Pi_0, Pi_1, Pi_2, r E) because its errors reach phi or t / r_o amplified
constexpr int CODE_F64_SHIFT = 11;
constexpr double MIXED_GAIN_MAX = 2.0;

// Strided view of one ray's record inside the structure-of-arrays buffer.
struct RecView {
  const double* base;  // &rec[ray]
  int64_t stride;      // npix
  KG_HD double operator[](int k) const {
#if defined(__CUDA_ARCH__)
    return __ldg(base + (int64_t)k * stride);
#else
    return base[(int64_t)k * stride];
#endif
  }
};

struct RayRec {
  double f[NUM_FIELDS];
  int code;  // rcase | thbranch << 4 | (kk == 0) << 8 | minspin << 9
};

KG_HD int code_rcase(int code) { return code & 15; }
KG_HD int code_th(int code) { return (code >> 4) & 15; }
KG_HD bool code_kk0(int code) { return (code >> 8) & 1; }
KG_HD bool code_minspin(int code) { return (code >> 9) & 1; }
KG_HD bool code_step(int code) { return (code >> 10) & 1; }
KG_HD bool code_f64(int code, int i) { return (code >> (CODE_F64_SHIFT + i)) & 1; }

// One Carlson evaluation at (x, y, z) for up to three Pi's plus R_D; rho[i] = the (scaled)
// 1 - n_i sin^2. For rho_i < 0 the DLMF 19.20.14 transform is used; rho == 0 gives +inf
// like the reference. A non-finite rho_i (an infinite characteristic, whose Pi the callers set
// to the reference adapter's 0) gives NaN without entering the shared duplication, which a NaN
// parameter would keep from converging.
template <int NP>
KG_HD void carlson_set(double x, double y, double z, const double* rho, double* rj, double* rd, double* rf) {
  double p[NP + 1];
  double q[NP];
  bool neg[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    neg[i] = !(rho[i] > 0.0);
    q[i] = -rho[i];
    p[i] = neg[i] ? (z * (x + y + q[i]) - x * y) / (z + q[i]) : rho[i];
    if (rho[i] == 0.0 || !std::isfinite(rho[i])) p[i] = z;  // placeholder, result replaced below
  }
  p[NP] = z;  // R_D(x,y,z) = R_J(x,y,z,z)
  double out[NP + 1];
  rj_multi<NP + 1>(x, y, z, p, out, rf);
  *rd = out[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    if (rho[i] == 0.0) {
      rj[i] = kg_inf();
    } else if (!std::isfinite(rho[i])) {
      rj[i] = kg_nan();
    } else if (neg[i]) {
      double pq = p[i] * q[i];
      double xy = x * y;
      double rc = carlson_rc(xy + pq, pq);
      rj[i] = ((p[i] - z) * out[i] - 3.0 * (*rf) + 3.0 * sqrt((xy * z) / (xy + pq)) * rc) / (q[i] + z);
    } else {
      rj[i] = out[i];
    }
  }
}

// F(phi|m), E(phi|m) and Pi(n_i; phi|m) at one amplitude with the semantics of ellip_f,
// ellip_e_inc and ellip_pi_ref (kgeo/scipy_ellip_binding.py:87-237 special cases included),
// from one shared Carlson duplication at the reduced amplitude; beyond |phi| > pi/2 the periodic
// parts come from `complete` (this function's result at pi/2 for the same m and n).
template <int NP>
struct EllipSet {
  double F, E, P[NP];
};

template <int NP>
KG_HD EllipSet<NP> ellip_set_at(double phi, double m, const double* n, const EllipSet<NP>* complete) {
  const double nr = rint(phi / PI);
  const double p0 = phi - nr * PI;
  const double s = sin(p0), c = cos(p0);
  double rho[NP], rj[NP], rd, rf;
#pragma unroll
  for (int i = 0; i < NP; ++i) rho[i] = 1.0 - n[i] * s * s;
  carlson_set<NP>(c * c, 1.0 - m * s * s, 1.0, rho, rj, &rd, &rf);
  const double s3 = s * s * s;
  EllipSet<NP> out;
  const double F0 = s * rf;
  out.F = nr == 0.0 ? F0 : F0 + 2.0 * nr * complete->F;
  const double E0 = s * rf - (m / 3.0) * s3 * rd;
  out.E = nr == 0.0 ? E0 : E0 + 2.0 * nr * complete->E;
  // ellip_pi_ref's rules, tested on the full amplitude
  const double sf = sin(phi);
  const double yf = 1.0 - m * sf * sf;
  const double aphi = fabs(phi);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    const double ni = n[i];
    const double rhof = 1.0 - ni * sf * sf;
    double v;
    if (aphi <= PHI_ZERO) v = phi;
    else if (m < M_NEG_INF) v = 0.0;
    else if (yf < 0.0) v = kg_nan();
    else if (aphi > HALFPI && m >= 1.0) v = kg_nan();
    else if (aphi > HALFPI && ni == 1.0) v = kg_inf();
    else if (rhof == 0.0) v = kg_inf();
    else if (std::isinf(ni)) v = 0.0;
    else {
      const double core = fabs(p0) <= PHI_ZERO && aphi > HALFPI ? p0 : s * rf + (ni / 3.0) * s3 * rj[i];
      v = aphi > HALFPI ? 2.0 * nr * complete->P[i] + core : core;
    }
    out.P[i] = v;
  }
  return out;
}

// ---------------------------------------------------------------------------
// building blocks at a generic amplitude (ray constants)
// ---------------------------------------------------------------------------

// S1, S2 of GL19a B92/B93 (kgeo/kerr_raytracing_ana.py:638-663) at amplitude phi, from
// F(phi|j), E(phi|j) and Pi(1 + al^2; phi|j) evaluated by the caller (ellip_set_at).
KG_HD void s1s2_at(double al, double phi, double j, double F, double E, double Pi, bool want_s2, double* S1,
                   double* S2) {
  double al2 = al * al;
  double al2p1 = 1 + al2;
  double al2j = 1 - j + al2;
  double sphi = sin(phi);
  double s2phi = sqrt(1. - j * (sphi * sphi));
  double p2 = sqrt(al2p1 / al2j);
  double f2 = 0.5 * p2 * log(fabs(((1 - p2) * (1 + p2 * s2phi)) / ((1 + p2) * (1 - p2 * s2phi))));
  *S1 = (F + al2 * Pi - al * f2) / al2p1;
  if (want_s2) {
    double tanphi = tan(phi);
    double S2a = (1 - j) * F + al2 * E + al2 * s2phi * (al - tanphi) / (1 + al * tanphi) - al2 * al;
    S2a = -S2a / (al2p1 * al2j);
    double S2b = *S1 * (1. / al2p1 + (1 - j) / al2j);
    *S2 = S2a + S2b;
  }
}

// R1, R2 of GL19a B62/B65 (kgeo/kerr_raytracing_ana.py:666-683) at amplitude phi, from
// F(phi|j), E(phi|j) and Pi(al^2 / (al^2 - 1); phi|j) evaluated by the caller.
KG_HD void r1r2_at(double al, double phi, double j, double F, double E, double Pi, bool want_r2, double* R1,
                   double* R2) {
  double al2 = al * al;
  double sphi = sin(phi);
  double s2phi = sqrt(1 - j * (sphi * sphi));
  double p1 = sqrt((al2 - 1) / (j + (1 - j) * al2));
  double f1 = 0.5 * p1 * log(fabs((p1 * s2phi + sphi) / (p1 * s2phi - sphi)));
  double nn = al2 / (al2 - 1);
  *R1 = (Pi - al * f1) / (1 - al2);
  if (want_r2) {
    double r2 = (F - (al2 / (j + (1 - j) * al2)) * (E - al * sphi * s2phi / (1 + al * cos(phi)))) / (al2 - 1);
    *R2 = r2 + (2 * j - nn) * *R1 / (j + (1 - j) * al2);
  }
}

// ---------------------------------------------------------------------------
// per-ray setup
// ---------------------------------------------------------------------------

struct Turning {
  double up, um;
};

// u_+, u_- with the reference's clamps (kgeo/kerr_raytracing_utils.py:290-326). Below
// MINSPIN the reference binds u_- to the same array as u_+, so every clamp lands on both.
KG_HD Turning u_turning(const Observer& o, double lam, double eta) {
  double up, um;
  if (o.minspin) {
    up = eta / (eta + lam * lam);
    if ((o.cos2 - up) > 0) up = o.cos2;
    if (up * up > 1) up = 1;
    if (up == 0 && eta < 0) up = EP;
    if (up == 0 && eta >= 0) up = -EP;
    if (eta < 0 && (o.cos2 - up) < 0) up = o.cos2;
    um = up;
  } else {
    const double a = o.a;
    double half = 0.5 * (1 - (eta + lam * lam) / (a * a));
    double root = sqrt(half * half + eta / (a * a));
    up = half + root;
    um = half - root;
    if ((o.cos2 - up) > 0) up = o.cos2;
    if (up * up > 1) up = 1;
    if (um == 0 && eta < 0) um = EP;
    if (um == 0 && eta >= 0) um = -EP;
    if (eta < 0 && (o.cos2 - um) < 0) um = o.cos2;
  }
  return Turning{up, um};
}

// u_+/u_- and a^2 u_- as uplus_uminus returns them (0 and -(eta + lam^2) below MINSPIN).
KG_HD void u_ratio(const Observer& o, double lam, double eta, const Turning& U, double* ratio, double* a2um) {
  if (o.minspin) {
    *ratio = 0. * U.um;
    *a2um = -(eta + lam * lam);
  } else {
    *ratio = U.up / U.um;
    *a2um = o.a2 * U.um;
  }
}


struct Roots {
  cplx r1, r2, r3, r4;
  int rclass;
};

// kgeo/kerr_raytracing_utils.py:330-380
KG_HD Roots radial_roots(const Observer& o, double lam, double eta) {
  double A = o.a2 - eta - lam * lam;
  double lma = lam - o.a;
  double B = 2 * (eta + lma * lma);
  double C = -(o.a2) * eta;
  double P = -(A * A) / 12. - C;
  double Q = (-A / 3.) * ((A * A) / 36. - C) - (B * B) / 8.;
  cplx disc = cx_real(4 * cube_rn(P) + 27 * (Q * Q));
  cplx sd = csqrt(disc / cx_real(108.));
  cplx wp3 = cx_real(-0.5 * Q) + sd;
  cplx wm3 = cx_real(-0.5 * Q) - sd;
  cplx xi0 = cbrt_max_real(wp3) + cbrt_max_real(wm3) - cx_real(A / 3.);
  cplx z = csqrt(cx_real(0.5) * xi0);
  cplx zz = z * z;
  cplx bz = cx_real(0.25 * B) / z;
  cplx base = cx_real(-0.5 * A) - zz;
  cplx s_lo = csqrt(base + bz);
  cplx s_hi = csqrt(base - bz);
  Roots R;
  R.r1 = -z - s_lo;
  R.r2 = -z + s_lo;
  R.r3 = z - s_hi;
  R.r4 = z + s_hi;
  int rc = 0;
  if (R.r2.im != 0) rc = 4;
  if (R.r2.im == 0 && R.r4.im != 0) rc = 3;
  if (R.r2.im == 0 && R.r4.im == 0 && R.r4.re < o.rplus) rc = 2;
  if (R.r2.im == 0 && R.r4.im == 0 && R.r4.re > o.rplus) rc = 1;
  R.rclass = rc;
  return R;
}

// Total Mino time from the observer to the horizon or back out to infinity
// (kgeo/kerr_raytracing_utils.py:382-548, regions IV, III, II, I).
KG_HD double mino_total(const Observer& o, const Roots& R) {
  const double rplus = o.rplus, r_o = o.r_o;
  double tau_tot = 0.0;
  bool m4 = R.r1.im != 0;
  bool m3 = (R.r3.im != 0) && !m4;
  bool mII = (R.r3.im == 0.) && (R.r3.re < rplus || (R.r3.re == rplus && R.r3.im < 0)) && !m3;
  bool mI = (R.r3.im == 0.) && (R.r3.re > rplus || (R.r3.re == rplus && R.r3.im > 0)) && !mII;
  if (m4) {
    double a1 = R.r4.im, b1 = R.r4.re, a2i = R.r2.im, b2 = R.r2.re;
    double CC = sqrt((a1 - a2i) * (a1 - a2i) + (b1 - b2) * (b1 - b2));
    double DD = sqrt((a1 + a2i) * (a1 + a2i) + (b1 - b2) * (b1 - b2));
    double k4 = (4 * CC * DD) / ((CC + DD) * (CC + DD));
    double g0 = sqrt((4 * (a2i * a2i) - (CC - DD) * (CC - DD)) / ((CC + DD) * (CC + DD) - 4 * (a2i * a2i)));
    double x4rp = (rplus + b1) / a2i;
    double x4ro = o.r_o_inf ? kg_inf() : (r_o + b1) / a2i;
    double pref = 2. / (CC + DD);
    double I4rp = pref * ellip_f(atan(x4rp) + atan(g0), k4);
    double I4ro = pref * ellip_f(atan(x4ro) + atan(g0), k4);
    tau_tot = I4ro - I4rp;
  }
  if (m3) {
    double a1 = R.r4.im, b1 = R.r4.re, rr1 = R.r1.re, rr2 = R.r2.re;
    double rr21 = rr2 - rr1;
    double rrp1 = rplus - rr1, rrp2 = rplus - rr2;
    double AA = sqrt(a1 * a1 + (b1 - rr2) * (b1 - rr2));
    double BB = sqrt(a1 * a1 + (b1 - rr1) * (b1 - rr1));
    double k3 = ((AA + BB) * (AA + BB) - rr21 * rr21) / (4 * AA * BB);
    double x3rp = (AA * rrp1 - BB * rrp2) / (AA * rrp1 + BB * rrp2);
    double x3ro;
    if (o.r_o_inf) x3ro = (AA - BB) / (AA + BB);
    else x3ro = (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2));
    double pref = 1. / sqrt(AA * BB);
    double I3rp = pref * ellip_f(acos(x3rp), k3);
    double I3ro = pref * ellip_f(acos(x3ro), k3);
    tau_tot = I3ro - I3rp;
  }
  if (mII || mI) {
    double rr1 = R.r1.re, rr2 = R.r2.re, rr3 = R.r3.re, rr4 = R.r4.re;
    double rr31 = rr3 - rr1, rr32 = rr3 - rr2, rr41 = rr4 - rr1, rr42 = rr4 - rr2;
    double k2 = (rr32 * rr41) / (rr31 * rr42);
    double x2ro = o.r_o_inf ? sqrt(rr31 / rr41) : sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)));
    double pref = 2. / sqrt(rr31 * rr42);
    if (mII) {
      double x2rp = sqrt((rr31 * (rplus - rr4)) / (rr41 * (rplus - rr3)));
      double I2rp = pref * ellip_f(asin(x2rp), k2);
      double I2ro = pref * ellip_f(asin(x2ro), k2);
      tau_tot = I2ro - I2rp;
    } else {
      double I2ro = pref * ellip_f(asin(x2ro), k2);
      tau_tot = 2 * I2ro;
    }
  }
  return tau_tot;
}

// Everything that depends only on the ray. Writes the record, returns the flags it raises.
// `anyflags` are the launch-wide flags (only FLAG_ANY_ETA_POS is read, and only by
// eta == 0 rays; pass FLAG_ANY_ETA_POS when unknown and fix up later).
KG_HD unsigned ray_setup(const Observer& o, double alpha, double beta, double maxtaufrac,
                         RayRec* rec, int* rclass_out, int* thclass_out) {
  unsigned flags = 0;
  double* f = rec->f;
  for (int i = 0; i < NUM_FIELDS; ++i) f[i] = 0.0;
  const double a = o.a, a2 = o.a2;

  // conserved quantities, kgeo/kerr_raytracing_ana.py:151-158
  double lam = -alpha * o.sin_th;
  double eta = (alpha * alpha - a2) * o.cos2 + beta * beta;
  if (o.minspin && eta < 0) eta = EP;
  if (eta > 0) flags |= FLAG_ANY_ETA_POS;
  if (eta <= 0) flags |= FLAG_ANY_ETA_NONPOS;
  if (o.minspin && eta <= 0) flags |= FLAG_MINSPIN_VORTICAL;
  double s = beta >= 0 ? 1.0 : -1.0;  // my_sign, kgeo/kerr_raytracing_utils.py:857-864
  f[F_LAM] = lam;
  f[F_S] = s;
  f[G_A] = a;
  f[G_RP] = o.rplus;
  f[G_RM] = o.rminus;
  f[G_RO] = o.r_o;
  {
    const double rp = o.rplus, rm = o.rminus;
    const double c2 = 2 * a / (rp - rm), c4 = 4 / (rp - rm);
    f[F_CP] = c2 * (rp - 0.5 * a * lam);
    f[F_CM] = c2 * (rm - 0.5 * a * lam);
    f[F_TP] = c4 * (rp * rp - 0.5 * a * lam * rp);
    f[F_TM] = c4 * (rm * rm - 0.5 * a * lam * rm);
  }

  // u_+, u_- with clamps, kgeo/kerr_raytracing_utils.py:290-326
  Turning U = u_turning(o, lam, eta);
  const double up = U.up, um = U.um;
  *thclass_out = eta > 0 ? 1 : (eta < 0 ? 2 : 3);

  // radial roots and rclass
  Roots R = radial_roots(o, lam, eta);
  *rclass_out = R.rclass;

  // ---- total Mino time, kgeo/kerr_raytracing_utils.py:382-548
  const double rplus = o.rplus, rminus = o.rminus, r_o = o.r_o;
  double tau_tot = mino_total(o, R);
  f[F_TAUTOT] = tau_tot;
  double taumax = maxtaufrac * tau_tot;
  f[F_TAUMAX] = taumax;

  // ---- theta constants, kgeo/kerr_raytracing_ana.py:216-363
  int th = TH_ZERO;
  bool kk0 = false;
  if (eta >= 0.) {
    // ordinary (taken by eta == 0 rays only when some eta > 0; the kernel decides)
    th = TH_ORD;
    double kk, a2um;
    if (o.minspin) {
      kk = 0.0;
      a2um = -(eta + lam * lam);
      kk0 = true;
    } else {
      kk = up / um;
      a2um = a * a * um;
      kk0 = (kk == 0);
    }
    double pref = 1 / sqrt(-a2um);
    double arg = asin(o.cos_th / sqrt(up));
    // F, E, Pi at the observer's amplitude and the complete set, each from one duplication
    const double nth[1] = {up};
    const EllipSet<1> cth = ellip_set_at<1>(HALFPI, kk, nth, nullptr);
    const EllipSet<1> ath = ellip_set_at<1>(arg, kk, nth, &cth);
    double F = ath.F;
    double Gth_o = -pref * F;
    double Gph_o = -pref * ath.P[0];
    {
      // state at tau = 0: snarg = -s F(arg | kk), so the amplitude is -s arg
      const double sa = o.cos_th / sqrt(up);
      f[T_SN0] = -s * sa;
      f[T_CN0] = sqrt(1.0 - sa * sa);
      f[T_DN0] = sqrt(1.0 - kk * (sa * sa));
      f[T_E0] = -s * (ath.E - F);
      f[T_PI0] = -s * ath.P[0];
    }
    double Gt_o;
    if (kk == 0) Gt_o = 2 * up * pref * 0.125 * (-2 * arg + sin(2 * arg));
    else Gt_o = 2 * up * pref * (ath.E - F) / (2 * kk);
    double m = kk / (kk - 1);
    f[T_SCALE] = sqrt(-a2um);
    f[T_GTH] = Gth_o;
    f[T_M] = m;
    f[T_S1M] = sqrt(1 - m);
    f[T_K2] = 2.0 * ellip_k(m);
    f[T_N] = up;
    f[T_KK] = kk;
    f[T_PIC] = cth.P[0];
    f[T_EC] = cth.E;
    f[T_KC] = cth.F;
    f[T_PREF] = pref;
    f[T_GPH] = Gph_o;
    f[T_GT] = Gt_o;
    f[T_UP] = up;
    f[T_UM] = um;
    f[T_GTC] = kk == 0 ? 0.0 : -(2 * up * pref) / (2 * kk);
    f[T_NSQUP] = -s * sqrt(up);
  }
  if (eta < 0.) {
    th = TH_VORT;
    double ratio = up / um;
    double a2um = a * a * um;
    double h = (o.th_o <= PI / 2) ? 1. : -1.;
    double prefA = 1 / sqrt(a2um);
    double prefB = prefA / (1. - um);
    double prefC = sqrt(um / (a * a));
    double nu_o = asin(sqrt((o.cos2 - um) / (up - um)));
    double kk = 1 - ratio;
    double upm = (up - um) / (1. - um);
    const double nth[1] = {upm};
    const EllipSet<1> cth = ellip_set_at<1>(HALFPI, kk, nth, nullptr);
    const EllipSet<1> ath = ellip_set_at<1>(nu_o, kk, nth, &cth);
    double Gth_o = -h * prefA * ath.F;
    double Gph_o = -h * prefB * ath.P[0];
    double Gt_o = -h * prefC * ath.E;
    {
      // state at tau = 0: snarg = -s h F(nu_o | kk), amplitude -s h nu_o
      const double sn = sqrt((o.cos2 - um) / (up - um));
      f[T_SN0] = -s * h * sn;
      f[T_CN0] = sqrt(1.0 - sn * sn);
      f[T_DN0] = sqrt(1.0 - kk * (sn * sn));
      f[T_E0] = -s * h * ath.E;
      f[T_PI0] = -s * h * ath.P[0];
    }
    double m = kk / (kk - 1);
    f[T_SCALE] = sqrt(a2um);
    f[T_GTH] = Gth_o;
    f[T_M] = m;
    f[T_S1M] = sqrt(1 - m);
    f[T_K2] = 2.0 * ellip_k(m);
    f[T_N] = upm;
    f[T_KK] = kk;
    f[T_PIC] = cth.P[0];
    f[T_EC] = cth.E;
    f[T_KC] = cth.F;
    f[T_PREF] = prefB;
    f[T_GPH] = Gph_o;
    f[T_GT] = Gt_o;
    f[T_UP] = up;
    f[T_UM] = um;
    f[T_PREFC] = prefC;
    f[T_H] = h;
  }

  // ---- radial constants, kgeo/kerr_raytracing_ana.py:389-624
  int rcase = RCASE_NONE;
  bool c4 = R.r1.im != 0;
  bool c3 = (R.r3.im != 0) && !c4;
  bool c2 = (R.r3.im == 0.) && !c3;
  if (c4) {
    rcase = RCASE_4;
    double a1 = R.r4.im, b1 = R.r4.re, a2i = R.r2.im, b2 = R.r2.re;
    double CC = sqrt((a1 - a2i) * (a1 - a2i) + (b1 - b2) * (b1 - b2));
    double DD = sqrt((a1 + a2i) * (a1 + a2i) + (b1 - b2) * (b1 - b2));
    double k4 = (4 * CC * DD) / ((CC + DD) * (CC + DD));
    double x4rp = (rplus + b1) / a2i;
    double x4rm = (rminus + b1) / a2i;
    double x4ro = o.r_o_inf ? kg_inf() : (r_o + b1) / a2i;
    double g0 = sqrt((4 * (a2i * a2i) - (CC - DD) * (CC - DD)) / ((CC + DD) * (CC + DD) - 4 * (a2i * a2i)));
    double gp = (g0 * x4rp - 1.) / (g0 + x4rp);
    double gm = (g0 * x4rm - 1.) / (g0 + x4rm);
    double aux = atan(x4ro) + atan(g0);
    double pref = 2. / (CC + DD);
    const double nn4[3] = {1 + g0 * g0, 1 + gp * gp, 1 + gm * gm};
    const EllipSet<3> comp = ellip_set_at<3>(HALFPI, k4, nn4, nullptr);
    const EllipSet<3> at = ellip_set_at<3>(aux, k4, nn4, &comp);
    {
      // state at tau = 0: X = F(aux | k), so sn = sin(aux), cn = cos(aux)
      const double sn = sin(aux), cn = cos(aux);
      f[R_SN0] = sn;
      f[R_CN0] = cn;
      f[R_DN0] = sqrt(1.0 - k4 * (sn * sn));
      f[R_E0] = at.E;
      f[R_PA0] = at.P[0];
      f[R_PA1] = at.P[1];
      f[R_PA2] = at.P[2];
    }
    double Ir_o = pref * at.F;
    double S1b0, S2b0, S1bp, S1bm, dummy;
    s1s2_at(g0, aux, k4, at.F, at.E, at.P[0], true, &S1b0, &S2b0);
    s1s2_at(gp, aux, k4, at.F, at.E, at.P[1], false, &S1bp, &dummy);
    s1s2_at(gm, aux, k4, at.F, at.E, at.P[2], false, &S1bm, &dummy);
    double aa0 = (a2i / g0) * (1 + g0 * g0);
    double aa1 = (a2i / g0 - b1);
    f[R_XS] = 1. / pref;
    f[R_IRO] = Ir_o;
    f[R_M] = k4;
    f[R_KC] = comp.F;
    f[R_K2] = 2.0 * f[R_KC];
    f[R_EC] = comp.E;
    f[R_N0] = nn4[0];
    f[R_N1] = nn4[1];
    f[R_N2] = nn4[2];
    f[R_PIC0] = comp.P[0];
    f[R_PIC1] = comp.P[1];
    f[R_PIC2] = comp.P[2];
    f[R_C0] = a2i;
    f[R_C1] = b1;
    f[R_C2] = g0;
    f[R_C3] = gp;
    f[R_C4] = gm;
    f[R_C5] = S1b0;
    f[R_C6] = S2b0;
    f[R_C7] = S1bp;
    f[R_C8] = S1bm;
    f[R_C9] = pref * aa0;                                     // Pi_1 = s*pref*aa0*(..)
    f[R_C10] = pref * (aa0 * aa0);                            // Pi_2
    f[R_C11] = pref * (1 + g0 * g0) / (g0 * g0 + g0 * x4rp);  // Pi_p
    f[R_C12] = pref * (1 + g0 * g0) / (g0 * g0 + g0 * x4rm);  // Pi_m
    f[R_C13] = aa1;
    f[R_C14] = g0 / (a2i - a2i * g0 * x4rp);
    f[R_C15] = g0 / (a2i - a2i * g0 * x4rm);
    const double g4[3] = {g0, gp, gm};
    for (int i = 0; i < 3; ++i) {  // p2 of S1_S2 for g0, gp, gm
      const double gg = g4[i] * g4[i];
      f[R_C20 + i] = sqrt((1 + gg) / (1 - k4 + gg));
    }
    const double g02 = g0 * g0, g02p1 = 1 + g02, g02j = 1 - k4 + g02;
    f[R_C23] = -1.0 / (g02p1 * g02j);           // S2 = S2a f[R_C23] + S1_0 f[R_C24]
    f[R_C24] = 1. / g02p1 + (1 - k4) / g02j;
    for (int i = 0; i < 3; ++i) f[R_D0 + i] = 1.0 / (1 + g4[i] * g4[i]);
  }
  if (c3) {
    rcase = RCASE_3;
    double a1 = R.r4.im, b1 = R.r4.re, rr1 = R.r1.re, rr2 = R.r2.re;
    double rr21 = rr2 - rr1;
    double rrp1 = rplus - rr1, rrp2 = rplus - rr2, rrm1 = rminus - rr1, rrm2 = rminus - rr2;
    double AA = sqrt(a1 * a1 + (b1 - rr2) * (b1 - rr2));
    double BB = sqrt(a1 * a1 + (b1 - rr1) * (b1 - rr1));
    double k3 = ((AA + BB) * (AA + BB) - rr21 * rr21) / (4 * AA * BB);
    double x3rp = (AA * rrp1 - BB * rrp2) / (AA * rrp1 + BB * rrp2);
    double x3rm = (AA * rrm1 - BB * rrm2) / (AA * rrm1 + BB * rrm2);
    double x3ro;
    if (o.r_o_inf) x3ro = (AA - BB) / (AA + BB);
    else x3ro = (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2));
    double alp = -1. / x3rp;
    double alm = -1. / x3rm;
    double al0 = (BB + AA) / (BB - AA);
    double aux = acos(x3ro);
    double pref = (1. / sqrt(AA * BB));
    double a0s = al0 * al0, aps = alp * alp, ams = alm * alm;
    const double nn3[3] = {a0s / (a0s - 1), aps / (aps - 1), ams / (ams - 1)};
    const EllipSet<3> comp = ellip_set_at<3>(HALFPI, k3, nn3, nullptr);
    const EllipSet<3> at = ellip_set_at<3>(aux, k3, nn3, &comp);
    {
      // state at tau = 0: X = F(aux | k), so sn = sin(aux), cn = cos(aux)
      const double sn = sqrt(1.0 - x3ro * x3ro), cn = x3ro;
      f[R_SN0] = sn;
      f[R_CN0] = cn;
      f[R_DN0] = sqrt(1.0 - k3 * (sn * sn));
      f[R_E0] = at.E;
      f[R_PA0] = at.P[0];
      f[R_PA1] = at.P[1];
      f[R_PA2] = at.P[2];
    }
    double Ir_o = pref * at.F;
    double R1b0, R2b0, R1bp, R1bm = 0.0, dummy;
    r1r2_at(al0, aux, k3, at.F, at.E, at.P[0], true, &R1b0, &R2b0);
    r1r2_at(alp, aux, k3, at.F, at.E, at.P[1], false, &R1bp, &dummy);
    if (fabs(a) > MINSPIN) r1r2_at(alm, aux, k3, at.F, at.E, at.P[2], false, &R1bm, &dummy);
    double sAB = sqrt(AA * BB);
    f[R_XS] = 1. / pref;
    f[R_IRO] = Ir_o;
    f[R_M] = k3;
    f[R_KC] = comp.F;
    f[R_K2] = 2.0 * f[R_KC];
    f[R_EC] = comp.E;
    f[R_N0] = nn3[0];
    f[R_N1] = nn3[1];
    f[R_N2] = nn3[2];
    f[R_PIC0] = comp.P[0];
    f[R_PIC1] = comp.P[1];
    f[R_PIC2] = comp.P[2];
    f[R_C0] = AA;
    f[R_C1] = BB;
    f[R_C2] = rr1;
    f[R_C3] = rr2;
    f[R_C4] = al0;
    f[R_C5] = alp;
    f[R_C6] = alm;
    f[R_C7] = R1b0;
    f[R_C8] = R2b0;
    f[R_C9] = R1bp;
    f[R_C10] = R1bm;
    f[R_C11] = (2 * rr21 * sAB) / (BB * BB - AA * AA);    // Pi_1 coefficient
    f[R_C12] = (2 * rr21 * sAB) / (BB * rrp2 - AA * rrp1);  // Pi_p
    f[R_C13] = (2 * rr21 * sAB) / (BB * rrm2 - AA * rrm1);  // Pi_m
    f[R_C14] = ((BB * rr2 + AA * rr1) / (BB + AA));        // pref of I1/I2
    f[R_C15] = sAB;
    f[R_C16] = (BB * rrp2 + AA * rrp1);
    f[R_C17] = (BB * rrm2 + AA * rrm1);
    f[R_C18] = sqrt((a0s - 1) / (k3 + (1 - k3) * a0s));  // p1 of R1_R2 for al0, alp, alm
    f[R_C19] = sqrt((aps - 1) / (k3 + (1 - k3) * aps));
    f[R_C20] = sqrt((ams - 1) / (k3 + (1 - k3) * ams));
    const double jd = k3 + (1 - k3) * a0s;
    f[R_D0] = 1.0 / (1 - a0s);
    f[R_D1] = 1.0 / (1 - aps);
    f[R_D2] = 1.0 / (1 - ams);
    f[R_D3] = a0s / jd;
    f[R_D4] = 1.0 / (a0s - 1);
    f[R_D5] = (2 * k3 - nn3[0]) / jd;
    f[R_D6] = 1.0 / f[R_C16];
    f[R_D7] = 1.0 / f[R_C17];
  }
  if (c2) {
    rcase = RCASE_2;
    double rr1 = R.r1.re, rr2 = R.r2.re, rr3 = R.r3.re, rr4 = R.r4.re;
    double rr31 = rr3 - rr1, rr32 = rr3 - rr2, rr41 = rr4 - rr1, rr42 = rr4 - rr2, rr43 = rr4 - rr3;
    double rrp3 = rplus - rr3, rrm3 = rminus - rr3, rrp4 = rplus - rr4, rrm4 = rminus - rr4;
    double k2 = (rr32 * rr41) / (rr31 * rr42);
    double x2ro = o.r_o_inf ? sqrt(rr31 / rr41) : sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)));
    double aux = asin(x2ro);
    double n1 = rr41 / rr31;
    double np = (rrp3 * rr41) / (rrp4 * rr31);
    double nm = (rrm3 * rr41) / (rrm4 * rr31);
    const double nn2[3] = {n1, np, nm};
    const EllipSet<3> comp = ellip_set_at<3>(HALFPI, k2, nn2, nullptr);
    const EllipSet<3> at = ellip_set_at<3>(aux, k2, nn2, &comp);
    {
      // state at tau = 0: X = F(aux | k), so sn = sin(aux), cn = cos(aux)
      const double sn = x2ro, cn = sqrt(1.0 - x2ro * x2ro);
      f[R_SN0] = sn;
      f[R_CN0] = cn;
      f[R_DN0] = sqrt(1.0 - k2 * (sn * sn));
      f[R_E0] = at.E;
      f[R_PA0] = at.P[0];
      f[R_PA1] = at.P[1];
      f[R_PA2] = at.P[2];
    }
    double Ir_o = 2 * at.F / sqrt(rr31 * rr42);
    double Rpot_o = (r_o - rr1) * (r_o - rr2) * (r_o - rr3) * (r_o - rr4);
    double drs_o = sqrt(Rpot_o);
    double c2c = 2. / sqrt(rr31 * rr42);
    f[R_XS] = 0.5 * sqrt(rr31 * rr42);
    f[R_IRO] = Ir_o;
    f[R_M] = k2;
    f[R_KC] = comp.F;
    f[R_K2] = 2.0 * f[R_KC];
    f[R_EC] = comp.E;
    f[R_N0] = n1;
    f[R_N1] = np;
    f[R_N2] = nm;
    f[R_PIC0] = comp.P[0];
    f[R_PIC1] = comp.P[1];
    f[R_PIC2] = comp.P[2];
    f[R_C0] = rr1;
    f[R_C1] = rr2;
    f[R_C2] = rr3;
    f[R_C3] = rr4;
    f[R_C4] = at.E;                          // E(aux)
    f[R_C5] = at.P[0];                       // Pi(n1; aux)
    f[R_C6] = at.P[1];
    f[R_C7] = at.P[2];
    f[R_C8] = drs_o / (r_o - rr3);           // second term of H
    f[R_C9] = c2c;
    f[R_C10] = c2c * (rr43 / (rrp3 * rrp4));
    f[R_C11] = c2c * (rr43 / (rrm3 * rrm4));
    f[R_C12] = sqrt(rr31 * rr42);
    f[R_C13] = rrp3;
    f[R_C14] = rrm3;
    f[R_C15] = 0.5 * (rr1 * rr4 + rr2 * rr3);
    f[R_C16] = rr31;
    f[R_C17] = rr41;
    f[R_C18] = rr43;
    f[R_C20] = 1.0 / rrp3;
    f[R_C21] = 1.0 / rrm3;
  }
  rec->code = rcase | (th << 4) | ((kk0 ? 1 : 0) << 8) | ((o.minspin ? 1 : 0) << 9);
  return flags;
}

// ---------------------------------------------------------------------------
// per-sample evaluation
//
// A sample is evaluated in two stages: the elliptic state of the ray at that Mino time
// (Jacobi sn, cn, dn of the theta and r arguments and the running values of E, E - F and
// every Pi), then the assembly of r, theta, G_phi, G_t, I_phi, I_t, I_sigma from that state
// (GL19a B46-B116 and 29-68, as kgeo/kerr_raytracing_ana.py:216-633 combines them).
// The state comes either from a direct evaluation (Landen + Carlson, any tau) or from the
// previous sample of an evenly spaced Mino grid by the addition theorems of sn, cn, dn
// (DLMF 22.8.1-3), of E (DLMF 22.16.27 / 19.11.2) and of Pi:
//   Pi(n; am(u+v)) = Pi(n; am u) + Pi(n; am v) + n S3 sgn(X) R_C(X^2, X^2 - n (m - n)(1 - n) S3^2),
//   S3 = sn u sn v sn(u+v),  X = 1 - n sn^2(u+v) + n sn u sn v cn(u+v) dn(u+v),
// which follows from Jacobi's addition theorem for the third kind after eliminating the
// characteristic's parameter (n = m sn^2 a). For small steps the R_C ratio is tiny and
// R_C is a short series.
// ---------------------------------------------------------------------------

struct Sample {
  double t, r, th, ph, sig;
};

// Pi(n; Phi | m) for the amplitude Phi = nr*pi + phi0, |phi0| <= pi/2, from the
// shared Carlson values; mirrors the special cases of kgeo/scipy_ellip_binding.py:125-162.
// inc = Pi(n; phi0 | m) already evaluated (finite path), pic = Pi(n | m).
KG_HD double pi_assemble(double n, double Phi, double nr, double inc, double pic, double m) {
  double aphi = fabs(Phi);
  if (aphi <= PHI_ZERO) return Phi;
  if (m < M_NEG_INF) return 0.0;
  if (aphi > HALFPI && n == 1.0) return kg_inf();
  if (std::isinf(n)) return 0.0;
  return nr == 0.0 ? inc : 2.0 * nr * pic + inc;
}


// ---- addition theorems -----------------------------------------------------

struct JacobiW {
  double sn, cn, dn;
};

// sn, cn, dn(u + v | m) from the values at u and v (DLMF 22.8.1-3), any real m.
KG_HD JacobiW jacobi_add(double snu, double cnu, double dnu, double snv, double cnv, double dnv, double m) {
  double inv = rcp_fast(1.0 - m * (snu * snu) * (snv * snv));
  JacobiW w;
  w.sn = (snu * cnv * dnv + snv * cnu * dnu) * inv;
  w.cn = (cnu * cnv - snu * snv * dnu * dnv) * inv;
  w.dn = (dnu * dnv - m * snu * snv * cnu * cnv) * inv;
  return w;
}

// jacobi_add with the step's products q = (m sn_v^2, cn_v dn_v, sn_v dn_v, m sn_v cn_v) formed
// once per ray.
KG_HD JacobiW jacobi_add_q(double snu, double cnu, double dnu, double snv, double cnv, double dnv,
                           const double q[4]) {
  const double inv = rcp_fast(fma(-q[0], snu * snu, 1.0));
  JacobiW w;
  w.sn = fma(snu, q[1], snv * (cnu * dnu)) * inv;
  w.cn = fma(-(snu * dnu), q[2], cnu * cnv) * inv;
  w.dn = fma(-(snu * cnu), q[3], dnu * dnv) * inv;
  return w;
}

KG_HD void jacobi_step_products(double snv, double cnv, double dnv, double m, double* q) {
  q[0] = m * (snv * snv);
  q[1] = cnv * dnv;
  q[2] = snv * dnv;
  q[3] = m * snv * cnv;
}

// Distance rho = 1 - n sn^2 to a pole (n > 1) or near-pole (n slightly below 1, at a
// turning point close to the polar axis) of a Pi integrand. Within rho < POLE_RHO_PI of any
// characteristic, at the previous or the new sample, the recurrence state's rounding is
// amplified by 1/rho: that sample and the one after it are evaluated directly and the
// recurrence is re-seeded from them (in the radial state, with one characteristic near its
// pole, only that Pi is re-evaluated, from fresh sn, cn, dn; E and the other Pi keep stepping).
// The radial characteristic n0 is also the pole of the r
// formula (r ~ 1 / (1 - n0 sn^2)), so r carries the recurrence's drift of sn amplified by
// 1 / rho over the wider zone rho < POLE_RHO_R: there the step keeps its integrals but takes
// sn, cn, dn from a direct Jacobi evaluation. The radial state's drift grows with the steps
// taken since its sn, cn, dn were last evaluated directly (k), and with it the error the pole
// amplifies: the radial Pi zone is POLE_RHO_PI up to k = PI_ZONE_K0 and widens in proportion to
// k beyond (2.6e-3 at the 63rd step of a 64-sample chunk). On a seeded 1/64 of the
// 2048^2-plus-band rays a flat 1e-3 zone left phi up to 1.2x the 1e-10 bar at k = 56-63 and rho
// just above 1e-3 (0.6x at k < 32), from the radial Pi; with the widening zone 0.74x. The theta
// zone stays at POLE_RHO_PI (widening it too cost 2 % more and moved phi's maximum to 0.73x).
// (FP64 parity within the conditioning bar max(1e-10, 10 eps / rho), measured over seeded
// 512x512-range draws and that workload.) POLE_RHO is the float-float path's zone (kg_mixed.cuh,
// kg_mixed2.cuh).
constexpr double POLE_RHO = 2.0e-2;
constexpr double POLE_RHO_R = 5.0e-3;
constexpr double POLE_RHO_PI = 1.0e-3;
constexpr int PI_ZONE_K0 = 24;

// The radial Pi zone after k steps of the recurrence since the last direct Jacobi evaluation.
KG_HD double pi_zone(int k) { return k > PI_ZONE_K0 ? POLE_RHO_PI * ((double)k / PI_ZONE_K0) : POLE_RHO_PI; }

KG_HD bool near_pi_pole(double n, double sn, double rho_max = POLE_RHO) {
  return n > 0.0 && fabs(1.0 - n * (sn * sn)) < rho_max;
}

// Pi(n; am(u+v)) - Pi(n; am u) - Pi(n; am v) for parameter m, c = n (m - n)(1 - n):
//   n S3 sgn(X) R_C(X^2, X^2 - c S3^2)
// written in branch-continuous form: (n / sqrt(-c)) atan2(sqrt(-c) S3, X) for c < 0 and
// (n / 2 sqrt(c)) ln|(X + sqrt(c) S3) / (X - sqrt(c) S3)| for c > 0 (the principal value when
// the step crosses a pole of the integrand, as the reference's Pi takes it there); the
// R_C series n t R_C(1, 1 - c t^2), t = S3 / X, when z2 = c t^2 is small. For c > 0 the log
// form is (n / sqrt c) atanh(sqrt(c) t) = n t R_C(1, 1 - z2) at either sign of X (past a pole,
// X < 0); for c < 0 the series is the atan2 form only at X > 0 (at X < 0 atan2 adds +-pi).
KG_HD double pi_add_term(double n, double c, double snu, double snv, const JacobiW& w) {
  double S3 = snu * snv * w.sn;
  double X = 1.0 - n * (w.sn * w.sn) + n * snu * snv * w.cn * w.dn;
  double iX = rcp_fast(X);
  double t = S3 * iX;
  double z2 = c * (t * t);
  if ((X > 0.0 || c > 0.0) && fabs(z2) < 2.0e-3) return n * t * rc_one(-z2);
  if (c > 0.0) {
    double sc = sqrt(c);
    double q = sc * S3;
    return n / (2.0 * sc) * log(fabs((X + q) / (X - q)));
  }
  if (c < 0.0) {
    double sc = sqrt(-c);
    return n / sc * atan2(sc * S3, X);
  }
  return n * S3 / X;
}

// pi_add_term with q = sqrt|c| and qn = n / (2 q) (c > 0) or n / q (c < 0) taken from the
// per-ray record (the same quotients, formed once per ray).
KG_HD double pi_add_term_q(double n, double c, double q, double qn, double snu, double snv, const JacobiW& w) {
  double S3 = snu * snv * w.sn;
  double X = 1.0 - n * (w.sn * w.sn) + n * snu * snv * w.cn * w.dn;
  double iX = rcp_fast(X);
  double t = S3 * iX;
  double z2 = c * (t * t);
  if ((X > 0.0 || c > 0.0) && fabs(z2) < 2.0e-3) return n * t * rc_one(-z2);
  if (c > 0.0) {
    double qs = q * S3;
    return qn * log(fabs((X + qs) / (X - qs)));
  }
  if (c < 0.0) return qn * atan2(q * S3, X);
  return n * t;
}

// ---- theta -----------------------------------------------------------------

struct ThetaState {
  double sn, cn, dn;  // Jacobi functions of snarg for the (negative) parameter kk
  double e;           // (E - F)(Phi | kk) for ordinary motion, E(Phi | kk) for vortical
  double pi;          // Pi(n; Phi | kk)
  double Phi;         // amplitude (direct evaluations only)
};

struct ThetaOut {
  double th, Gph, Gt;
};

// Direct evaluation at snarg (kgeo/kerr_raytracing_ana.py:254-277, 330-352): the amplitude
// Phi = am(snarg | kk) via the m = kk / (kk - 1) transform, the half period reduced.
template <class FV>
KG_HD ThetaState theta_state_direct(const FV& f, int code, double snarg) {
  const double m = f[T_M], s1m = f[T_S1M], n = f[T_N], kk = f[T_KK];
  double x = snarg / s1m;
  double v;
  double nr = reduce_half_period(x, f[T_K2], &v);
  Jacobi J = jacobi_landen(v, m);
  double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
  double ys = s1m * J.sn;  // sin(phi0) * dn(v | m)
  ThetaState st;
  st.Phi = nr * PI + atan2(ys, J.cn);
  double idn = 1.0 / J.dn;
  st.sn = odd * ys * idn;
  st.cn = odd * J.cn * idn;
  st.dn = idn;
  // Carlson at (cos^2 phi0, 1 - kk sin^2 phi0, 1) scaled by dn^2: (cn^2, 1, dn^2)
  double xc = J.cn * J.cn, zc = J.dn * J.dn;
  double rho = zc - n * (ys * ys);
  double rj, rd, rf;
  carlson_set<1>(xc, 1.0, zc, &rho, &rj, &rd, &rf);
  double ys3 = ys * ys * ys;
  st.pi = pi_assemble(n, st.Phi, nr, ys * rf + (n / 3.0) * ys3 * rj, f[T_PIC], kk);
  if (code_th(code) == TH_ORD) {
    double emf = -(kk / 3.0) * ys3 * rd;  // (E - F)(phi0 | kk)
    if (nr != 0.0) emf += 2.0 * nr * (f[T_EC] - f[T_KC]);
    st.e = emf;
  } else {
    double E = ys * rf - (kk / 3.0) * ys3 * rd;
    if (nr != 0.0) E += 2.0 * nr * f[T_EC];
    st.e = E;
  }
  return st;
}

template <class FV>
KG_HD double theta_snarg(const FV& f, double tau) {
  return f[T_SCALE] * (-tau + f[F_S] * f[T_GTH]);
}

// The theta state at tau = 0 (the observer) from the record: what theta_state_direct gives at
// theta_snarg(f, 0), from the setup's integrals at the observer's amplitude.
template <class FV>
KG_HD ThetaState theta_state_seed(const FV& f) {
  ThetaState st;
  st.sn = f[T_SN0];
  st.cn = f[T_CN0];
  st.dn = f[T_DN0];
  st.e = f[T_E0];
  st.pi = f[T_PI0];
  st.Phi = atan2(st.sn, st.cn);
  return st;
}

// theta, G_phi, G_t from the state (kgeo/kerr_raytracing_ana.py:280-296, 355-363).
template <class FV>
KG_HD ThetaOut theta_assemble(const FV& f, int code, const ThetaState& st) {
  ThetaOut out;
  const double s = f[F_S];
  out.Gph = f[T_PREF] * st.pi - s * f[T_GPH];
  if (code_th(code) == TH_ORD) {
    out.th = acos(f[T_NSQUP] * st.sn);
    double gt;
    if (code_kk0(code)) gt = -2 * f[T_UP] * f[T_PREF] * 0.125 * (-2 * st.Phi + sin(2 * st.Phi));
    else gt = f[T_GTC] * st.e;
    out.Gt = gt - s * f[T_GT];
  } else {
    const double up = f[T_UP], um = f[T_UM];
    out.th = acos(f[T_H] * sqrt(um + (up - um) * (st.sn * st.sn)));
    out.Gt = f[T_PREFC] * st.e - s * f[T_GT];
  }
  return out;
}

// One step snarg -> snarg - dth (the next sample of the even Mino grid).
// Returns false (state untouched) when the step passes too close to a pole of Pi.
template <class FV>
KG_HD bool theta_step(const FV& f, ThetaState* st) {
  const double kk = f[T_KK], n = f[T_N];
  const double snv = -f[S_TSN], cnv = f[S_TCN], dnv = f[S_TDN];
  const double q[4] = {f[S_TJ0], f[S_TJ1], f[S_TJ2], f[S_TJ3]};
  JacobiW w = jacobi_add_q(st->sn, st->cn, st->dn, snv, cnv, dnv, q);
  double S3 = st->sn * snv * w.sn;
  if (near_pi_pole(n, st->sn, POLE_RHO_PI) || near_pi_pole(n, w.sn, POLE_RHO_PI)) return false;
  double pi = st->pi - f[S_TPI] + pi_add_term_q(n, f[S_TC], f[S_TQ], f[S_TQN], st->sn, snv, w);
  st->e = st->e - f[S_TE] - kk * S3;
  st->pi = pi;
  st->sn = w.sn;
  st->cn = w.cn;
  st->dn = w.dn;
  return true;
}

// ---- r ---------------------------------------------------------------------

struct RadialState {
  double X;           // Jacobi argument (F(am X | k) = X)
  double sn, cn, dn;  // of X
  double E;           // E(am X | k)
  double P[3];        // Pi(n_i; am X | k)
  double am;          // amplitude (direct evaluations only)
  int k = 0;          // recurrence steps since sn, cn, dn were last evaluated directly
};

struct RadialOut {
  double r, Ip, Im, I1, I2;
};

template <class FV>
KG_HD double radial_X(const FV& f, double tau) {
  return f[R_XS] * (-tau + f[R_IRO]);
}

// The radial state at tau = 0 (X = radial_X(f, 0)) from the record, as theta_state_seed.
template <class FV>
KG_HD RadialState radial_state_seed(const FV& f, double X) {
  RadialState st;
  st.X = X;
  st.sn = f[R_SN0];
  st.cn = f[R_CN0];
  st.dn = f[R_DN0];
  st.E = f[R_E0];
  st.P[0] = f[R_PA0];
  st.P[1] = f[R_PA1];
  st.P[2] = f[R_PA2];
  st.am = atan2(st.sn, st.cn);
  return st;
}

// Direct evaluation at X (kgeo/kerr_raytracing_ana.py:434-440, 510-515, 584-591 and the
// elliptic integrals of S1_S2 / R1_R2 / case 2 at am X).
template <class FV>
KG_HD RadialState radial_state_direct(const FV& f, int code, double X, bool want_integrals) {
  RadialState st;
  st.X = X;
  double v;
  double nr = reduce_half_period(X, f[R_K2], &v);
  const double k = f[R_M];
  Jacobi J = jacobi_landen(v, k);
  double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
  st.sn = odd * J.sn;
  st.cn = odd * J.cn;
  st.dn = J.dn;
  st.am = nr * PI + atan2(J.sn, J.cn);
  st.E = 0.0;
  st.P[0] = st.P[1] = st.P[2] = 0.0;
  if (!want_integrals) return st;
  double s2r = J.sn * J.sn;
  double rho[3] = {1.0 - f[R_N0] * s2r, 1.0 - f[R_N1] * s2r, 1.0 - f[R_N2] * s2r};
  double rj[3], rd, rf;
  carlson_set<3>(J.cn * J.cn, J.dn * J.dn, 1.0, rho, rj, &rd, &rf);
  double sn3 = J.sn * J.sn * J.sn;
  double Finc = J.sn * rf;
  double Einc = Finc - (k / 3.0) * sn3 * rd;
  st.E = nr == 0.0 ? Einc : Einc + 2.0 * nr * f[R_EC];
  const double nn[3] = {f[R_N0], f[R_N1], f[R_N2]};
  const double pic[3] = {f[R_PIC0], f[R_PIC1], f[R_PIC2]};
#pragma unroll
  for (int i = 0; i < 3; ++i) st.P[i] = pi_assemble(nn[i], st.am, nr, Finc + (nn[i] / 3.0) * sn3 * rj[i], pic[i], k);
  return st;
}

// One step X -> X - dX. Returns false (state untouched) when the step passes too close to a
// pole of one of the Pi's.
template <class FV>
KG_HD bool radial_step(const FV& f, RadialState* st, double Xnew) {
  const double k = f[R_M];
  const double snv = -f[S_RSN], cnv = f[S_RCN], dnv = f[S_RDN];
  const double q[4] = {f[S_RJ0], f[S_RJ1], f[S_RJ2], f[S_RJ3]};
  JacobiW w = jacobi_add_q(st->sn, st->cn, st->dn, snv, cnv, dnv, q);
  const double nn[3] = {f[R_N0], f[R_N1], f[R_N2]};
  // characteristics whose pole is within the Pi zone of the previous sample or this one
  const double zone = pi_zone(st->k + 1);
  bool pole[3];
  int npole = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    pole[i] = near_pi_pole(nn[i], st->sn, zone) || near_pi_pole(nn[i], w.sn, zone);
    npole += pole[i] ? 1 : 0;
  }
  if (npole > 1) return false;
  // next to the pole of the r formula or of a Pi: fresh sn, cn, dn at the new argument
  int nr = 0;
  double Jsn = 0.0, am = 0.0;
  bool fresh = false;
  if (npole == 1 || near_pi_pole(nn[0], st->sn, POLE_RHO_R) || near_pi_pole(nn[0], w.sn, POLE_RHO_R)) {
    fresh = true;
    double v;
    nr = (int)reduce_half_period(Xnew, f[R_K2], &v);
    const Jacobi J = jacobi_landen(v, k);
    const double odd = (nr & 1) ? -1.0 : 1.0;
    w.sn = odd * J.sn;
    w.cn = odd * J.cn;
    w.dn = J.dn;
    Jsn = J.sn;
    am = nr * PI + atan2(J.sn, J.cn);
  }
  double S3 = st->sn * snv * w.sn;
  double pnew[3];
  const double sp[3] = {f[S_RP0], f[S_RP1], f[S_RP2]};
  const double sc[3] = {f[S_RC0], f[S_RC1], f[S_RC2]};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (pole[i]) {
      // that Pi directly at the new amplitude (one Carlson set: R_F, R_D and its R_J)
      const double rho = 1.0 - nn[i] * (Jsn * Jsn);
      double rj, rd, rf;
      carlson_set<1>(w.cn * w.cn, w.dn * w.dn, 1.0, &rho, &rj, &rd, &rf);
      const double pic = i == 0 ? f[R_PIC0] : (i == 1 ? f[R_PIC1] : f[R_PIC2]);
      pnew[i] = pi_assemble(nn[i], am, (double)nr, Jsn * rf + (nn[i] / 3.0) * (Jsn * Jsn * Jsn) * rj, pic, k);
    } else {
      pnew[i] = st->P[i] - sp[i] + pi_add_term_q(nn[i], sc[i], f[S_RQ0 + i], f[S_RQN0 + i], st->sn, snv, w);
    }
  }
  double p0 = pnew[0], p1 = pnew[1], p2 = pnew[2];
  st->E = st->E - f[S_RE] - k * S3;
  st->P[0] = p0;
  st->P[1] = p1;
  st->P[2] = p2;
  st->sn = w.sn;
  st->cn = w.cn;
  st->dn = w.dn;
  st->X = Xnew;
  st->k = fresh ? 0 : st->k + 1;
  return true;
}

// r, I_+, I_-, I_1, I_2 from the state (kgeo/kerr_raytracing_ana.py:441-471, 516-552, 592-624).
template <class FV>
KG_HD RadialOut radial_assemble(const FV& f, int code, double tau, const RadialState& st, bool want_phi_t) {
  RadialOut o{0.0, 0.0, 0.0, 0.0, 0.0};
  const int rc = code_rcase(code);
  const double k = f[R_M];
  const double snX = st.sn, cnX = st.cn, dnX = st.dn;
  if (rc == RCASE_2) {
    const double rr1 = f[R_C0], rr2 = f[R_C1], rr3 = f[R_C2], rr4 = f[R_C3];
    const double rr31 = f[R_C16], rr41 = f[R_C17], rr43 = f[R_C18];
    (void)rr1;
    (void)rr2;
    double sn2 = snX * snX;
    double rs = (rr4 * rr31 - rr3 * rr41 * sn2) / (rr31 - rr41 * sn2);
    o.r = rs;
    if (!want_phi_t) return o;
    double dX = -f[R_XS];
    double dsn2 = 2 * snX * cnX * dnX * dX;
    double den = rr31 - rr41 * sn2;
    // H = (dr/dX) / (r - r3) - C8 with dr/dX = -rr31 rr43 rr41 dsn2 / den^2 and
    // r - r3 = rr31 rr43 / den: the quotient is -rr41 dsn2 / den (no cancellation in r - r3)
    double H = -(rr41 * dsn2) / den - f[R_C8];
    double Eterm = f[R_C12] * (st.E - f[R_C4]);
    double Pi_1 = f[R_C9] * (st.P[0] - f[R_C5]);
    double Pi_p = f[R_C10] * (st.P[1] - f[R_C6]);
    double Pi_m = f[R_C11] * (st.P[2] - f[R_C7]);
    o.I1 = rr3 * (-tau) + rr43 * Pi_1;
    o.I2 = H - f[R_C15] * (-tau) - Eterm;
    o.Ip = tau * f[R_C20] - Pi_p;
    o.Im = tau * f[R_C21] - Pi_m;
    return o;
  }
  if (rc == RCASE_3) {
    const double AA = f[R_C0], BB = f[R_C1], rr1 = f[R_C2], rr2 = f[R_C3];
    o.r = ((BB * rr2 - AA * rr1) + (BB * rr2 + AA * rr1) * cnX) / ((BB - AA) + (BB + AA) * cnX);
    if (!want_phi_t) return o;
    const double al[3] = {f[R_C4], f[R_C5], f[R_C6]};
    const double nn[3] = {f[R_N0], f[R_N1], f[R_N2]};
    double R1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double a_ = al[i];
      double al2 = a_ * a_;
      double p1 = f[R_C18 + i];
      double f1 = 0.5 * p1 * log(fabs((p1 * dnX + snX) / (p1 * dnX - snX)));
      R1[i] = (st.P[i] - a_ * f1) * f[R_D0 + i];
      (void)nn;
      (void)al2;
    }
    double R2 = (st.X - f[R_D3] * (st.E - al[0] * snX * dnX / (1 + al[0] * cnX))) * f[R_D4];
    R2 = R2 + f[R_D5] * R1[0];
    const bool use_m = !code_minspin(code);
    double R1m = use_m ? R1[2] : 0.0;
    double R1bm = use_m ? f[R_C10] : 0.0;
    double c0 = f[R_C11];
    double Pi_1 = c0 * (R1[0] - f[R_C7]);
    double Pi_2 = (c0 * c0) * (R2 - f[R_C8]);
    double Pi_p = f[R_C12] * (R1[1] - f[R_C9]);
    double Pi_m = f[R_C13] * (R1m - R1bm);
    double pr = f[R_C14];
    o.I1 = pr * (-tau) + Pi_1;
    o.I2 = (pr * pr) * (-tau) + 2 * pr * Pi_1 + f[R_C15] * Pi_2;
    o.Ip = -((BB + AA) * (-tau) + Pi_p) * f[R_D6];
    o.Im = -((BB + AA) * (-tau) + Pi_m) * f[R_D7];
    return o;
  }
  if (rc == RCASE_4) {
    const double a2i = f[R_C0], b1 = f[R_C1], g0 = f[R_C2];
    double sc = snX / cnX;
    o.r = -a2i * (g0 - sc) / (1 + g0 * sc) - b1;
    if (!want_phi_t) return o;
    const double gs[3] = {g0, f[R_C3], f[R_C4]};
    double S1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double al = gs[i];
      double al2 = al * al;
      double al2p1 = 1 + al2;
      double p2 = f[R_C20 + i];
      double f2 = 0.5 * p2 * log(fabs(((1 - p2) * (1 + p2 * dnX)) / ((1 + p2) * (1 - p2 * dnX))));
      S1[i] = (st.X + al2 * st.P[i] - al * f2) * f[R_D0 + i];
      (void)al2p1;
    }
    double al2 = g0 * g0;
    double S2a = (1 - k) * st.X + al2 * st.E + al2 * dnX * (g0 - sc) / (1 + g0 * sc) - al2 * g0;
    S2a = S2a * f[R_C23];
    double S2b = S1[0] * f[R_C24];
    double S2 = S2a + S2b;
    double Pi_1 = f[R_C9] * (S1[0] - f[R_C5]);
    double Pi_2 = f[R_C10] * (S2 - f[R_C6]);
    double Pi_p = f[R_C11] * (S1[1] - f[R_C7]);
    double Pi_m = f[R_C12] * (S1[2] - f[R_C8]);
    double aa1 = f[R_C13];
    o.I1 = aa1 * (-tau) - Pi_1;
    o.I2 = (aa1 * aa1) * (-tau) - 2 * aa1 * Pi_1 + Pi_2;
    o.Ip = f[R_C14] * (-tau - Pi_p);
    o.Im = f[R_C15] * (-tau - Pi_m);
    return o;
  }
  return o;
}

// ---- combination -------------------------------------------------------------

// t, phi, sigma from the theta and r parts (kgeo/kerr_raytracing_ana.py:186-188, 626-633).
template <class FV>
KG_HD Sample combine(const Observer& ob, const FV& f, double tau, const ThetaOut& T, const RadialOut& R) {
  const double lam = f[F_LAM];
  double I_0 = -tau;
  double I_phi = f[F_CP] * R.Ip - f[F_CM] * R.Im;
  double I_tA = f[F_TP] * R.Ip - f[F_TM] * R.Im;
  double I_t = I_tA + 4 * I_0 + 2 * R.I1 + R.I2;
  Sample S;
  S.sig = 0 + R.I2 + ob.a2 * T.Gt;
  S.t = 0 + I_t + ob.a2 * T.Gt;
  S.ph = 0 + I_phi + lam * T.Gph;
  S.r = R.r;
  S.th = T.th;
  return S;
}

template <class FV>
KG_HD bool theta_active(const FV& f, int code, bool ordinary_active) {
  int th = code_th(code);
  return th == TH_VORT || (th == TH_ORD && ordinary_active);
}

// Direct evaluation of the theta part at tau (zeros where the reference leaves them zero).
template <class FV>
KG_HD ThetaOut sample_theta(const FV& f, int code, double tau, bool ordinary_active) {
  if (!theta_active(f, code, ordinary_active)) return ThetaOut{0.0, 0.0, 0.0};
  ThetaState st = theta_state_direct(f, code, theta_snarg(f, tau));
  return theta_assemble(f, code, st);
}

template <class FV>
KG_HD RadialOut sample_radial(const FV& f, int code, double tau, bool want_phi_t) {
  if (code_rcase(code) == RCASE_NONE) return RadialOut{0.0, 0.0, 0.0, 0.0, 0.0};
  RadialState st = radial_state_direct(f, code, radial_X(f, tau), want_phi_t);
  return radial_assemble(f, code, tau, st, want_phi_t);
}

// Element g of numpy.linspace(0, stop, G) for an array stop (numpy's arithmetic:
// g * (stop / (G - 1)), or (g / (G - 1)) * stop when any step of the array is zero,
// then + start, and the last element set to stop exactly).
KG_HD double linspace_at(int64_t g, int64_t G, double stop, bool any_step_zero) {
  if (G == 1) return 0.0 * stop + 0.0;
  if (g == G - 1) return stop;
  double div = (double)(G - 1);
  if (any_step_zero) return ((double)g / div) * stop + 0.0;
  return (double)g * (stop / div) + 0.0;
}

// The even grid with its step computed once (same arithmetic as linspace_at).
struct EvenGrid {
  double stop, step, div;
  int64_t G;
  bool step_zero;
  KG_HD EvenGrid(double stop_, int64_t G_, bool step_zero_)
      : stop(stop_), step(G_ > 1 ? stop_ / (double)(G_ - 1) : 0.0), div((double)(G_ - 1)), G(G_),
        step_zero(step_zero_) {}
  KG_HD double at(int64_t g) const {
    if (G == 1) return 0.0 * stop + 0.0;
    if (g == G - 1) return stop;
    if (step_zero) return ((double)g / div) * stop + 0.0;
    return (double)g * step + 0.0;
  }
};

// All five coordinates at Mino time tau by direct evaluation.
template <class FV>
KG_HD Sample sample_all(const Observer& ob, const FV& f, int code, double tau, bool ordinary_active) {
  ThetaOut T = sample_theta(f, code, tau, ordinary_active);
  RadialOut R = sample_radial(f, code, tau, true);
  return combine(ob, f, tau, T, R);
}

// Samples g0 .. g1-1 of one ray on the even Mino grid (G samples, last one = taumax):
// a direct evaluation at g0 and at the final sample, the addition-theorem recurrence in
// between (direct everywhere for rays without CODE_STEP). emit(g, tau, Sample) stores.
template <class FV, class Emit>
KG_HD void ray_chunk(const Observer& ob, const FV& f, int code, int64_t g0, int64_t g1, int64_t G,
                     bool ordinary_active, bool step_zero, Emit emit) {
  const EvenGrid grid(f[F_TAUMAX], G, step_zero);
  const bool thact = theta_active(f, code, ordinary_active);
  const bool stepping = code_step(code);
  const bool rdo = code_rcase(code) != RCASE_NONE;
  ThetaState ts;
  RadialState rs;
  ts.sn = ts.cn = ts.dn = ts.e = ts.pi = ts.Phi = 0.0;
  rs.X = rs.sn = rs.cn = rs.dn = rs.E = rs.am = 0.0;
  rs.P[0] = rs.P[1] = rs.P[2] = 0.0;
  // a ray that ends at the horizon (radial cases 3 and 4, case 2 with r3 inside the horizon):
  // its last sample, 1e-10 tau_tot before the horizon, is evaluated directly; an escaping ray's
  // last sample is back at r_o and takes its step (the zone of the r formula's pole refreshes
  // sn, cn, dn there)
  const bool captured = code_rcase(code) != RCASE_2 || f[R_C2] < ob.rplus;
  for (int64_t g = g0; g < g1; ++g) {
    const double tau = grid.at(g);
    const double X = radial_X(f, tau);
    if (g == 0 && G > 1 && stepping && tau == 0.0) {
      // the observer: the setup's states
      if (thact) ts = theta_state_seed(f);
      if (rdo) rs = radial_state_seed(f, X);
    } else if (g == g0 || (g == G - 1 && captured) || !stepping) {
      if (thact) ts = theta_state_direct(f, code, theta_snarg(f, tau));
      if (rdo) rs = radial_state_direct(f, code, X, true);
    } else {
      if (thact && !theta_step(f, &ts)) ts = theta_state_direct(f, code, theta_snarg(f, tau));
      if (rdo && !radial_step(f, &rs, X)) rs = radial_state_direct(f, code, X, true);
    }
    ThetaOut T = thact ? theta_assemble(f, code, ts) : ThetaOut{0.0, 0.0, 0.0};
    RadialOut R = rdo ? radial_assemble(f, code, tau, rs, true) : RadialOut{0.0, 0.0, 0.0, 0.0, 0.0};
    emit(g, tau, combine(ob, f, tau, T, R));
  }
}

// ---- theta and r only ----------------------------------------------------------

// sn, cn, dn of the theta amplitude at snarg (the Jacobi part of theta_state_direct).
template <class FV>
KG_HD ThetaState theta_sncd_direct(const FV& f, double snarg) {
  double v;
  const double nr = reduce_half_period(snarg / f[T_S1M], f[T_K2], &v);
  const Jacobi J = jacobi_landen(v, f[T_M]);
  const double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
  const double idn = 1.0 / J.dn;
  ThetaState st;
  st.sn = odd * (f[T_S1M] * J.sn) * idn;
  st.cn = odd * J.cn * idn;
  st.dn = idn;
  st.e = st.pi = st.Phi = 0.0;
  return st;
}

// theta from sn (theta_assemble's first line for each branch).
template <class FV>
KG_HD double theta_of_sn(const FV& f, int code, double sn) {
  const double up = f[T_UP];
  if (code_th(code) == TH_ORD) return acos(-f[F_S] * sqrt(up) * sn);
  const double um = f[T_UM];
  return acos(f[T_H] * sqrt(um + (up - um) * (sn * sn)));
}

// One radial step of sn, cn, dn alone; fresh Jacobi functions next to the pole of the r
// formula (the n0 characteristic), as radial_step does.
template <class FV>
KG_HD void radial_sncd_step(const FV& f, RadialState* st, double Xnew) {
  const double k = f[R_M];
  const double q[4] = {f[S_RJ0], f[S_RJ1], f[S_RJ2], f[S_RJ3]};
  JacobiW w = jacobi_add_q(st->sn, st->cn, st->dn, -f[S_RSN], f[S_RCN], f[S_RDN], q);
  if (near_pi_pole(f[R_N0], st->sn, POLE_RHO_R) || near_pi_pole(f[R_N0], w.sn, POLE_RHO_R)) {
    double v;
    const int nr = (int)reduce_half_period(Xnew, f[R_K2], &v);
    const Jacobi J = jacobi_landen(v, k);
    const double odd = (nr & 1) ? -1.0 : 1.0;
    w.sn = odd * J.sn;
    w.cn = odd * J.cn;
    w.dn = J.dn;
  }
  st->sn = w.sn;
  st->cn = w.cn;
  st->dn = w.dn;
  st->X = Xnew;
}

// Samples g0 .. g1-1 of theta and r alone (t, phi and sigma not requested): ray_chunk's grid,
// chunk starts and addition-theorem steps on the Jacobi functions only, with no E or Pi (and
// so none of their pole re-seeds). emit(g, tau, r, theta) stores.
template <class FV, class Emit>
KG_HD void ray_chunk_rth(const FV& f, int code, int64_t g0, int64_t g1, int64_t G, bool ordinary_active,
                         bool step_zero, Emit emit) {
  const EvenGrid grid(f[F_TAUMAX], G, step_zero);
  const bool thact = theta_active(f, code, ordinary_active);
  const bool stepping = code_step(code);
  const bool rdo = code_rcase(code) != RCASE_NONE;
  ThetaState ts;
  RadialState rs;
  ts.sn = ts.cn = ts.dn = ts.e = ts.pi = ts.Phi = 0.0;
  rs.X = rs.sn = rs.cn = rs.dn = rs.E = rs.am = 0.0;
  rs.P[0] = rs.P[1] = rs.P[2] = 0.0;
  for (int64_t g = g0; g < g1; ++g) {
    const double tau = grid.at(g);
    const double X = radial_X(f, tau);
    if (g == 0 && G > 1 && stepping && tau == 0.0) {
      if (thact) ts = theta_state_seed(f);
      if (rdo) rs = radial_state_seed(f, X);
    } else if (g == g0 || g == G - 1 || !stepping) {
      if (thact) ts = theta_sncd_direct(f, theta_snarg(f, tau));
      if (rdo) rs = radial_state_direct(f, code, X, false);
    } else {
      if (thact) {
        const double q[4] = {f[S_TJ0], f[S_TJ1], f[S_TJ2], f[S_TJ3]};
        const JacobiW w = jacobi_add_q(ts.sn, ts.cn, ts.dn, -f[S_TSN], f[S_TCN], f[S_TDN], q);
        ts.sn = w.sn;
        ts.cn = w.cn;
        ts.dn = w.dn;
      }
      if (rdo) radial_sncd_step(f, &rs, X);
    }
    const double th = thact ? theta_of_sn(f, code, ts.sn) : 0.0;
    const double r = rdo ? radial_assemble(f, code, tau, rs, false).r : 0.0;
    emit(g, tau, r, th);
  }
}

struct GainArgs {
  double a, rp, rm, r_o;
};

template <class FV>
KG_HD GainArgs ob_gain_args(const FV& f) {
  return GainArgs{f[G_A], f[G_RP], f[G_RM], f[G_RO]};
}

// Amplification of an absolute error in each elliptic integral into phi and into t / r_o,
// following the combinations of radial_assemble / theta_assemble / combine. gain[0]: theta Pi,
// gain[1..3]: r Pi_0..2, gain[4]: r E.
template <class FV>
KG_HD void mixed_gains(const GainArgs& g, const FV& f, int code, double* gain) {
  const double lam = f[F_LAM];
  const double tsc = 1.0 / (g.r_o > 0 && g.r_o < 1e300 ? g.r_o : 1.0);
  const double cphi_p = fabs(2 * g.a / (g.rp - g.rm) * (g.rp - 0.5 * g.a * lam));
  const double cphi_m = fabs(2 * g.a / (g.rp - g.rm) * (g.rm - 0.5 * g.a * lam));
  const double ct_p = fabs(4 / (g.rp - g.rm) * (g.rp * g.rp - 0.5 * g.a * lam * g.rp)) * tsc;
  const double ct_m = fabs(4 / (g.rp - g.rm) * (g.rm * g.rm - 0.5 * g.a * lam * g.rm)) * tsc;
  const double wp = fmax(cphi_p, ct_p), wm = fmax(cphi_m, ct_m);
  gain[0] = fabs(lam * f[T_PREF]);
  gain[1] = gain[2] = gain[3] = gain[4] = 0.0;
  const int rc = code_rcase(code);
  const double k = f[R_M];
  if (rc == RCASE_2) {
    gain[1] = fabs(f[R_C9] * f[R_C18]) * 3 * tsc;
    gain[2] = fabs(f[R_C10]) * wp;
    gain[3] = fabs(f[R_C11]) * wm;
    gain[4] = fabs(f[R_C12]) * tsc;
  } else if (rc == RCASE_3) {
    const double al0 = f[R_C4], alp = f[R_C5], alm = f[R_C6];
    const double c0 = f[R_C11], pr = f[R_C14], sAB = f[R_C15];
    const double a02 = al0 * al0, jd = k + (1 - k) * a02;
    const double r2f = fabs(sAB * c0 * c0);
    gain[1] = fabs(c0 / (1 - a02)) * (3 + 2 * fabs(pr) + r2f * fabs((2 * k - f[R_N0]) / jd)) * tsc;
    gain[2] = fabs(f[R_C12] / ((1 - alp * alp) * f[R_C16])) * wp;
    gain[3] = code_minspin(code) ? 0.0 : fabs(f[R_C13] / ((1 - alm * alm) * f[R_C17])) * wm;
    gain[4] = r2f * fabs(a02 / (jd * (a02 - 1))) * tsc;
  } else if (rc == RCASE_4) {
    const double g0 = f[R_C2], gp = f[R_C3], gm = f[R_C4];
    const double aa1 = f[R_C13];
    const double a02 = g0 * g0, a02p1 = 1 + a02, a02j = 1 - k + a02;
    const double s2w = fabs(f[R_C10] / f[R_C9]) * (1. / a02p1 + (1 - k) / a02j);
    gain[1] = (a02 / a02p1) * fabs(f[R_C9]) * (3 + 2 * fabs(aa1) + s2w) * tsc;
    gain[2] = (gp * gp / (1 + gp * gp)) * fabs(f[R_C11] * f[R_C14]) * wp;
    gain[3] = (gm * gm / (1 + gm * gm)) * fabs(f[R_C12] * f[R_C15]) * wm;
    gain[4] = fabs(f[R_C10]) * a02 / (a02p1 * a02j) * tsc;
  }
}

// Per-ray constants of one step of the even Mino grid (Mino step dtau): the Jacobi
// functions and the integrals at the step itself. Sets CODE_STEP when the ray can be
// stepped (finite constants, no n = 1 theta characteristic, not the a < MINSPIN limit).
// q, qn of pi_add_term_q for characteristic n and c = n (m - n)(1 - n).
KG_HD void pi_add_consts(double n, double c, double* q, double* qn) {
  if (c > 0.0) {
    const double sc = sqrt(c);
    *q = sc;
    *qn = n / (2.0 * sc);
  } else if (c < 0.0) {
    const double sc = sqrt(-c);
    *q = sc;
    *qn = n / sc;
  } else {
    *q = 0.0;
    *qn = n;
  }
}

template <class FV>
KG_HD int step_constants(FV f, int code, double dtau, double* out /* f itself, writable */) {
  bool ok = dtau > 0 && std::isfinite(dtau) && code_rcase(code) != RCASE_NONE && code_th(code) != TH_ZERO &&
            !code_kk0(code) && f[T_KK] >= M_NEG_INF;
  if (ok) {
    double dth = f[T_SCALE] * dtau;
    ThetaState ts = theta_state_direct(f, code, dth);
    out[S_TSN] = ts.sn;
    out[S_TCN] = ts.cn;
    out[S_TDN] = ts.dn;
    out[S_TE] = ts.e;
    out[S_TPI] = ts.pi;
    const double n = f[T_N], kk = f[T_KK];
    out[S_TC] = n * (kk - n) * (1 - n);
    double dX = f[R_XS] * dtau;
    RadialState rs = radial_state_direct(f, code, dX, true);
    out[S_RSN] = rs.sn;
    out[S_RCN] = rs.cn;
    out[S_RDN] = rs.dn;
    out[S_RE] = rs.E;
    out[S_RP0] = rs.P[0];
    out[S_RP1] = rs.P[1];
    out[S_RP2] = rs.P[2];
    const double k = f[R_M];
    const double nn[3] = {f[R_N0], f[R_N1], f[R_N2]};
    out[S_RC0] = nn[0] * (k - nn[0]) * (1 - nn[0]);
    out[S_RC1] = nn[1] * (k - nn[1]) * (1 - nn[1]);
    out[S_RC2] = nn[2] * (k - nn[2]) * (1 - nn[2]);
    jacobi_step_products(-ts.sn, ts.cn, ts.dn, kk, out + S_TJ0);
    pi_add_consts(n, out[S_TC], out + S_TQ, out + S_TQN);
    for (int i = 0; i < 3; ++i) pi_add_consts(nn[i], out[S_RC0 + i], out + S_RQ0 + i, out + S_RQN0 + i);
    jacobi_step_products(-rs.sn, rs.cn, rs.dn, k, out + S_RJ0);
    ok = n != 1.0 && std::isfinite(f[T_PIC]);
    for (int i = S_TSN; i <= S_RC2; ++i) ok = ok && std::isfinite(out[i]);
    for (int i = S_TJ0; i <= S_RJ3; ++i) ok = ok && std::isfinite(out[i]);
  }
  code = ok ? (code | CODE_STEP) : (code & ~CODE_STEP);
  // gains by which an error in each integral's increments reaches phi (scale 1) or t (scale r_o)
  double gain[5];
  mixed_gains(ob_gain_args(f), f, code, gain);
  for (int i = 0; i < 5; ++i) {
    if (!(gain[i] <= MIXED_GAIN_MAX)) code |= 1 << (CODE_F64_SHIFT + i);
    else code &= ~(1 << (CODE_F64_SHIFT + i));
  }
  return code;
}

}  // namespace kg
