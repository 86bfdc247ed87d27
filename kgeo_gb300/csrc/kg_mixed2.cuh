// Mixed-precision recurrence on the FP32 pipe: the Jacobi states, the E / Pi accumulators,
// r and the combination into t, phi, sigma are carried in float-float (kg_ff.cuh, ~48 bits),
// the Pi and E increments of a step as a float-float leading term plus an FP32 correction (or
// the FP32 atan2 / log form of kg_mixed.cuh); FP64 is left to the chunk starts (the direct
// evaluation by Landen Jacobi functions and Carlson integrals of kg_ray.cuh seeds the state),
// the samples next to a Pi pole, the increments the per-ray precision planner flags, and the
// final horizon-adjacent sample.
//
// Same sample order and outputs as ray_chunk (kg_ray.cuh); the formulas are those of
// theta_step / radial_step / theta_assemble / radial_assemble / combine, regrouped so that
// every ray constant is formed once per chunk in FP64 and held in float-float.
#pragma once

#include "kg_ff.cuh"
#include "kg_mixed.cuh"

namespace kg {

// Step constants of a Jacobi addition u -> u + v with parameter m.
struct FFJac {
  ff snv, cnv, dnv;
  ff cvdv, svdv, msvcv, msv2;  // cn_v dn_v, sn_v dn_v, m sn_v cn_v, m sn_v^2
  float m;
};

KG_HD FFJac ff_jac(double snv, double cnv, double dnv, double m) {
  FFJac J;
  J.snv = ff_from(snv);
  J.cnv = ff_from(cnv);
  J.dnv = ff_from(dnv);
  J.cvdv = ff_from(cnv * dnv);
  J.svdv = ff_from(snv * dnv);
  J.msvcv = ff_from(m * snv * cnv);
  J.msv2 = ff_from(m * snv * snv);
  J.m = (float)m;
  return J;
}

struct FFState {
  ff sn, cn, dn;
};

// DLMF 22.8.1-3 in float-float.
KG_HD FFState ff_jacobi_add(const FFState& u, const FFJac& J) {
  const ff den = ff_one_minus(ff_mul(ff_sqr(u.sn), J.msv2));
  const ff inv = ff_rcp(den);
  FFState w;
  w.sn = ff_mul(ff_add(ff_mul(u.sn, J.cvdv), ff_mul(J.snv, ff_mul(u.cn, u.dn))), inv);
  w.cn = ff_mul(ff_sub(ff_mul(u.cn, J.cnv), ff_mul(ff_mul(u.sn, u.dn), J.svdv)), inv);
  w.dn = ff_mul(ff_sub(ff_mul(u.dn, J.dnv), ff_mul(ff_mul(u.sn, u.cn), J.msvcv)), inv);
  return w;
}

KG_HD FFState ff_state(double sn, double cn, double dn) { return FFState{ff_from(sn), ff_from(cn), ff_from(dn)}; }

KG_HD JacobiW to_w(const FFState& s) { return JacobiW{ff_to_double(s.sn), ff_to_double(s.cn), ff_to_double(s.dn)}; }

// rho = 1 - n sn^2 from sn^2
KG_HD float ff_rho(float n, const ff& sn2) { return ff_one_minus(ff_mul_f(sn2, n)).hi; }

KG_HD bool rho_near_pole(float n, float rho) { return n > 0.0f && fabsf(rho) < (float)POLE_RHO; }

#if defined(__CUDA_ARCH__)
#define KG_COLD __device__ __noinline__
#else
#define KG_COLD inline
#endif

// The FP64 direct evaluations and FP64 fallbacks of the mixed recurrence run once per chunk or
// at rare samples; out of line they keep the per-step loop's code compact.
template <class FV>
KG_COLD ThetaState theta_direct_cold(FV f, int code, double snarg) { return theta_state_direct(f, code, snarg); }
template <class FV>
KG_COLD RadialState radial_direct_cold(FV f, int code, double X) { return radial_state_direct(f, code, X, true); }
template <class FV>
KG_COLD RadialState radial_sncd_cold(FV f, int code, double X) { return radial_state_direct(f, code, X, false); }
KG_COLD double pi_add_term_cold(double n, double c, double snu, double snv, JacobiW w) {
  return pi_add_term(n, c, snu, snv, w);
}
KG_COLD double log_term_cold(double ald, double pd, double sn, double dn, int rc3) {
  if (rc3) return ald * (0.5 * pd * log(fabs((pd * dn + sn) / (pd * dn - sn))));
  return ald * (0.5 * pd * log(fabs(((1 - pd) * (1 + pd * dn)) / ((1 + pd) * (1 - pd * dn)))));
}

// Constants of the radial assembly, by case (indices into FFRay::K).
enum : int {
  // case 2
  K2_N0 = 0, K2_N1, K2_D0, K2_D1, K2_RR3, K2_C8, K2_C12, K2_C4, K2_C9, K2_C5, K2_C10, K2_C6, K2_C11, K2_C7,
  K2_RR43, K2_C15, K2_IC13, K2_IC14,
  // case 3
  K3_P0 = 0, K3_P1, K3_Q0, K3_Q1, K3_I1A0, K3_I1A1, K3_I1A2, K3_AL2JD, K3_IAL2M1, K3_KN0JD, K3_C0, K3_C02, K3_C7,
  K3_C8, K3_C9, K3_C12, K3_C13, K3_R1BM, K3_PR, K3_PR2, K3_2PR, K3_C15, K3_IC16, K3_IC17,
  // case 4
  K4_A2I = 0, K4_G0, K4_B1, K4_AL2_0, K4_AL2_1, K4_AL2_2, K4_IP1_0, K4_IP1_1, K4_IP1_2, K4_1MK, K4_IS2A, K4_CS2B,
  K4_C9, K4_C5, K4_C10, K4_C6, K4_C11, K4_C7, K4_C12, K4_C8, K4_AA1, K4_AA12, K4_2AA1, K4_C14, K4_C15,
  K_COUNT = 25
};

// Everything a chunk of samples of one ray needs, in float-float / FP32.
struct FFRay {
  FFJac tj, rj;
  ff t_e, t_pi;             // theta step increments of E and Pi (subtracted)
  ff r_e, r_p[3];           // radial step increments
  ff dX;                    // radial argument step (X decreases by dX)
  float tn, tkk, tc;        // theta Pi characteristic, parameter, c
  float rn[3], rc[3], rk;
  ff tnf, tkkf, rnf[3], rkf; // the same in float-float (they multiply float-float values)
  // theta assembly
  ff pref, sgph, gtc, sgt;
  float s, squp, up, omu, um, upm, h;
  bool ord;
  // radial assembly
  ff K[K_COUNT];
  float al[3], pp[3];       // case 3: alpha_i, p1_i; case 4: g_i, p2_i
  ff alf[3];                // alpha_i / g_i in float-float (the log terms multiply them exactly)
  ff ppf[3];                // p1_i / p2_i in float-float
  ff dxsf;                  // case 2: -2 R_XS in float-float (dsn2 carries the factor 2)
  // combination
  ff cp, cm, tp, tm, a2, lam;
  ff step;                  // Mino step
  float pad;                // makes the size an odd number of 4-byte words (conflict-free
                            // shared-memory slots, one per thread)
};
static_assert(sizeof(FFRay) % 8 == 4, "FFRay slots must be an odd number of 4-byte words");

template <class FV>
KG_HD void ff_ray_consts(const Observer& ob, const FV& f, int code, double step, FFRay* c) {
  c->tj = ff_jac(-f[S_TSN], f[S_TCN], f[S_TDN], f[T_KK]);
  c->rj = ff_jac(-f[S_RSN], f[S_RCN], f[S_RDN], f[R_M]);
  c->t_e = ff_from(f[S_TE]);
  c->t_pi = ff_from(f[S_TPI]);
  c->r_e = ff_from(f[S_RE]);
  c->r_p[0] = ff_from(f[S_RP0]);
  c->r_p[1] = ff_from(f[S_RP1]);
  c->r_p[2] = ff_from(f[S_RP2]);
  c->dX = ff_from(f[R_XS] * step);
  c->tn = (float)f[T_N];
  c->tkk = (float)f[T_KK];
  c->tc = (float)f[S_TC];
  c->rn[0] = (float)f[R_N0];
  c->rn[1] = (float)f[R_N1];
  c->rn[2] = (float)f[R_N2];
  c->rc[0] = (float)f[S_RC0];
  c->rc[1] = (float)f[S_RC1];
  c->rc[2] = (float)f[S_RC2];
  c->rk = (float)f[R_M];
  c->tnf = ff_from(f[T_N]);
  c->tkkf = ff_from(f[T_KK]);
  c->rnf[0] = ff_from(f[R_N0]);
  c->rnf[1] = ff_from(f[R_N1]);
  c->rnf[2] = ff_from(f[R_N2]);
  c->rkf = ff_from(f[R_M]);
  const double s = f[F_S];
  c->s = (float)s;
  c->pref = ff_from(f[T_PREF]);
  c->sgph = ff_from(s * f[T_GPH]);
  c->sgt = ff_from(s * f[T_GT]);
  c->ord = code_th(code) == TH_ORD;
  c->up = (float)f[T_UP];
  c->omu = (float)(1.0 - f[T_UP]);
  c->squp = (float)(-s * sqrt(f[T_UP]));
  c->um = (float)f[T_UM];
  c->upm = (float)(f[T_UP] - f[T_UM]);
  c->h = (float)f[T_H];
  c->gtc = c->ord ? ff_from(-(2 * f[T_UP] * f[T_PREF]) / (2 * f[T_KK])) : ff_from(f[T_PREFC]);
  const double k = f[R_M];
  const int rc = code_rcase(code);
  for (int i = 0; i < K_COUNT; ++i) c->K[i] = ff_c(0.0f);
  c->al[0] = c->al[1] = c->al[2] = c->pp[0] = c->pp[1] = c->pp[2] = 0.0f;
  c->alf[0] = c->alf[1] = c->alf[2] = ff_c(0.0f);
  c->ppf[0] = c->ppf[1] = c->ppf[2] = ff_c(0.0f);
  c->dxsf = ff_c(0.0f);
  if (rc == RCASE_2) {
    const double rr3 = f[R_C2], rr4 = f[R_C3], rr31 = f[R_C16], rr41 = f[R_C17], rr43 = f[R_C18];
    c->K[K2_N0] = ff_from(rr4 * rr31);
    c->K[K2_N1] = ff_from(rr3 * rr41);
    c->K[K2_D0] = ff_from(rr31);
    c->K[K2_D1] = ff_from(rr41);
    c->K[K2_RR3] = ff_from(rr3);
    c->K[K2_C8] = ff_from(f[R_C8]);
    c->K[K2_C12] = ff_from(f[R_C12]);
    c->K[K2_C4] = ff_from(f[R_C4]);
    c->K[K2_C9] = ff_from(f[R_C9]);
    c->K[K2_C5] = ff_from(f[R_C5]);
    c->K[K2_C10] = ff_from(f[R_C10]);
    c->K[K2_C6] = ff_from(f[R_C6]);
    c->K[K2_C11] = ff_from(f[R_C11]);
    c->K[K2_C7] = ff_from(f[R_C7]);
    c->K[K2_RR43] = ff_from(rr43);
    c->K[K2_C15] = ff_from(f[R_C15]);
    c->K[K2_IC13] = ff_from(1.0 / f[R_C13]);
    c->K[K2_IC14] = ff_from(1.0 / f[R_C14]);
    c->dxsf = ff_from(-2.0 * f[R_XS]);
  } else if (rc == RCASE_3) {
    const double AA = f[R_C0], BB = f[R_C1], rr1 = f[R_C2], rr2 = f[R_C3];
    c->K[K3_P0] = ff_from(BB * rr2 - AA * rr1);
    c->K[K3_P1] = ff_from(BB * rr2 + AA * rr1);
    c->K[K3_Q0] = ff_from(BB - AA);
    c->K[K3_Q1] = ff_from(BB + AA);
    const double al[3] = {f[R_C4], f[R_C5], f[R_C6]};
    for (int i = 0; i < 3; ++i) {
      const double al2 = al[i] * al[i];
      c->al[i] = (float)al[i];
      c->alf[i] = ff_from(al[i]);
      const double p1d = (i == 0) ? f[R_C18] : (i == 1 ? f[R_C19] : sqrt((al2 - 1) / (k + (1 - k) * al2)));
      c->pp[i] = (float)p1d;
      c->ppf[i] = ff_from(p1d);
      c->K[K3_I1A0 + i] = ff_from(1.0 / (1 - al2));
    }
    const double al2 = al[0] * al[0], jd = k + (1 - k) * al2;
    c->K[K3_AL2JD] = ff_from(al2 / jd);
    c->K[K3_IAL2M1] = ff_from(1.0 / (al2 - 1));
    c->K[K3_KN0JD] = ff_from((2 * k - f[R_N0]) / jd);
    const double c0 = f[R_C11];
    c->K[K3_C0] = ff_from(c0);
    c->K[K3_C02] = ff_from(c0 * c0);
    c->K[K3_C7] = ff_from(f[R_C7]);
    c->K[K3_C8] = ff_from(f[R_C8]);
    c->K[K3_C9] = ff_from(f[R_C9]);
    c->K[K3_C12] = ff_from(f[R_C12]);
    c->K[K3_C13] = ff_from(f[R_C13]);
    c->K[K3_R1BM] = ff_from(code_minspin(code) ? 0.0 : f[R_C10]);
    const double pr = f[R_C14];
    c->K[K3_PR] = ff_from(pr);
    c->K[K3_PR2] = ff_from(pr * pr);
    c->K[K3_2PR] = ff_from(2 * pr);
    c->K[K3_C15] = ff_from(f[R_C15]);
    c->K[K3_IC16] = ff_from(1.0 / f[R_C16]);
    c->K[K3_IC17] = ff_from(1.0 / f[R_C17]);
  } else if (rc == RCASE_4) {
    const double a2i = f[R_C0], b1 = f[R_C1], g0 = f[R_C2];
    c->K[K4_A2I] = ff_from(a2i);
    c->K[K4_G0] = ff_from(g0);
    c->K[K4_B1] = ff_from(b1);
    const double gs[3] = {g0, f[R_C3], f[R_C4]};
    for (int i = 0; i < 3; ++i) {
      const double al2 = gs[i] * gs[i], al2p1 = 1 + al2, al2j = 1 - k + al2;
      c->al[i] = (float)gs[i];
      c->alf[i] = ff_from(gs[i]);
      const double p2d = sqrt(al2p1 / al2j);
      c->pp[i] = (float)p2d;
      c->ppf[i] = ff_from(p2d);
      c->K[K4_AL2_0 + i] = ff_from(al2);
      c->K[K4_IP1_0 + i] = ff_from(1.0 / al2p1);
    }
    const double al2 = g0 * g0, al2p1 = 1 + al2, al2j = 1 - k + al2;
    c->K[K4_1MK] = ff_from(1 - k);
    c->K[K4_IS2A] = ff_from(-1.0 / (al2p1 * al2j));
    c->K[K4_CS2B] = ff_from(1. / al2p1 + (1 - k) / al2j);
    c->K[K4_C9] = ff_from(f[R_C9]);
    c->K[K4_C5] = ff_from(f[R_C5]);
    c->K[K4_C10] = ff_from(f[R_C10]);
    c->K[K4_C6] = ff_from(f[R_C6]);
    c->K[K4_C11] = ff_from(f[R_C11]);
    c->K[K4_C7] = ff_from(f[R_C7]);
    c->K[K4_C12] = ff_from(f[R_C12]);
    c->K[K4_C8] = ff_from(f[R_C8]);
    const double aa1 = f[R_C13];
    c->K[K4_AA1] = ff_from(aa1);
    c->K[K4_AA12] = ff_from(aa1 * aa1);
    c->K[K4_2AA1] = ff_from(2 * aa1);
    c->K[K4_C14] = ff_from(f[R_C14]);
    c->K[K4_C15] = ff_from(f[R_C15]);
  }
  const double a = ob.a, rp = ob.rplus, rm = ob.rminus, lam = f[F_LAM];
  c->cp = ff_from((2 * a / (rp - rm)) * (rp - 0.5 * a * lam));
  c->cm = ff_from((2 * a / (rp - rm)) * (rm - 0.5 * a * lam));
  c->tp = ff_from((4 / (rp - rm)) * (rp * rp - 0.5 * a * lam * rp));
  c->tm = ff_from((4 / (rp - rm)) * (rm * rm - 0.5 * a * lam * rm));
  c->a2 = ff_from(ob.a2);
  c->lam = ff_from(lam);
  c->step = ff_from(step);
}

struct FFTheta {
  FFState j;
  ff e, pi;
  float rho;
};

struct FFRadial {
  FFState j;
  ff E, P[3], X;
  float rho[3];
};

KG_HD FFTheta ff_theta_from(const ThetaState& st, const ff& n) {
  FFTheta t;
  t.j = ff_state(st.sn, st.cn, st.dn);
  t.e = ff_from(st.e);
  t.pi = ff_from(st.pi);
  t.rho = ff_one_minus(ff_mul(ff_sqr(t.j.sn), n)).hi;
  return t;
}

KG_HD FFRadial ff_radial_from(const RadialState& st, const FFRay& c) {
  FFRadial r;
  r.j = ff_state(st.sn, st.cn, st.dn);
  r.E = ff_from(st.E);
  for (int i = 0; i < 3; ++i) r.P[i] = ff_from(st.P[i]);
  r.X = ff_from(st.X);
  const ff s2 = ff_sqr(r.j.sn);
  for (int i = 0; i < 3; ++i) r.rho[i] = ff_one_minus(ff_mul(s2, c.rnf[i])).hi;
  return r;
}

// R_C(1, 1 + e) - 1 = sum_{k >= 1} (-e)^k / (2k + 1) for |e| <= 1/4, to FP32 relative precision
// (16 terms: 4^-16 / 33 < 2e-11), without the leading 1 so that it keeps its own precision.
constexpr float RC_SERIES_MAX = 0.25f;
KG_HD float rc_one_m1_f(float e) {
  const float x = -e;
  float p = 1.0f / 33.0f;
#pragma unroll
  for (int j = 14; j >= 0; --j) p = fmaf(p, x, 1.0f / (float)(2 * j + 3));
  return x * p;
}

// Pi increment of one step (pi_add_term's formula) from float-float S3 and X. Where the R_C
// argument z2 = c (S3 / X)^2 is below 1/4 the increment n t R_C(1, 1 - z2), t = S3 / X, is
// formed as n t in float-float plus an FP32 correction n t (R_C - 1) (error ~1e-8 of the
// increment); otherwise the FP32 atan2 / log form, or FP64 within MIXED_RHO of a pole or where
// the planner flags the integral.
KG_HD ff pi_inc_ff(const ff& nf, float c, const ff& S3, const ff& X, float rho_u, float rho_w, bool flagged,
                   double nd, double cd, const ff& snu_f, double snv_neg, const FFState& w) {
  const float n = nf.hi;
  // n S3 sgn(X) R_C(X^2, X^2 - c S3^2) = n t R_C(1, 1 - z2) for either sign of X when c > 0
  // (the principal-value log form); for c < 0 and X < 0 the atan2 branch decides.
  if (X.hi > 0.0f || c > 0.0f) {
    const ff t = ff_div(S3, X);
    const float z2 = c * (t.hi * t.hi);
    if (fabsf(z2) < RC_SERIES_MAX) {
      const ff nt = ff_mul(t, nf);
      return ff_add_f(nt, nt.hi * rc_one_m1_f(-z2));
    }
  }
  if (flagged || fabsf(rho_u) < (float)MIXED_RHO || fabsf(rho_w) < (float)MIXED_RHO)
    return ff_from(pi_add_term_cold(nd, cd, ff_to_double(snu_f), -snv_neg, to_w(w)));
  return ff_c(pi_add_term_f(n, c, X.hi, S3.hi));
}

// Within RESEED_RHO of an elliptic-Pi pole an increment is ill-conditioned like 1/rho^2 in the
// state's rounding, so the characteristic's Pi is re-evaluated directly in FP64 from the
// float-float Jacobi state instead (Carlson R_F, R_J at the state's amplitude; the state's
// ~1e-13 error then reaches Pi as ~1e-13 / rho, the conditioning of Pi itself). The zone is
// small enough that few lanes of a warp enter it at the same step.
constexpr float RESEED_RHO = 1.0e-3f;

// Within DEEP_RHO of a pole even the FP64 Pi from the float-float state is not enough: the
// state's own ~1e-13 error reaches the sample as ~1e-13 / rho (1e-8 at the zone's edge). There
// the whole theta or radial state is re-seeded from the FP64 direct evaluation at the sample
// (Landen Jacobi functions, Carlson integrals), as the FP64 recurrence does next to a pole, so
// the error falls to the FP64 path's ~eps / rho. 4e-5 of the samples of the 2048^2-plus-band
// workload lie in the zone.
constexpr float DEEP_RHO = 1.0e-5f;

template <class FV>
KG_COLD ff radial_pi_direct(FV f, int i, FFState w, ff Xw) {
  const double X = ff_to_double(Xw);
  double v;
  const double nr = reduce_half_period(X, f[R_K2], &v);
  const double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
  const double sn = odd * ff_to_double(w.sn), cn = odd * ff_to_double(w.cn), dn = ff_to_double(w.dn);
  const double n = i == 0 ? f[R_N0] : (i == 1 ? f[R_N1] : f[R_N2]);
  const double pic = i == 0 ? f[R_PIC0] : (i == 1 ? f[R_PIC1] : f[R_PIC2]);
  const double s2 = sn * sn, x = cn * cn, y = dn * dn;
  const double rf = carlson_rf(x, y, 1.0);
  const double rj = rj_any(x, y, 1.0, 1.0 - n * s2, rf);
  const double am = nr * PI + atan2(sn, cn);
  return ff_from(pi_assemble(n, am, nr, sn * rf + (n / 3.0) * (s2 * sn) * rj, pic, f[R_M]));
}

// theta_state_direct's Pi from the float-float Jacobi state (no Landen): the reduced Jacobi
// values at parameter m follow from sn, cn, dn at parameter kk (J.dn = 1 / dn, J.cn = odd cn / dn,
// sin(phi0) dn(v|m) = odd sn / dn), the half-period count from the sample's snarg.
template <class FV>
KG_COLD ff theta_pi_direct(FV f, double tau, FFState w) {
  const double x = theta_snarg(f, tau) / f[T_S1M];
  double v;
  const double nr = reduce_half_period(x, f[T_K2], &v);
  const double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
  const double dn = ff_to_double(w.dn);
  const double idn = 1.0 / dn;
  const double Jdn = idn, Jcn = odd * ff_to_double(w.cn) * idn, ys = odd * ff_to_double(w.sn) * idn;
  const double n = f[T_N];
  const double xc = Jcn * Jcn, zc = Jdn * Jdn;
  const double rf = carlson_rf(xc, 1.0, zc);
  const double rj = rj_any(xc, 1.0, zc, zc - n * (ys * ys), rf);
  const double Phi = nr * PI + atan2(ys, Jcn);
  return ff_from(pi_assemble(n, Phi, nr, ys * rf + (n / 3.0) * (ys * ys * ys) * rj, f[T_PIC], f[T_KK]));
}

// One theta step. Unlike the FP64 recurrence it does not stop at a Pi pole: the float-float
// state carries ~48 bits, so the 1/rho amplification near a pole stays far below the mixed
// error bars, and the increments there are taken in FP64 (pi_inc_ff).
template <class FV>
KG_HD void ff_theta_step(const FV& f, const FFRay& c, int code, double tau, FFTheta* st) {
  const FFState w = ff_jacobi_add(st->j, c.tj);
  const ff rho_w = ff_one_minus(ff_mul(ff_sqr(w.sn), c.tnf));
  const ff S3 = ff_mul(ff_mul(st->j.sn, c.tj.snv), w.sn);
  const ff q = ff_mul(ff_mul(st->j.sn, c.tj.snv), ff_mul(w.cn, w.dn));
  const ff X = ff_add(rho_w, ff_mul(q, c.tnf));
  st->e = ff_sub(ff_sub(st->e, c.t_e), ff_mul(S3, c.tkkf));
  if (c.tn > 0.0f && (fabsf(st->rho) < RESEED_RHO || fabsf(rho_w.hi) < RESEED_RHO)) {
    // theta Pi from the FP64 direct evaluation at this sample
    st->pi = theta_pi_direct(f, tau, w);
  } else {
    const ff inc = pi_inc_ff(c.tnf, c.tc, S3, X, st->rho, rho_w.hi, code_f64(code, 0), f[T_N], f[S_TC],
                             st->j.sn, f[S_TSN], w);
    st->pi = ff_add(ff_sub(st->pi, c.t_pi), inc);
  }
  st->j = w;
  st->rho = rho_w.hi;
}

template <class FV>
KG_HD void ff_radial_step(const FV& f, const FFRay& c, int code, FFRadial* st) {
  const FFState w = ff_jacobi_add(st->j, c.rj);
  const ff s2 = ff_sqr(w.sn);
  ff rho_w[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) rho_w[i] = ff_one_minus(ff_mul(s2, c.rnf[i]));
  const ff uv = ff_mul(st->j.sn, c.rj.snv);
  const ff S3 = ff_mul(uv, w.sn);
  const ff q = ff_mul(uv, ff_mul(w.cn, w.dn));
  const double cd[3] = {f[S_RC0], f[S_RC1], f[S_RC2]};
  const double nd[3] = {f[R_N0], f[R_N1], f[R_N2]};
  const ff Xw = ff_sub(st->X, c.dX);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (c.rn[i] > 0.0f && (fabsf(st->rho[i]) < RESEED_RHO || fabsf(rho_w[i].hi) < RESEED_RHO)) {
      st->P[i] = radial_pi_direct(f, i, w, Xw);
    } else {
      const ff X = ff_add(rho_w[i], ff_mul(q, c.rnf[i]));
      const ff inc = pi_inc_ff(c.rnf[i], c.rc[i], S3, X, st->rho[i], rho_w[i].hi, code_f64(code, 1 + i), nd[i],
                               cd[i], st->j.sn, f[S_RSN], w);
      st->P[i] = ff_add(ff_sub(st->P[i], c.r_p[i]), inc);
    }
    st->rho[i] = rho_w[i].hi;
  }
  st->E = ff_sub(ff_sub(st->E, c.r_e), ff_mul(S3, c.rkf));
  st->X = Xw;
  st->j = w;
}

struct FFOut {
  ff Gph, Gt;     // theta parts
  float th;
  ff r, Ip, Im, I1, I2;
};

KG_HD void ff_theta_assemble(const FFRay& c, const FFTheta& st, FFOut* o) {
  o->Gph = ff_sub(ff_mul(c.pref, st.pi), c.sgph);
  o->Gt = ff_sub(ff_mul(c.gtc, st.e), c.sgt);
  const float sn = st.j.sn.hi, cn = st.j.cn.hi;
  if (c.ord) {
    const float cth = c.squp * sn;
    const float sth = sqrtf(c.omu + c.up * (cn * cn));
    o->th = atan2f(sth, cth);
  } else {
    const float cth = c.h * sqrtf(c.um + c.upm * (sn * sn));
    const float sth = sqrtf(c.omu + c.upm * (cn * cn));
    o->th = atan2f(sth, cth);
  }
}

// atanh(x) for |x| <= 1/2: the leading term x in float-float plus the FP32 series tail
// x^3 (1/3 + x^2/5 + ...) (error ~1e-9 of the value).
KG_HD ff ff_atanh_small(const ff& x) {
  const float xf = x.hi, x2 = xf * xf;
  float p = 1.0f / 27.0f;
#pragma unroll
  for (int j = 12; j >= 0; --j) p = fmaf(p, x2, 1.0f / (float)(2 * j + 3));
  return ff_add_f(x, xf * x2 * p);
}

// L(a) = ln|(1 + a) / (1 - a)| = 2 atanh(x), x = a for |a| < 1 and 1 / a for |a| > 1, in
// float-float: |x| <= 1/2 directly, 1/2 < |x| <= 0.99 by atanh(x) = atanh(x0) + atanh((x - x0) /
// (1 - x x0)) with x0 = 3/4 or 15/16 (exact in FP32; atanh(x0) as float-float constants),
// closer to 1 in FP32.
KG_HD ff ff_logratio(const ff& a) {
  ff x = fabsf(a.hi) <= 1.0f ? a : ff_rcp(a);
  const float ax = fabsf(x.hi);
  if (ax <= 0.5f) return ff_mul_f(ff_atanh_small(x), 2.0f);
  if (ax <= 0.99f) {
    const bool neg = x.hi < 0.0f;
    if (neg) x = ff_neg(x);
    const bool far = ax > 0.9f;
    const float x0 = far ? 0.9375f : 0.75f;
    const ff c0 = far ? ff{1.7169935703277588f, 3.1914815679101594e-08f} : ff{0.972955048084259f, 2.6443396805575503e-08f};
    const ff z = ff_div(ff_add_f(x, -x0), ff_one_minus(ff_mul_f(x, x0)));
    ff r = ff_add(c0, ff_atanh_small(z));
    if (neg) r = ff_neg(r);
    return ff_mul_f(r, 2.0f);
  }
  return ff_c(2.0f * atanhf(x.hi));
}

// alpha_i times the log term of R1 (case 3, f1 = p1 / 2 L(sn / (p1 dn))) or S1 (case 4,
// f2 = p2 / 2 (L(p2 dn) - L(p2))), in float-float, and in FP64 where the planner flags the
// integral, within MIXED_LOG_RHO of the pole of the Pi it cancels, or next to the log's own pole
// (0.99 < |x| < 1 / 0.99, where ff_logratio would fall back to FP32). The zone: host-build runs
// of the mixed recurrence against the oracle on six 30x30 grids (a 0.2-0.94, theta_o 17-85 deg)
// kept every output at the same fraction of its bar (phi 0.15) with a zone of 0.1, 0.05, 0.03,
// 0.02 or 0.01, and missed the phi bar by up to 4.8x with none; with 0.1 (the increments' zone,
// MIXED_RHO) 37-64 % of the log terms of case-3 and case-4 rays ran in FP64.
KG_HD bool ff_log_near_pole(const ff& x) {
  const float ax = fabsf(x.hi);
  return ax > 0.99f && ax < 1.0f / 0.99f;
}

constexpr float MIXED_LOG_RHO = 0.03f;  // 3x the smallest zone measured to keep the bars

template <class FV>
KG_HD ff ff_logterm(const FV& f, const FFRay& c, int code, int rc, int i, const FFRadial& st) {
  const bool flagged = code_f64(code, 1 + i) || fabsf(st.rho[i]) < MIXED_LOG_RHO;
  if (rc == RCASE_3) {
    const ff x = ff_div(st.j.sn, ff_mul(st.j.dn, c.ppf[i]));
    if (flagged || ff_log_near_pole(x))
      return ff_from(log_term_cold(ff_to_double(c.alf[i]), ff_to_double(c.ppf[i]), ff_to_double(st.j.sn),
                                   ff_to_double(st.j.dn), 1));
    const ff L = ff_logratio(x);
    return ff_mul(c.alf[i], ff_mul_f(ff_mul(L, c.ppf[i]), 0.5f));
  }
  // ((1 - p2)(1 + p2 dn)) / ((1 + p2)(1 - p2 dn)) = (1 + y) / (1 - y) with
  // y = p2 (dn - 1) / (1 - p2^2 dn) and dn - 1 = -k sn^2 / (1 + dn): no cancellation as dn -> 1
  const ff om = ff_div(ff_mul(c.rkf, ff_sqr(st.j.sn)), ff_add_f(st.j.dn, 1.0f));
  const ff y = ff_neg(ff_div(ff_mul(c.ppf[i], om), ff_one_minus(ff_mul(ff_sqr(c.ppf[i]), st.j.dn))));
  if (flagged || ff_log_near_pole(y))
    return ff_from(log_term_cold(ff_to_double(c.alf[i]), ff_to_double(c.ppf[i]), 0.0, ff_to_double(st.j.dn), 0));
  const ff L = ff_logratio(y);
  return ff_mul(c.alf[i], ff_mul_f(ff_mul(L, c.ppf[i]), 0.5f));
}

template <class FV>
KG_HD void ff_radial_assemble(const FV& f, const FFRay& c, int code, const ff& tau, const FFRadial& st, FFOut* o) {
  const int rc = code_rcase(code);
  const ff* K = c.K;
  const ff mtau = ff_neg(tau);
  if (rc == RCASE_2) {
    const ff sn2 = ff_sqr(st.j.sn);
    const ff den = ff_sub(K[K2_D0], ff_mul(K[K2_D1], sn2));
    const ff num = ff_sub(K[K2_N0], ff_mul(K[K2_N1], sn2));
    o->r = ff_div(num, den);
    // H = dr/dX / (r - r3) - C8 = -rr41 dsn2 / den - C8 in float-float (r - r3 = rr31 rr43 / den
    // and dr/dX = -rr31 rr43 rr41 dsn2 / den^2; near the observer dr/dX ~ r^2 is large)
    const ff dsn2 = ff_mul(ff_mul(st.j.sn, st.j.cn), ff_mul(st.j.dn, c.dxsf));
    const ff H = ff_sub(ff_neg(ff_div(ff_mul(K[K2_D1], dsn2), den)), K[K2_C8]);
    const ff Eterm = ff_mul(K[K2_C12], ff_sub(st.E, K[K2_C4]));
    const ff Pi_1 = ff_mul(K[K2_C9], ff_sub(st.P[0], K[K2_C5]));
    const ff Pi_p = ff_mul(K[K2_C10], ff_sub(st.P[1], K[K2_C6]));
    const ff Pi_m = ff_mul(K[K2_C11], ff_sub(st.P[2], K[K2_C7]));
    o->I1 = ff_add(ff_mul(K[K2_RR3], mtau), ff_mul(K[K2_RR43], Pi_1));
    o->I2 = ff_sub(ff_sub(H, ff_mul(K[K2_C15], mtau)), Eterm);
    o->Ip = ff_sub(ff_mul(tau, K[K2_IC13]), Pi_p);
    o->Im = ff_sub(ff_mul(tau, K[K2_IC14]), Pi_m);
    return;
  }
  if (rc == RCASE_3) {
    const ff cn = st.j.cn;
    o->r = ff_div(ff_add(K[K3_P0], ff_mul(K[K3_P1], cn)), ff_add(K[K3_Q0], ff_mul(K[K3_Q1], cn)));
    ff R1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) R1[i] = ff_mul(ff_sub(st.P[i], ff_logterm(f, c, code, rc, i, st)), K[K3_I1A0 + i]);
    // al0 sn dn / (1 + al0 cn): 1 + al0 cn cancels near a pole of this term, so float-float
    const ff tmp = ff_div(ff_mul(ff_mul(c.alf[0], st.j.sn), st.j.dn), ff_add_f(ff_mul(c.alf[0], st.j.cn), 1.0f));
    ff R2 = ff_mul(ff_sub(st.X, ff_mul(K[K3_AL2JD], ff_sub(st.E, tmp))), K[K3_IAL2M1]);
    R2 = ff_add(R2, ff_mul(K[K3_KN0JD], R1[0]));
    const ff R1m = code_minspin(code) ? ff_c(0.0f) : R1[2];
    const ff Pi_1 = ff_mul(K[K3_C0], ff_sub(R1[0], K[K3_C7]));
    const ff Pi_2 = ff_mul(K[K3_C02], ff_sub(R2, K[K3_C8]));
    const ff Pi_p = ff_mul(K[K3_C12], ff_sub(R1[1], K[K3_C9]));
    const ff Pi_m = ff_mul(K[K3_C13], ff_sub(R1m, K[K3_R1BM]));
    o->I1 = ff_add(ff_mul(K[K3_PR], mtau), Pi_1);
    o->I2 = ff_add(ff_add(ff_mul(K[K3_PR2], mtau), ff_mul(K[K3_2PR], Pi_1)), ff_mul(K[K3_C15], Pi_2));
    const ff bt = ff_mul(K[K3_Q1], mtau);
    o->Ip = ff_neg(ff_mul(ff_add(bt, Pi_p), K[K3_IC16]));
    o->Im = ff_neg(ff_mul(ff_add(bt, Pi_m), K[K3_IC17]));
    return;
  }
  if (rc == RCASE_4) {
    const ff sc = ff_div(st.j.sn, st.j.cn);
    const ff qv = ff_div(ff_sub(K[K4_G0], sc), ff_add_f(ff_mul(K[K4_G0], sc), 1.0f));
    o->r = ff_sub(ff_neg(ff_mul(K[K4_A2I], qv)), K[K4_B1]);
    ff S1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
      S1[i] = ff_mul(ff_sub(ff_add(st.X, ff_mul(K[K4_AL2_0 + i], st.P[i])), ff_logterm(f, c, code, rc, i, st)),
                     K[K4_IP1_0 + i]);
    const ff al2 = K[K4_AL2_0];
    ff S2a = ff_add(ff_mul(K[K4_1MK], st.X), ff_mul(al2, st.E));
    S2a = ff_add(S2a, ff_mul(al2, ff_mul(st.j.dn, qv)));
    S2a = ff_sub(S2a, ff_mul(al2, K[K4_G0]));
    S2a = ff_mul(S2a, K[K4_IS2A]);
    const ff S2 = ff_add(S2a, ff_mul(S1[0], K[K4_CS2B]));
    const ff Pi_1 = ff_mul(K[K4_C9], ff_sub(S1[0], K[K4_C5]));
    const ff Pi_2 = ff_mul(K[K4_C10], ff_sub(S2, K[K4_C6]));
    const ff Pi_p = ff_mul(K[K4_C11], ff_sub(S1[1], K[K4_C7]));
    const ff Pi_m = ff_mul(K[K4_C12], ff_sub(S1[2], K[K4_C8]));
    o->I1 = ff_sub(ff_mul(K[K4_AA1], mtau), Pi_1);
    o->I2 = ff_add(ff_sub(ff_mul(K[K4_AA12], mtau), ff_mul(K[K4_2AA1], Pi_1)), Pi_2);
    o->Ip = ff_mul(K[K4_C14], ff_sub(mtau, Pi_p));
    o->Im = ff_mul(K[K4_C15], ff_sub(mtau, Pi_m));
  }
}

// t, phi, sigma (kgeo/kerr_raytracing_ana.py:186-188, 626-633) in float-float.
KG_HD Sample ff_combine(const FFRay& c, const ff& tau, const FFOut& o) {
  const ff I_phi = ff_sub(ff_mul(c.cp, o.Ip), ff_mul(c.cm, o.Im));
  const ff I_tA = ff_sub(ff_mul(c.tp, o.Ip), ff_mul(c.tm, o.Im));
  const ff I_t = ff_add(ff_add(I_tA, ff_mul_f(tau, -4.0f)), ff_add(ff_mul_f(o.I1, 2.0f), o.I2));
  const ff a2Gt = ff_mul(c.a2, o.Gt);
  Sample S;
  S.sig = ff_to_double(ff_add(o.I2, a2Gt));
  S.t = ff_to_double(ff_add(I_t, a2Gt));
  S.ph = ff_to_double(ff_add(I_phi, ff_mul(c.lam, o.Gph)));
  S.r = ff_to_double(o.r);
  S.th = f2d_exact(o.th);
  return S;
}

// Samples g0 .. g1-1 of one ray on the even Mino grid with the float-float recurrence: an FP64
// direct evaluation seeds the chunk, every later sample is one float-float step; the final
// sample of the grid is the FP64 direct evaluation (as in ray_chunk). All lanes of a warp
// share g, so these branches do not diverge.
// cp: the thread's FFRay slot (shared memory in the kernels, so that the ~170 constants do
// not occupy registers or stack).
template <class FV, class Emit>
KG_HD void ray_chunk_ff(const Observer& ob, const FV& f, int code, int64_t g0, int64_t g1, int64_t G,
                        bool ordinary_active, bool step_zero, Emit emit, FFRay* cp) {
  const bool thact = theta_active(f, code, ordinary_active);
  if (!code_step(code) || !thact || step_zero) {
    ray_chunk(ob, f, code, g0, g1, G, ordinary_active, step_zero, emit);
    return;
  }
  const EvenGrid grid(f[F_TAUMAX], G, step_zero);
  ff_ray_consts(ob, f, code, grid.step, cp);
  const FFRay& c = *cp;
  FFTheta ts;
  FFRadial rs;
  // a ray that ends at the horizon (radial cases 3 and 4, case 2 with r3 inside the horizon);
  // an escaping ray's last sample is back at r_o, as conditioned as the others
  const bool captured = code_rcase(code) != RCASE_2 || f[R_C2] < ob.rplus;
  for (int64_t g = g0; g < g1; ++g) {
    const double tau = grid.at(g);
    if (g == G - 1 && g != g0 && captured) {
      // the horizon-adjacent last sample: r, I_+-, I_1, I_2 diverge there (condition ~1e10), so
      // the radial part is the FP64 direct evaluation; theta stays well conditioned and takes
      // its float-float step
      ff_theta_step(f, c, code, tau, &ts);
      FFOut o;
      ff_theta_assemble(c, ts, &o);
      const ThetaOut T{(double)o.th, ff_to_double(o.Gph), ff_to_double(o.Gt)};
      const RadialState r0 = radial_direct_cold(f, code, radial_X(f, tau));
      emit(g, tau, combine(ob, f, tau, T, radial_assemble(f, code, tau, r0, true)));
      continue;
    }
    if (g == g0 || (g == G - 1 && captured)) {
      // chunk start (and a last sample that starts its chunk): FP64 direct evaluation (the start
      // seeds the float-float state)
      const bool observer = g == 0 && G > 1 && tau == 0.0;
      const ThetaState t0 = observer ? theta_state_seed(f) : theta_direct_cold(f, code, theta_snarg(f, tau));
      const RadialState r0 = observer ? radial_state_seed(f, radial_X(f, tau)) : radial_direct_cold(f, code, radial_X(f, tau));
      if (g == G - 1) {
        emit(g, tau, combine(ob, f, tau, theta_assemble(f, code, t0), radial_assemble(f, code, tau, r0, true)));
        continue;
      }
      ts = ff_theta_from(t0, c.tnf);
      rs = ff_radial_from(r0, c);
    } else {
      ff_theta_step(f, c, code, tau, &ts);
      ff_radial_step(f, c, code, &rs);
      if (g == G - 1) {
        // an escaping ray's last sample, back at r_o next to the pole of the r formula: sn, cn,
        // dn from the FP64 Jacobi evaluation (the integrals keep their steps)
        const RadialState rj = radial_sncd_cold(f, code, radial_X(f, tau));
        rs.j = ff_state(rj.sn, rj.cn, rj.dn);
        const ff s2 = ff_sqr(rs.j.sn);
#pragma unroll
        for (int i = 0; i < 3; ++i) rs.rho[i] = ff_one_minus(ff_mul(s2, c.rnf[i])).hi;
      }
      if (c.tn > 0.0f && fabsf(ts.rho) < DEEP_RHO)
        ts = ff_theta_from(theta_direct_cold(f, code, theta_snarg(f, tau)), c.tnf);
      bool deep = false;
#pragma unroll
      for (int i = 0; i < 3; ++i) deep = deep || (c.rn[i] > 0.0f && fabsf(rs.rho[i]) < DEEP_RHO);
      if (deep) rs = ff_radial_from(radial_direct_cold(f, code, radial_X(f, tau)), c);
    }
    FFOut o;
    const ff tau_ff = ff_mul_f(c.step, (float)g);
    ff_theta_assemble(c, ts, &o);
    ff_radial_assemble(f, c, code, tau_ff, rs, &o);
    emit(g, tau, ff_combine(c, tau_ff, o));
  }
}

}  // namespace kg
