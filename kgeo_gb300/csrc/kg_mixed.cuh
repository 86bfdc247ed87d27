// Mixed-precision evaluation of the even Mino grid.
//
// What stays FP64: the per-ray setup and step constants, the Jacobi state (sn, cn, dn of
// the theta and r arguments) and its addition-theorem update, r itself (near the observer r
// is conditioned like r / r_4 ~ 1e3 in sn^2), the accumulators of E and Pi, and the final
// combination into t, phi, sigma. What moves to FP32: the Pi and E increments of each step,
// the Carlson integrals of the direct evaluation at a chunk start, theta (from a
// well-conditioned atan2 of cos and sin theta), and the logarithmic terms of R1 / S1 / H.
// Samples next to a Pi pole (|1 - n sn^2| < POLE_RHO) and the final, horizon-adjacent sample
// are evaluated in full FP64.
#pragma once

#include "kg_elliptic_f32.cuh"
#include "kg_ray.cuh"

namespace kg {

KG_HD float __frcp_rn_compat(float x) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}

// Pi increment of one step in FP32 (see pi_add_term for the formula); X is formed in FP64
// by the caller (it cancels near a pole) and handed over rounded.
KG_HD float pi_add_term_f(float n, float c, float X, float S3) {
  float iX = __frcp_rn_compat(X);
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

// Below this distance rho = |1 - n sn^2| to a Pi pole a characteristic's increment and the log
// term that cancels its pole in R1 / S1 are kept in FP64 (FP32 would lose ~eps32 / rho).
constexpr double MIXED_RHO = 0.1;

KG_HD bool mixed_fp64(double n, double sn) { return n > 0.0 && fabs(1.0 - n * (sn * sn)) < MIXED_RHO; }

// X of the Pi addition term in FP64.
KG_HD double pi_add_X(double n, double snu, double snv, const JacobiW& w) {
  return 1.0 - n * (w.sn * w.sn) + n * snu * snv * w.cn * w.dn;
}

template <class FV>
KG_HD bool theta_near_pole(const FV& f, double sn) {
  return near_pi_pole(f[T_N], sn);
}

template <class FV>
KG_HD bool radial_near_pole(const FV& f, double sn) {
  return near_pi_pole(f[R_N0], sn) || near_pi_pole(f[R_N1], sn) || near_pi_pole(f[R_N2], sn);
}

// Direct theta state with FP64 Jacobi functions and FP32 integrals.
template <class FV>
KG_HD ThetaState theta_state_direct_mixed(const FV& f, int code, double snarg) {
  const double m = f[T_M], s1m = f[T_S1M], n = f[T_N], kk = f[T_KK];
  double x = snarg / s1m;
  double v;
  double nr = reduce_half_period(x, f[T_K2], &v);
  Jacobi J = jacobi_landen(v, m);
  double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
  double ys = s1m * J.sn;
  ThetaState st;
  st.Phi = 0.0;
  double idn = 1.0 / J.dn;
  st.sn = odd * ys * idn;
  st.cn = odd * J.cn * idn;
  st.dn = idn;
  float xc = (float)(J.cn * J.cn), zc = (float)(J.dn * J.dn);
  float rho = (float)((1.0 - n) * (J.dn * J.dn) + n * (J.cn * J.cn));  // (1 - n sin^2 phi0) dn^2
  float rj, rd, rf;
  carlson_set_f<1>(xc, 1.0f, zc, &rho, &rj, &rd, &rf);
  double ys3 = ys * ys * ys;
  double pi0 = ys * (double)rf + (n / 3.0) * ys3 * (double)rj;
  st.pi = nr == 0.0 ? pi0 : 2.0 * nr * f[T_PIC] + pi0;
  if (code_th(code) == TH_ORD) {
    double emf = -(kk / 3.0) * ys3 * (double)rd;
    if (nr != 0.0) emf += 2.0 * nr * (f[T_EC] - f[T_KC]);
    st.e = emf;
  } else {
    double E = ys * (double)rf - (kk / 3.0) * ys3 * (double)rd;
    if (nr != 0.0) E += 2.0 * nr * f[T_EC];
    st.e = E;
  }
  return st;
}

// Direct r state with FP64 Jacobi functions; the integrals in FP32 except those the ray's
// error budget flags (code bits), which get an FP64 Carlson evaluation of their own.
template <class FV>
KG_HD RadialState radial_state_direct_mixed(const FV& f, int code, double X) {
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
  st.am = 0.0;
  const double s2r = J.sn * J.sn, c2r = J.cn * J.cn, d2r = J.dn * J.dn;
  const double nn[3] = {f[R_N0], f[R_N1], f[R_N2]};
  double rho[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) rho[i] = nn[i] < 1.0 ? (1.0 - nn[i]) + nn[i] * c2r : 1.0 - nn[i] * s2r;
  const double sn3 = J.sn * J.sn * J.sn;
  const double pic[3] = {f[R_PIC0], f[R_PIC1], f[R_PIC2]};
  int nflag = 0, which = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (code_f64(code, 1 + i)) ++nflag, which = i;
  double P[3], E;
  if (nflag >= 2) {
    double rj[3], rd, rf;
    carlson_set<3>(c2r, d2r, 1.0, rho, rj, &rd, &rf);
    double Finc = J.sn * rf;
    E = Finc - (k / 3.0) * sn3 * rd;
#pragma unroll
    for (int i = 0; i < 3; ++i) P[i] = Finc + (nn[i] / 3.0) * sn3 * rj[i];
  } else {
    float rho32[3] = {(float)rho[0], (float)rho[1], (float)rho[2]};
    float rj[3], rd, rf;
    carlson_set_f<3>((float)c2r, (float)d2r, 1.0f, rho32, rj, &rd, &rf);
    double Finc = J.sn * (double)rf;
    E = Finc - (k / 3.0) * sn3 * (double)rd;
#pragma unroll
    for (int i = 0; i < 3; ++i) P[i] = Finc + (nn[i] / 3.0) * sn3 * (double)rj[i];
    if (nflag == 1 || code_f64(code, 4)) {
      double rj1, rd1, rf1;
      carlson_set<1>(c2r, d2r, 1.0, &rho[which], &rj1, &rd1, &rf1);
      double F64 = J.sn * rf1;
      if (nflag == 1) P[which] = F64 + (nn[which] / 3.0) * sn3 * rj1;
      if (code_f64(code, 4)) E = F64 - (k / 3.0) * sn3 * rd1;
    }
  }
  st.E = nr == 0.0 ? E : E + 2.0 * nr * f[R_EC];
#pragma unroll
  for (int i = 0; i < 3; ++i) st.P[i] = nr == 0.0 ? P[i] : 2.0 * nr * pic[i] + P[i];
  return st;
}

template <class FV>
KG_HD bool theta_step_mixed(const FV& f, int code, ThetaState* st) {
  const double kk = f[T_KK], n = f[T_N];
  const double snv = -f[S_TSN], cnv = f[S_TCN], dnv = f[S_TDN];
  JacobiW w = jacobi_add(st->sn, st->cn, st->dn, snv, cnv, dnv, kk);
  if (near_pi_pole(n, st->sn) || near_pi_pole(n, w.sn)) return false;
  float S3 = (float)st->sn * (float)snv * (float)w.sn;
  double inc = (code_f64(code, 0) || mixed_fp64(n, st->sn) || mixed_fp64(n, w.sn))
                   ? pi_add_term(n, f[S_TC], st->sn, snv, w)
                   : (double)pi_add_term_f((float)n, (float)f[S_TC], (float)pi_add_X(n, st->sn, snv, w), S3);
  st->e = st->e - f[S_TE] - (double)((float)kk * S3);
  st->pi = st->pi - f[S_TPI] + inc;
  st->sn = w.sn;
  st->cn = w.cn;
  st->dn = w.dn;
  return true;
}

template <class FV>
KG_HD bool radial_step_mixed(const FV& f, int code, RadialState* st, double Xnew) {
  const double k = f[R_M];
  const double snv = -f[S_RSN], cnv = f[S_RCN], dnv = f[S_RDN];
  JacobiW w = jacobi_add(st->sn, st->cn, st->dn, snv, cnv, dnv, k);
  const double n0 = f[R_N0], n1 = f[R_N1], n2 = f[R_N2];
  if (near_pi_pole(n0, st->sn) || near_pi_pole(n1, st->sn) || near_pi_pole(n2, st->sn) ||
      near_pi_pole(n0, w.sn) || near_pi_pole(n1, w.sn) || near_pi_pole(n2, w.sn))
    return false;
  float S3 = (float)st->sn * (float)snv * (float)w.sn;
  const double nn[3] = {n0, n1, n2};
  const double cc[3] = {f[S_RC0], f[S_RC1], f[S_RC2]};
  const double pv[3] = {f[S_RP0], f[S_RP1], f[S_RP2]};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double inc = (code_f64(code, 1 + i) || mixed_fp64(nn[i], st->sn) || mixed_fp64(nn[i], w.sn))
                     ? pi_add_term(nn[i], cc[i], st->sn, snv, w)
                     : (double)pi_add_term_f((float)nn[i], (float)cc[i], (float)pi_add_X(nn[i], st->sn, snv, w), S3);
    st->P[i] = st->P[i] - pv[i] + inc;
  }
  st->E = st->E - f[S_RE] - (code_f64(code, 4) ? k * (st->sn * snv * w.sn) : (double)((float)k * S3));
  st->sn = w.sn;
  st->cn = w.cn;
  st->dn = w.dn;
  st->X = Xnew;
  return true;
}

// theta from atan2 of its sine and cosine (no acos ill-conditioning near the turning points).
template <class FV>
KG_HD ThetaOut theta_assemble_mixed(const FV& f, int code, const ThetaState& st) {
  ThetaOut out;
  const double s = f[F_S];
  out.Gph = f[T_PREF] * st.pi - s * f[T_GPH];
  const float up = (float)f[T_UP];
  // 1 - u_+ in FP64: for observers near the pole u_+ is within 1e-4 of 1, where an FP32
  // difference would keep only a few bits of sin(theta)
  const float omu = (float)(1.0 - f[T_UP]);
  const float sn = (float)st.sn, cn = (float)st.cn;
  if (code_th(code) == TH_ORD) {
    float cth = (float)(-s) * sqrtf(up) * sn;
    float sth = sqrtf(omu + up * (cn * cn));
    out.th = (double)atan2f(sth, cth);
    out.Gt = -(2 * f[T_UP] * f[T_PREF] * st.e) / (2 * f[T_KK]) - s * f[T_GT];
  } else {
    const float um = (float)f[T_UM];
    const float upm = (float)(f[T_UP] - f[T_UM]);
    float cth = (float)f[T_H] * sqrtf(um + upm * (sn * sn));
    float sth = sqrtf(omu + upm * (cn * cn));
    out.th = (double)atan2f(sth, cth);
    out.Gt = f[T_PREFC] * st.e - s * f[T_GT];
  }
  return out;
}

// r in FP64, the remaining terms of I_+, I_-, I_1, I_2 with FP32 logarithms / ratios.
template <class FV>
KG_HD RadialOut radial_assemble_mixed(const FV& f, int code, double tau, const RadialState& st) {
  RadialOut o{0.0, 0.0, 0.0, 0.0, 0.0};
  const int rc = code_rcase(code);
  const double k = f[R_M];
  const double snX = st.sn, cnX = st.cn, dnX = st.dn;
  if (rc == RCASE_2) {
    const double rr3 = f[R_C2], rr4 = f[R_C3];
    const double rr31 = f[R_C16], rr41 = f[R_C17], rr43 = f[R_C18];
    double sn2 = snX * snX;
    double den = rr31 - rr41 * sn2;
    double rs = (rr4 * rr31 - rr3 * rr41 * sn2) / den;
    o.r = rs;
    float dX = (float)(-f[R_XS]);
    float dsn2 = 2.0f * (float)snX * (float)cnX * (float)dnX * dX;
    float dn2 = (float)den;
    float drs = -((float)(rr31 * rr43 * rr41) * dsn2 / (dn2 * dn2));
    double H = (double)(drs / (float)(rs - rr3)) - f[R_C8];
    double Eterm = f[R_C12] * (st.E - f[R_C4]);
    double Pi_1 = f[R_C9] * (st.P[0] - f[R_C5]);
    double Pi_p = f[R_C10] * (st.P[1] - f[R_C6]);
    double Pi_m = f[R_C11] * (st.P[2] - f[R_C7]);
    o.I1 = rr3 * (-tau) + rr43 * Pi_1;
    o.I2 = H - f[R_C15] * (-tau) - Eterm;
    o.Ip = tau / f[R_C13] - Pi_p;
    o.Im = tau / f[R_C14] - Pi_m;
    return o;
  }
  if (rc == RCASE_3) {
    const double AA = f[R_C0], BB = f[R_C1], rr1 = f[R_C2], rr2 = f[R_C3];
    o.r = ((BB * rr2 - AA * rr1) + (BB * rr2 + AA * rr1) * cnX) / ((BB - AA) + (BB + AA) * cnX);
    const double al[3] = {f[R_C4], f[R_C5], f[R_C6]};
    double R1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double a_ = al[i];
      double al2 = a_ * a_;
      double p1d = (i == 0) ? f[R_C18] : (i == 1 ? f[R_C19] : sqrt((al2 - 1) / (k + (1 - k) * al2)));
      double f1;
      if (code_f64(code, 1 + i) || mixed_fp64(al2 / (al2 - 1), snX)) {
        f1 = 0.5 * p1d * log(fabs((p1d * dnX + snX) / (p1d * dnX - snX)));
      } else {
        float p1 = (float)p1d, sn = (float)snX, dn = (float)dnX;
        f1 = (double)(0.5f * p1 * logf(fabsf((p1 * dn + sn) / (p1 * dn - sn))));
      }
      R1[i] = (st.P[i] - a_ * f1) / (1 - al2);
    }
    double al2 = al[0] * al[0];
    double jd = k + (1 - k) * al2;
    double nn0 = f[R_N0];
    double R2 = (st.X - (al2 / jd) * (st.E - al[0] * snX * dnX / (1 + al[0] * cnX))) / (al2 - 1);
    R2 = R2 + (2 * k - nn0) * R1[0] / jd;
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
    o.Ip = -((BB + AA) * (-tau) + Pi_p) / f[R_C16];
    o.Im = -((BB + AA) * (-tau) + Pi_m) / f[R_C17];
    return o;
  }
  if (rc == RCASE_4) {
    const double a2i = f[R_C0], b1 = f[R_C1], g0 = f[R_C2];
    double sc = snX / cnX;
    o.r = -a2i * (g0 - sc) / (1 + g0 * sc) - b1;
    const double gs[3] = {g0, f[R_C3], f[R_C4]};
    double S1[3];
    float dn = (float)dnX;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double al = gs[i];
      double al2 = al * al;
      double al2p1 = 1 + al2;
      double al2j = 1 - k + al2;
      double p2d = sqrt(al2p1 / al2j);
      double f2;
      if (code_f64(code, 1 + i) || mixed_fp64(al2p1, snX)) {
        f2 = 0.5 * p2d * log(fabs(((1 - p2d) * (1 + p2d * dnX)) / ((1 + p2d) * (1 - p2d * dnX))));
      } else {
        float p2 = (float)p2d;
        f2 = (double)(0.5f * p2 * logf(fabsf(((1.0f - p2) * (1.0f + p2 * dn)) / ((1.0f + p2) * (1.0f - p2 * dn)))));
      }
      S1[i] = (st.X + al2 * st.P[i] - al * f2) / al2p1;
    }
    double al2 = g0 * g0, al2p1 = 1 + al2, al2j = 1 - k + al2;
    double S2a = (1 - k) * st.X + al2 * st.E + al2 * dnX * (g0 - sc) / (1 + g0 * sc) - al2 * g0;
    S2a = -S2a / (al2p1 * al2j);
    double S2b = S1[0] * (1. / al2p1 + (1 - k) / al2j);
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

// Mixed-precision counterpart of ray_chunk: same sample order and outputs.
template <class FV, class Emit>
KG_HD void ray_chunk_mixed(const Observer& ob, const FV& f, int code, int64_t g0, int64_t g1, int64_t G,
                           bool ordinary_active, bool step_zero, Emit emit) {
  if (!code_step(code)) {  // rays outside the recurrence take the FP64 path
    ray_chunk(ob, f, code, g0, g1, G, ordinary_active, step_zero, emit);
    return;
  }
  const EvenGrid grid(f[F_TAUMAX], G, step_zero);
  const bool thact = theta_active(f, code, ordinary_active);
  ThetaState ts;
  RadialState rs;
  ts.sn = ts.cn = ts.dn = ts.e = ts.pi = ts.Phi = 0.0;
  rs.X = rs.sn = rs.cn = rs.dn = rs.E = rs.am = 0.0;
  rs.P[0] = rs.P[1] = rs.P[2] = 0.0;
  for (int64_t g = g0; g < g1; ++g) {
    const double tau = grid.at(g);
    const double X = radial_X(f, tau);
    bool fp64 = (g == G - 1);  // the horizon-adjacent sample
    ThetaOut T{0.0, 0.0, 0.0};
    RadialOut R;
    if (fp64) {
      if (thact) ts = theta_state_direct(f, code, theta_snarg(f, tau));
      rs = radial_state_direct(f, code, X, true);
    } else if (g == g0) {
      // chunk start: FP64 Jacobi functions; integrals in FP32 unless the error budget or a
      // nearby Pi pole asks for FP64
      if (thact) {
        ts = code_f64(code, 0) ? theta_state_direct(f, code, theta_snarg(f, tau))
                               : theta_state_direct_mixed(f, code, theta_snarg(f, tau));
        if (theta_near_pole(f, ts.sn)) ts = theta_state_direct(f, code, theta_snarg(f, tau)), fp64 = true;
      }
      rs = radial_state_direct_mixed(f, code, X);
      if (radial_near_pole(f, rs.sn)) rs = radial_state_direct(f, code, X, true), fp64 = true;
    } else {
      if (thact && !theta_step_mixed(f, code, &ts)) ts = theta_state_direct(f, code, theta_snarg(f, tau)), fp64 = true;
      if (!radial_step_mixed(f, code, &rs, X)) rs = radial_state_direct(f, code, X, true), fp64 = true;
    }
    if (fp64) {
      if (thact) T = theta_assemble(f, code, ts);
      R = radial_assemble(f, code, tau, rs, true);
    } else {
      if (thact) T = theta_assemble_mixed(f, code, ts);
      R = radial_assemble_mixed(f, code, tau, rs);
    }
    emit(g, tau, combine(ob, f, tau, T, R));
  }
}

}  // namespace kg
