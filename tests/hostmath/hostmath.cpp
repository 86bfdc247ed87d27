// Host (g++) build of the device arithmetic headers, for CPU unit checks of the
// same code the CUDA kernels compile. Test-only: never loaded by the product.
#include "../../kgeo_gb300/csrc/kg_equatorial.cuh"
#include "../../kgeo_gb300/csrc/kg_image.cuh"
#include "../../kgeo_gb300/csrc/kg_polar.cuh"
#include "../../kgeo_gb300/csrc/kg_curves.cuh"
#include "../../kgeo_gb300/csrc/kg_mixed2.cuh"
#include "../../kgeo_gb300/csrc/kg_jetimg.cuh"

using namespace kg;

static Observer make_obs(const double* ob) {
  Observer o;
  o.a = ob[0]; o.a2 = ob[1]; o.r_o = ob[2]; o.th_o = ob[3]; o.sin_th = ob[4]; o.cos_th = ob[5];
  o.cos2 = ob[6]; o.rplus = ob[7]; o.rminus = ob[8]; o.minspin = (int)ob[9]; o.r_o_inf = (int)ob[10];
  return o;
}

// mi = (emissivity, velocity, retrograde); md = (emis_p0, emis_p1, mu_ring, vel_p0, vel_p1,
// vel_p2, emiscut_in, emiscut_out, specind, sinthb)
static EmissionModel make_model(const int* mi, const double* md) {
  EmissionModel M;
  M.emis = mi[0]; M.vel = mi[1]; M.retrograde = mi[2];
  M.emis_p[0] = md[0]; M.emis_p[1] = md[1]; M.mu_ring = md[2];
  M.vel_p[0] = md[3]; M.vel_p[1] = md[4]; M.vel_p[2] = md[5];
  M.emiscut_in = md[6]; M.emiscut_out = md[7]; M.specind = md[8]; M.sinthb = md[9];
  M.sinthb_pow = std::pow(md[9], 1 + md[8]);
  return M;
}

extern "C" {
int hm_num_fields() { return NUM_FIELDS; }
// Loop-cap word of the host build (note_loop_cap), returned and cleared.
unsigned hm_take_loop_cap() {
  unsigned w = host_loop_cap();
  host_loop_cap() = 0;
  return w;
}
double hm_rf(double x, double y, double z) { return carlson_rf(x, y, z); }
double hm_rj(double x, double y, double z, double p) { return carlson_rj(x, y, z, p); }
double hm_rd(double x, double y, double z) { return carlson_rd(x, y, z); }
double hm_rc(double x, double y) { return carlson_rc(x, y); }
double hm_ellipf(double phi, double m) { return ellip_f(phi, m); }
double hm_ellipe(double phi, double m) { return ellip_e_inc(phi, m); }
double hm_ellippi(double n, double phi, double m) { return ellip_pi_ref(n, phi, m); }
void hm_jacobi(double u, double m, double* out) {
  Jacobi J = jacobi_landen(u, m);
  out[0] = J.sn; out[1] = J.cn; out[2] = J.dn;
}
void hm_roots(const double* ob, double lam, double eta, double* out, int* rclass) {
  Observer o = make_obs(ob);
  Roots R = radial_roots(o, lam, eta);
  out[0] = R.r1.re; out[1] = R.r1.im; out[2] = R.r2.re; out[3] = R.r2.im;
  out[4] = R.r3.re; out[5] = R.r3.im; out[6] = R.r4.re; out[7] = R.r4.im;
  *rclass = R.rclass;
}
unsigned hm_setup(const double* ob, const double* alpha, const double* beta, long n, double maxtaufrac,
                  double* rec, int* code, int* rclass, int* thclass, long ngeo) {
  Observer o = make_obs(ob);
  unsigned flags = 0;
  for (long i = 0; i < n; ++i) {
    RayRec R;
    flags |= ray_setup(o, alpha[i], beta[i], maxtaufrac, &R, rclass + i, thclass + i);
    if (ngeo > 1) R.code = step_constants<const double*>(R.f, R.code, R.f[F_TAUMAX] / (double)(ngeo - 1), R.f);
    for (int k = 0; k < NUM_FIELDS; ++k) rec[k * n + i] = R.f[k];
    code[i] = R.code;
  }
  return flags;
}
void hm_samples(const double* ob, const double* rec, const int* code, long n, const double* tau, long ntau,
                int ordinary_active, double* t, double* r, double* th, double* ph, double* sig) {
  Observer o = make_obs(ob);
  for (long i = 0; i < n; ++i) {
    RecView f{rec + i, n};
    for (long g = 0; g < ntau; ++g) {
      Sample S = sample_all(o, f, code[i], tau[g * n + i], ordinary_active != 0);
      t[g * n + i] = S.t; r[g * n + i] = S.r; th[g * n + i] = S.th; ph[g * n + i] = S.ph; sig[g * n + i] = S.sig;
    }
  }
}
void hm_samples_stepped(const double* ob, const double* rec, const int* code, long n, long G, long chunk,
                        int ordinary_active, double* t, double* r, double* th, double* ph, double* sig, double* mino) {
  Observer o = make_obs(ob);
  for (long i = 0; i < n; ++i) {
    RecView f{rec + i, n};
    for (long g0 = 0; g0 < G; g0 += chunk) {
      long g1 = g0 + chunk < G ? g0 + chunk : G;
      ray_chunk(o, f, code[i], g0, g1, G, ordinary_active != 0, false, [&](long g, double tau, const Sample& S) {
        t[g * n + i] = S.t; r[g * n + i] = S.r; th[g * n + i] = S.th; ph[g * n + i] = S.ph; sig[g * n + i] = S.sig;
        mino[g * n + i] = tau;
      });
    }
  }
}
void hm_samples_rth(const double* ob, const double* rec, const int* code, long n, long G, long chunk,
                    int ordinary_active, double* r, double* th, double* mino) {
  (void)ob;
  for (long i = 0; i < n; ++i) {
    RecView f{rec + i, n};
    for (long g0 = 0; g0 < G; g0 += chunk) {
      long g1 = g0 + chunk < G ? g0 + chunk : G;
      ray_chunk_rth(f, code[i], g0, g1, G, ordinary_active != 0, false, [&](long g, double tau, double rr, double tt) {
        r[g * n + i] = rr; th[g * n + i] = tt; mino[g * n + i] = tau;
      });
    }
  }
}
void hm_samples_mixed(const double* ob, const double* rec, const int* code, long n, long G, long chunk,
                   int ordinary_active, double* t, double* r, double* th, double* ph, double* sig, double* mino) {
  Observer o = make_obs(ob);
  for (long i = 0; i < n; ++i) {
    RecView f{rec + i, n};
    for (long g0 = 0; g0 < G; g0 += chunk) {
      long g1 = g0 + chunk < G ? g0 + chunk : G;
      FFRay slot;
      ray_chunk_ff(o, f, code[i], g0, g1, G, ordinary_active != 0, false, [&](long g, double tau, const Sample& S) {
        t[g * n + i] = S.t; r[g * n + i] = S.r; th[g * n + i] = S.th; ph[g * n + i] = S.ph; sig[g * n + i] = S.sig;
        mino[g * n + i] = tau;
      }, &slot);
    }
  }
}
void hm_theta_debug(const double* ob, const double* rec, const int* code, long n, long i, long G, double* out) {
  Observer o = make_obs(ob);
  RecView f{rec + i, n};
  double taumax = f[F_TAUMAX];
  ThetaState ts;
  for (long g = 0; g < G; ++g) {
    double tau = linspace_at(g, G, taumax, false);
    ThetaState d = theta_state_direct(f, code[i], theta_snarg(f, tau));
    if (g == 0 || !theta_step(f, &ts)) ts = d;
    double* q = out + g * 10;
    q[0] = ts.sn; q[1] = ts.cn; q[2] = ts.dn; q[3] = ts.pi; q[4] = ts.e;
    q[5] = d.sn; q[6] = d.cn; q[7] = d.dn; q[8] = d.pi; q[9] = d.e;
  }
}
void hm_radial_debug(const double* ob, const double* rec, const int* code, long n, long i, long G, double* out) {
  RecView f{rec + i, n};
  double taumax = f[F_TAUMAX];
  RadialState rs;
  for (long g = 0; g < G; ++g) {
    double tau = linspace_at(g, G, taumax, false);
    double X = radial_X(f, tau);
    RadialState d = radial_state_direct(f, code[i], X, true);
    if (g == 0 || !radial_step(f, &rs, X)) rs = d;
    double* q = out + g * 14;
    q[0] = rs.sn; q[1] = rs.cn; q[2] = rs.dn; q[3] = rs.E; q[4] = rs.P[0]; q[5] = rs.P[1]; q[6] = rs.P[2];
    q[7] = d.sn; q[8] = d.cn; q[9] = d.dn; q[10] = d.E; q[11] = d.P[0]; q[12] = d.P[1]; q[13] = d.P[2];
  }
}
void hm_requatorial(const double* ob, const double* alpha, const double* beta, long n, int mbar_lo, int nord,
                    double* r_s, double* Ir, double* Imax, double* Nmax) {
  Observer o = make_obs(ob);
  for (long i = 0; i < n; ++i) {
    EqResult r = r_equatorial_px(o, alpha[i], beta[i], mbar_lo, nord, r_s + i, Ir + i, n);
    Imax[i] = r.Imax;
    Nmax[i] = r.Nmax;
  }
}
void hm_crossings(const double* ob, const double* alpha, const double* beta, long n, const double* tau, long ntau,
                  double* n_eq, double* n_pol, double* outside) {
  Observer o = make_obs(ob);
  for (long i = 0; i < n; ++i) {
    double lam = -alpha[i] * o.sin_th;
    double eta = (alpha[i] * alpha[i] - o.a2) * o.cos2 + beta[i] * beta[i];
    outside[i] = outside_crit(o, lam, eta);
    EqConsts c = eq_consts(o, lam, eta);
    double Kc = c.vort ? 0.0 : ellip_k(c.ratio);
    for (long g = 0; g < ntau; ++g) {
      n_eq[g * n + i] = n_eq_at(o, c, beta[i], tau[g * n + i]);
      n_pol[g * n + i] = n_pol_at(c, Kc, tau[g * n + i]);
    }
  }
}
// image (npix, nord) outputs as kgeo_image
void hm_image(const double* ob, const int* mi, const double* md, const double* alpha, const double* beta, long n,
              int nord, double* I, double* g, double* r_s, double* Ir, double* sinthb, double* nmax, double* npol) {
  Observer o = make_obs(ob);
  EmissionModel M = make_model(mi, md);
  for (long i = 0; i < n; ++i) {
    PixelGeo p;
    for (int m0 = 0; m0 < nord; m0 += ORDER_GROUP) {
      const int k = std::min(ORDER_GROUP, nord - m0);
      pixel_geo(o, alpha[i], beta[i], m0, k, &p);
      for (int j = 0; j < k; ++j) {
        long q = i * nord + m0 + j;
        double II = 0, gg = 0, sb = 0;
        if (!image_zero(M, o, p, j)) {
          emission_px(M, o, p, j, &II, &gg);
          sb = M.sinthb;
        }
        I[q] = II; g[q] = gg; r_s[q] = p.r_s[j]; Ir[q] = p.Ir[j]; sinthb[q] = sb;
      }
    }
    nmax[i] = p.Nmax;
    npol[i] = p.npol;
  }
}
// image with options: oi = (polarization, pathlength, field, flag); od = (diskangle, c0, c1, c2).
// outs: I, Q, U, g, sinthb, lp, Ie (npix, nord)
void hm_image_opts(const double* ob, const int* mi, const double* md, const int* oi, const double* od,
                   const double* alpha, const double* beta, long n, int nord, double* I, double* Q, double* U,
                   double* g, double* sinthb, double* lp, double* Ie) {
  Observer o = make_obs(ob);
  EmissionModel M = make_model(mi, md);
  ImageOptions P;
  P.polarization = oi[0]; P.pathlength = oi[1]; P.field.field = oi[2]; P.field.flag = oi[3];
  P.diskangle = od[0]; P.field.c[0] = od[1]; P.field.c[1] = od[2]; P.field.c[2] = od[3];
  for (long i = 0; i < n; ++i) {
    PixelGeo p;
    for (int m0 = 0; m0 < nord; m0 += ORDER_GROUP) {
      const int k = std::min(ORDER_GROUP, nord - m0);
      pixel_geo(o, alpha[i], beta[i], m0, k, &p);
      for (int j = 0; j < k; ++j) {
        long q = i * nord + m0 + j;
        PixelOut px{0, 0, 0, 0, 0, 0, 0};
        if (!image_zero(M, o, p, j)) emission_px_opts(M, P, o, p, j, alpha[i], beta[i], &px);
        I[q] = px.I; Q[q] = px.Q; U[q] = px.U; g[q] = px.g; sinthb[q] = px.sinthb; lp[q] = px.lp; Ie[q] = px.Ie;
      }
    }
  }
}
// lab-frame field at (r, pi/2): out (n, 3)
void hm_bfield(int field, int flag, const double* c, double a, const double* r, long n, double* out) {
  FieldModel F{field, flag, {c[0], c[1], c[2]}};
  const double rp = 1 + std::sqrt(1 - a * a);
  for (long i = 0; i < n; ++i) {
    BLab B = bfield_lab(F, a, r[i], rp);
    out[3 * i] = B.b1; out[3 * i + 1] = B.b2; out[3 * i + 2] = B.b3;
  }
}
// rho of curve (observer ob with r_o = inf) at each varphi; status per angle
void hm_curve_rho(const double* ob, double r_eq, int mbar, double rho_min, double rho_max, const double* varphi,
                  long n, double xtol, double rtol, int maxiter, double* rho, int* status) {
  CurveSpec c;
  c.obs = make_obs(ob);
  c.r_target = r_eq;
  c.mbar = mbar;
  c.rho_min = rho_min;
  c.rho_max = rho_max;
  for (long i = 0; i < n; ++i) rho[i] = curve_rho(c, varphi[i], xtol, rtol, maxiter, status + i);
}
// stagnation radius r0 and Omega_F of the field line through theta; returns the status
int hm_jet_stagnation(double a, double th, double* out) { return jet_stagnation(a, th, out, out + 1); }
// per crossing (I, Q, U) of the jet emission; par = (field, nu, sigma, r0, specind), with the BZ
// f(r) table built here from the closed form
void hm_jet_stokes(const double* ob, const double* par, const double* alpha, const double* beta, const double* r,
                   const double* th, const double* kr, const double* kth, long n, double* out) {
  static double* tab = nullptr;
  if (!tab) {
    tab = new double[BZ_TABLE_N];
    for (int64_t k = 0; k < BZ_TABLE_N; ++k) {
      double f, fp;
      bz_f(bz_node(k), &f, &fp);
      tab[k] = f;
    }
  }
  Observer o = make_obs(ob);
  JetImgParams P{(int)par[0], par[1], par[2], par[3], par[4]};
  for (long i = 0; i < n; ++i) {
    Stokes S = jet_stokes(P, tab, o, alpha[i], beta[i], r[i], th[i], kr[i], kth[i]);
    out[3 * i] = S.I;
    out[3 * i + 1] = S.Q;
    out[3 * i + 2] = S.U;
  }
}
double hm_lambert_w0(double z) { return lambert_w0(z); }
double hm_re_li2(double x) { return re_li2(x); }
// per pixel and order dI/dq (npix, nord, NQ); rs_d (npix, nord, 2) = d r_s / d(a, th_o)
void hm_image_jac(const double* ob, const int* mi, const double* md, const double* alpha, const double* beta,
                  long n, int nord, double* jac, double* rs_d) {
  Observer o = make_obs(ob);
  EmissionModel M = make_model(mi, md);
  for (long i = 0; i < n; ++i) {
    for (int m0 = 0; m0 < nord; m0 += ORDER_GROUP) {
      const int k = std::min(ORDER_GROUP, nord - m0);
      PixelGeo p;
      pixel_geo(o, alpha[i], beta[i], m0, k, &p);
      D2 rs[ORDER_GROUP];
      bool live = p.eta > 0;
      if (live) rs_tangents(o, alpha[i], beta[i], p, k, rs);
      for (int j = 0; j < k; ++j) {
        long q = i * nord + m0 + j;
        rs_d[q * 2] = live ? rs[j].d[0] : 0.0;
        rs_d[q * 2 + 1] = live ? rs[j].d[1] : 0.0;
        for (int c = 0; c < NQ; ++c) jac[q * NQ + c] = 0.0;
        if (image_zero(M, o, p, j)) continue;
        Dual<NQ> I = emission_dual(M, o, p, j, alpha[i], beta[i], rs[j]);
        for (int c = 0; c < NQ; ++c) jac[q * NQ + c] = I.d[c];
      }
    }
  }
}
// float-float operations on split doubles: out = add, sub, mul, div, rcp(a), sqr(a), 1 - a
void hm_ff_ops(double a, double b, double* out) {
  ff A = ff_from(a), B = ff_from(b);
  out[0] = ff_to_double(ff_add(A, B));
  out[1] = ff_to_double(ff_sub(A, B));
  out[2] = ff_to_double(ff_mul(A, B));
  out[3] = ff_to_double(ff_div(A, B));
  out[4] = ff_to_double(ff_rcp(A));
  out[5] = ff_to_double(ff_sqr(A));
  out[6] = ff_to_double(ff_one_minus(A));
  out[7] = ff_to_double(A);
  out[8] = ff_to_double(B);
}
// L(a) = ln|(1 + a) / (1 - a)| in float-float, and R_C(1, 1 + e) - 1 in FP32
double hm_ff_logratio(double a) { return ff_to_double(ff_logratio(ff_from(a))); }
double hm_rc_one_m1(double e) { return (double)rc_one_m1_f((float)e); }
}

// The recurrence's observer states from the record (theta_state_seed, radial_state_seed) minus
// the direct evaluations at tau = 0, per stepping ray: out[i * 10 + k] for theta sn, cn, dn, e,
// pi and r sn, cn, dn, E, and the largest Pi difference over the three; the Pi differences are
// relative to max(1, |Pi|) and scaled by min(1, rho), rho = |1 - n sn^2| the distance to the
// pole that amplifies either evaluation's rounding (NaN where the ray does not step or has no
// such part).
extern "C" void hm_seed_check(const double* rec, const int* code, long n, double* out) {
  for (long i = 0; i < n; ++i) {
    double f[NUM_FIELDS];
    for (int k = 0; k < NUM_FIELDS; ++k) f[k] = rec[k * n + i];
    const double* fp = f;
    double* q = out + i * 10;
    for (int k = 0; k < 10; ++k) q[k] = NAN;
    if (!code_step(code[i])) continue;
    if (code_th(code[i]) != TH_ZERO) {
      const ThetaState d = theta_state_direct<const double*>(fp, code[i], theta_snarg<const double*>(fp, 0.0));
      const ThetaState s = theta_state_seed<const double*>(fp);
      const double rho = fmin(1.0, fabs(1.0 - fp[T_N] * d.sn * d.sn));
      q[0] = s.sn - d.sn; q[1] = s.cn - d.cn; q[2] = s.dn - d.dn; q[3] = s.e - d.e;
      q[4] = (s.pi - d.pi) / fmax(1.0, fabs(d.pi)) * rho;
    }
    if (code_rcase(code[i]) != RCASE_NONE) {
      const double X = radial_X<const double*>(fp, 0.0);
      const RadialState d = radial_state_direct<const double*>(fp, code[i], X, true);
      const RadialState s = radial_state_seed<const double*>(fp, X);
      q[5] = s.sn - d.sn; q[6] = s.cn - d.cn; q[7] = s.dn - d.dn; q[8] = s.E - d.E;
      double m = 0.0;
      const double nn[3] = {fp[R_N0], fp[R_N1], fp[R_N2]};
      for (int k = 0; k < 3; ++k) {
        const double rho = fmin(1.0, fabs(1.0 - nn[k] * d.sn * d.sn));
        m = fmax(m, fabs(s.P[k] - d.P[k]) / fmax(1.0, fabs(d.P[k])) * rho);
      }
      q[9] = m;
    }
  }
}
