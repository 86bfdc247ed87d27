// FP32 Carlson integrals for the mixed-precision sample path.
//
// The same published algorithms as kg_elliptic.cuh (Carlson 1995 duplication with the
// fifth-order tail, R_C from DLMF 19.2.17-20), with single-precision stopping constants:
// (3 r)^(-1/6) = 12.2 and (r / 4)^(-1/6) = 18.4 for r = 1e-7.
#pragma once

#include "kg_common.cuh"

namespace kg {

constexpr float RF_Q32 = 12.2f;
constexpr float RJ_Q32 = 18.4f;
constexpr int CARLSON_MAX_IT32 = 24;

// R_C(1, 1 + e), e > -1.
KG_HD float rc_one_f(float e) {
  if (fabsf(e) < 2.0e-2f) {
    return 1.0f + e * (-1.0f / 3.0f + e * (1.0f / 5.0f + e * (-1.0f / 7.0f + e * (1.0f / 9.0f + e * (-1.0f / 11.0f)))));
  }
  if (e > 0.0f) {
    float s = sqrtf(e);
    return atanf(s) / s;
  }
  float s = sqrtf(-e);
  return (log1pf(s) - 0.5f * log1pf(e)) / s;
}

// General R_C(x, y), y != 0 (Cauchy principal value for y < 0).
KG_HD float carlson_rc_f(float x, float y) {
  if (y < 0.0f) return sqrtf(x / (x - y)) * carlson_rc_f(x - y, -y);
  float d = y - x;
  if (fabsf(d) < 2.0e-2f * x) return rc_one_f(d / x) / sqrtf(x);
  if (d > 0.0f) {
    if (x == 0.0f) return 1.5707963f / sqrtf(y);
    return atanf(sqrtf(d / x)) / sqrtf(d);
  }
  float xd = -d;
  return logf((sqrtf(x) + sqrtf(xd)) / sqrtf(y)) / sqrtf(xd);
}

// R_F(x,y,z) and R_J(x,y,z,p[i]) for NP values p[i] > 0 sharing the x,y,z duplication.
template <int NP>
KG_HD void rj_multi_f(float x, float y, float z, const float* p_in, float* rj, float* rf) {
  const float x0 = x, y0 = y, z0 = z;
  const float Af0 = (x + y + z) * (1.0f / 3.0f);
  const float Qf = RF_Q32 * fmaxf(fmaxf(fabsf(Af0 - x), fabsf(Af0 - y)), fabsf(Af0 - z));
  float Af = Af0;
  float p[NP], A0[NP], A[NP], Q[NP], delta[NP], sum[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    p[i] = p_in[i];
    A0[i] = (x + y + z + 2.0f * p[i]) * 0.2f;
    A[i] = A0[i];
    delta[i] = (p[i] - x) * (p[i] - y) * (p[i] - z);
    sum[i] = 0.0f;
    Q[i] = RJ_Q32 * fmaxf(fmaxf(fabsf(A0[i] - x), fabsf(A0[i] - y)), fmaxf(fabsf(A0[i] - z), fabsf(A0[i] - p[i])));
  }
  float f = 1.0f, f3 = 1.0f;
  for (int it = 0; it < CARLSON_MAX_IT32; ++it) {
    bool done = f * Qf < fabsf(Af);
#pragma unroll
    for (int i = 0; i < NP; ++i) done = done && (f * Q[i] < fabsf(A[i]));
    if (done) break;
    float sx = sqrtf(x), sy = sqrtf(y), sz = sqrtf(z);
    float lam = sx * sy + sx * sz + sy * sz;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      float sp = sqrtf(p[i]);
      float d = (sp + sx) * (sp + sy) * (sp + sz);
      float e = f3 * delta[i] / (d * d);
      float term;
      if (fabsf(e) < 2.0e-2f) {
        term = rc_one_f(e) / d;
      } else {
        float al = p[i] * (sx + sy + sz) + sx * sy * sz;
        float pl = p[i] + lam;
        term = 0.5f * carlson_rc_f(al * al, p[i] * pl * pl);
      }
      sum[i] += f * term;
      p[i] = 0.25f * (p[i] + lam);
      A[i] = 0.25f * (A[i] + lam);
    }
    x = 0.25f * (x + lam);
    y = 0.25f * (y + lam);
    z = 0.25f * (z + lam);
    Af = 0.25f * (Af + lam);
    f *= 0.25f;
    f3 *= 0.015625f;
  }
  {
    float X = (Af0 - x0) * f / Af;
    float Y = (Af0 - y0) * f / Af;
    float Z = -(X + Y);
    float E2 = X * Y - Z * Z;
    float E3 = X * Y * Z;
    *rf = (1.0f - E2 * 0.1f + E3 * (1.0f / 14.0f) + E2 * E2 * (1.0f / 24.0f) - 3.0f * E2 * E3 * (1.0f / 44.0f)) * rsqrt_f(Af);
  }
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    float inv = f / A[i];
    float X = (A0[i] - x0) * inv;
    float Y = (A0[i] - y0) * inv;
    float Z = (A0[i] - z0) * inv;
    float P = -0.5f * (X + Y + Z);
    float XYZ = X * Y * Z;
    float P2 = P * P;
    float E2 = X * Y + X * Z + Y * Z - 3.0f * P2;
    float E3 = XYZ + 2.0f * E2 * P + 4.0f * P2 * P;
    float E4 = (2.0f * XYZ + E2 * P + 3.0f * P2 * P) * P;
    float E5 = XYZ * P2;
    float tail = 1.0f - 3.0f * E2 * (1.0f / 14.0f) + E3 * (1.0f / 6.0f) + 9.0f * E2 * E2 * (1.0f / 88.0f) -
                 3.0f * E4 * (1.0f / 22.0f) - 9.0f * E2 * E3 * (1.0f / 52.0f) + 3.0f * E5 * (1.0f / 26.0f);
    rj[i] = f * tail * rsqrt_f(A[i]) / A[i] + 6.0f * sum[i];
  }
}

// FP32 counterpart of carlson_set (kg_ray.cuh): up to NP Pi's plus R_D, DLMF 19.20.14 for rho < 0.
template <int NP>
KG_HD void carlson_set_f(float x, float y, float z, const float* rho, float* rj, float* rd, float* rf) {
  float p[NP + 1], q[NP];
  bool neg[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    neg[i] = !(rho[i] > 0.0f);
    q[i] = -rho[i];
    p[i] = neg[i] ? (z * (x + y + q[i]) - x * y) / (z + q[i]) : rho[i];
    if (rho[i] == 0.0f) p[i] = z;
  }
  p[NP] = z;
  float out[NP + 1];
  rj_multi_f<NP + 1>(x, y, z, p, out, rf);
  *rd = out[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    if (rho[i] == 0.0f) {
      rj[i] = __builtin_huge_valf();
    } else if (neg[i]) {
      float pq = p[i] * q[i];
      float xy = x * y;
      float rc = carlson_rc_f(xy + pq, pq);
      rj[i] = ((p[i] - z) * out[i] - 3.0f * (*rf) + 3.0f * sqrtf((xy * z) / (xy + pq)) * rc) / (q[i] + z);
    } else {
      rj[i] = out[i];
    }
  }
}

}  // namespace kg
