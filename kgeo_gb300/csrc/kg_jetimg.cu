// Stokes images of the off-equatorial jet crossings (kg_jetimg.cuh). FMA contraction off
// (-fmad=false): the emission formulas round term by term as numpy's arithmetic does.
#include <mutex>

#include "kg_launch.h"

namespace kg {

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_table_mu;
double* g_table[MAX_DEVICES] = {};

}  // namespace

__global__ void __launch_bounds__(256) bz_table_kernel(double* tab) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= BZ_TABLE_N) return;
  double f, fp;
  bz_f(bz_node(k), &f, &fp);
  tab[k] = f;
}

cudaError_t jet_bz_table(const double** tab) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_table_mu);
  if (!g_table[dev]) {
    double* t = nullptr;
    e = cudaMalloc(&t, sizeof(double) * BZ_TABLE_N);
    if (e != cudaSuccess) return e;
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      cudaFree(t);
      return e;
    }
    bz_table_kernel<<<(BZ_TABLE_N + 255) / 256, 256, 0, s>>>(t);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
      cudaFree(t);
      return e;
    }
    g_table[dev] = t;
  }
  *tab = g_table[dev];
  return cudaSuccess;
}

// One block: the first crossing of the first guess row (np.where(r[0] != 0)[0][0]), then the
// stagnation radius of its field line, the five Aberth roots iterated by lanes 0-4 of warp 0
// (the same arithmetic as quintic_max_real_root). par = (r0, Omega, status): status 1 when the
// row has no crossing (the reference's index lookup raises), 2 or 3 when the quintic has no
// root 4.
__global__ void __launch_bounds__(256) jet_stagnation_kernel(const double* r, const double* th, int64_t npix,
                                                             double a, double* par) {
  __shared__ unsigned long long first;
  __shared__ double coef[6];
  __shared__ Cplx z[5];
  __shared__ int state;
  if (threadIdx.x == 0) first = ~0ull;
  __syncthreads();
  for (int64_t base = 0; base < npix; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const bool hit = i < npix && !(r[i] == 0.0);
    if (hit) atomicMin(&first, (unsigned long long)i);
    if (__syncthreads_or(hit)) break;
  }
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  if (lane == 0) {
    state = 0;
    if (first == ~0ull) {
      state = 1;
    } else {
      double om = 0.0;
      stagnation_quintic(a, th[first], coef, &om);
      par[1] = om;
      if (!(coef[5] != 0.0) || !kg_finite(coef[5])) state = 2;
      else if (aberth_radius(coef) == 0.0) state = 3;
    }
  }
  __syncwarp();
  if (state != 0) {
    if (lane == 0) {
      par[0] = 0.0;
      if (state == 1) par[1] = 0.0;
      par[2] = (double)state;
    }
    return;
  }
  double c[6];
  for (int k = 0; k < 6; ++k) c[k] = coef[k];
  if (lane < 5) z[lane] = aberth_start(aberth_radius(c), lane);
  __syncwarp();
  for (int it = 0; it < ABERTH_MAXITER; ++it) {
    Cplx zl[5];
    for (int k = 0; k < 5; ++k) zl[k] = z[k];
    double corr = 0.0;
    Cplx zi{0.0, 0.0};
    if (lane < 5) {
      const Cplx w = aberth_correction(c, zl, lane);
      zi = c_sub(zl[lane], w);
      corr = c_abs(w) / fmax(c_abs(zi), 1e-300);
    }
    __syncwarp();
    if (lane < 5) z[lane] = zi;
    for (int o = 16; o > 0; o >>= 1) corr = fmax(corr, __shfl_xor_sync(0xffffffffu, corr, o));
    __syncwarp();
    if (corr < ABERTH_TOL) break;
  }
  if (lane == 0) {
    Cplx zl[5];
    for (int k = 0; k < 5; ++k) zl[k] = z[k];
    double r0 = 0.0;
    const int st = aberth_finish(c, zl, &r0);
    par[0] = r0;
    par[2] = (double)st;
  }
}

__global__ void __launch_bounds__(128) jet_stokes_kernel(JetStokesArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double st = a.par[2];
  if (i == 0) {
    if (a.stagnation) {
      a.stagnation[0] = a.par[0];
      a.stagnation[1] = a.par[1];
    }
    if (a.status) a.status[0] = (int32_t)st;
  }
  if (i >= a.npix) return;
  JetImgParams P = a.p;
  P.r0 = a.par[0];
  const bool ok = st == 0.0;
  const int64_t n = a.npix;
  for (int k = 0; k <= a.neqmax; ++k) {
    a.I[k * n + i] = 0.0;
    a.Q[k * n + i] = 0.0;
    a.U[k * n + i] = 0.0;
  }
  const double alpha = a.alpha[i], beta = a.beta[i];
  double tI = 0.0, tQ = 0.0, tU = 0.0;
  for (int64_t g = 0; g < a.nguess; ++g) {
    const int64_t q = g * n + i;
    Stokes S{0.0, 0.0, 0.0};
    if (ok) S = jet_stokes(P, a.tab, a.obs, alpha, beta, a.r[q], a.th[q], a.signpr[q], a.signpth[q]);
    if (a.Ic) a.Ic[q] = S.I;
    if (a.Qc) a.Qc[q] = S.Q;
    if (a.Uc) a.Uc[q] = S.U;
    tI += S.I;
    tQ += S.Q;
    tU += S.U;
    const double ne = a.neq[q];
    if (ne >= 0.0 && ne < (double)a.neqmax && ne == floor(ne)) {
      const int64_t o = (int64_t)ne * n + i;
      a.I[o] += S.I;
      a.Q[o] += S.Q;
      a.U[o] += S.U;
    }
  }
  const int64_t t = (int64_t)a.neqmax * n + i;
  a.I[t] = tI;
  a.Q[t] = tQ;
  a.U[t] = tU;
  if (a.evpa)
    for (int k = 0; k <= a.neqmax; ++k) a.evpa[k * n + i] = nan_to_num(0.5 * atan2(a.U[k * n + i], a.Q[k * n + i]));
}

cudaError_t launch_jet_stokes(const JetStokesArgs& a, cudaStream_t s) {
  jet_stagnation_kernel<<<1, 256, 0, s>>>(a.r, a.th, a.nguess > 0 ? a.npix : 0, a.obs.a, a.par);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t blocks = (a.npix + 127) / 128;
  jet_stokes_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
