// Jet field-line crossing kernels (kg_jet.cuh). FMA contraction off (-fmad=false), like the
// other kernels whose counts (ceil, sign changes) must round as numpy's arithmetic does.
#include "kg_jet.cuh"
#include "kg_launch.h"

namespace kg {

__global__ void __launch_bounds__(128) jet_guess_kernel(JetGuessArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  const double alpha = a.alpha[i], beta = a.beta[i];
  if (a.taumax) a.taumax[i] = jet_taumax(a.obs, alpha, beta, a.neqmax);
  if (!a.r) return;
  const int n = jet_pixel_guesses(a.obs, a.field, alpha, beta, a.r + i, a.th + i, a.mino + i, a.ngeo, a.npix,
                                  a.neqmax, nullptr, 0);
  if (a.count) a.count[i] = n;
  if (a.guesses) {
    for (int64_t g = 0; g < a.nguess; ++g) a.guesses[g * a.npix + i] = -1.0;
    if (n <= a.nguess)
      jet_pixel_guesses(a.obs, a.field, alpha, beta, a.r + i, a.th + i, a.mino + i, a.ngeo, a.npix, a.neqmax,
                        a.guesses + i, a.npix);
  }
}

cudaError_t launch_jet_guesses(const JetGuessArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  jet_guess_kernel<<<(unsigned)((a.npix + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) jet_solve_kernel(JetSolveArgs a) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.npix * a.nguess) return;
  const int64_t i = q % a.npix;
  const bool ordinary_active = (*a.flags & FLAG_ANY_ETA_POS) != 0;
  RecView f{a.rec + i, a.npix};
  const JetRoot R = jet_solve(a.obs, a.field, f, __ldg(a.code + i), ordinary_active, a.alpha[i], a.beta[i],
                              a.guesses[q], a.tol, a.maxiter);
  a.tau[q] = R.tau;
  if (a.r) a.r[q] = R.r;
  if (a.th) a.th[q] = R.th;
  if (a.signpr) a.signpr[q] = R.signpr;
  if (a.signpth) a.signpth[q] = R.signpth;
  if (a.neq) a.neq[q] = R.neq;
  if (a.status) a.status[q] = R.status;
}

cudaError_t launch_jet_solve(const JetSolveArgs& a, cudaStream_t s) {
  const int64_t n = a.npix * a.nguess;
  if (n <= 0) return cudaSuccess;
  jet_solve_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
