// Per-ray setup kernel. Compiled with FMA contraction off (-fmad=false) so that the
// classification arithmetic rounds one operation at a time, as numpy does.
#include "kg_launch.h"

namespace kg {

// The per-ray setup in numpy's one-operation-at-a-time rounding (the classification decides
// integer outputs, and several ray constants are ill-conditioned functions of the observer's
// position that the reference evaluates in that rounding). The step constants of the even
// Mino grid and the class-bucket counts follow in ray_step_kernel (kg_samples.cu), where FMA
// contraction is allowed.
__global__ void __launch_bounds__(128) ray_setup_kernel(SetupArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned fl = 0;
  loop_cap_begin();
  if (i < a.npix) {
    RayRec R;
    int rc = 0, tc = 0;
    fl = ray_setup(a.obs, a.alpha[i], a.beta[i], a.maxtaufrac, &R, &rc, &tc);
    const double* f = R.f;
#pragma unroll
    for (int k = 0; k < NUM_FIELDS; ++k) a.rec[(int64_t)k * a.npix + i] = f[k];
    a.code[i] = R.code;
    if (a.rclass) a.rclass[i] = rc;
    if (a.thclass) a.thclass[i] = tc;
    if (a.tau_tot) a.tau_tot[i] = f[F_TAUTOT];
    if (a.ngeo > 1 && f[F_TAUMAX] / (double)(a.ngeo - 1) == 0.0) fl |= FLAG_ANY_STEP_ZERO;
  }
  fl = __reduce_or_sync(0xffffffffu, fl);
  if ((threadIdx.x & 31) == 0 && fl) atomicOr(a.flags, fl);
  loop_cap_end(a.flags);
}

// Exclusive scan of the bucket counts into the cursors (one warp).
__global__ void bucket_scan_kernel(uint32_t* counts) {
  const int lane = threadIdx.x;
  uint32_t c = counts[lane];
  uint32_t v = c;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  counts[NBUCKET + lane] = v - c;
}

// Scatter rays into their buckets (order inside a bucket follows warp arrival; the
// computation of a ray does not depend on its position).
__global__ void __launch_bounds__(128) bucket_scatter_kernel(const int* code, int64_t npix, uint32_t* counts, int* perm) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int key = i < npix ? ray_bucket(code[i]) : -1;
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(grp) - 1;
  uint32_t base = 0;
  if (key >= 0 && lane == leader) base = atomicAdd(counts + NBUCKET + key, (uint32_t)__popc(grp));
  base = __shfl_sync(grp, base, leader);
  if (key >= 0) perm[base + __popc(grp & ((1u << lane) - 1u))] = (int)i;
}

cudaError_t launch_ray_setup(const SetupArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  const int64_t grid = (a.npix + block - 1) / block;
  ray_setup_kernel<<<(unsigned)grid, block, 0, s>>>(a);
  if (launch_ray_step(a, s) != cudaSuccess) return cudaGetLastError();
  bucket_scan_kernel<<<1, 32, 0, s>>>(a.counts);
  bucket_scatter_kernel<<<(unsigned)grid, block, 0, s>>>(a.code, a.npix, a.counts, a.perm);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) equatorial_kernel(EquatorialArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  EqResult r = r_equatorial_px(a.obs, a.alpha[i], a.beta[i], a.mbar_lo, a.nord, a.r_s + i, a.Ir + i, a.npix);
  if (a.Imax) a.Imax[i] = r.Imax;
  if (a.Nmax) a.Nmax[i] = r.Nmax;
}

cudaError_t launch_equatorial(const EquatorialArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  equatorial_kernel<<<(unsigned)((a.npix + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) crossings_kernel(CrossingArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  const Observer& o = a.obs;
  double alpha = a.alpha[i], beta = a.beta[i];
  double lam = -alpha * o.sin_th;
  double eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  if (a.outside) a.outside[i] = outside_crit(o, lam, eta);
  if (a.ntau > 0 && a.n_turn) {
    const TurnConsts tc = turn_consts(o, lam, eta);
    for (int64_t g = 0; g < a.ntau; ++g) a.n_turn[g * a.npix + i] = n_turn_at(tc, beta, a.tau[g * a.npix + i]);
  }
  if (a.ntau <= 0 || (!a.n_eq && !a.n_pol)) return;
  EqConsts c = eq_consts(o, lam, eta);
  double Kc = c.vort ? 0.0 : ellip_k(c.ratio);
  for (int64_t g = 0; g < a.ntau; ++g) {
    double tau = a.tau[g * a.npix + i];
    if (a.n_eq) a.n_eq[g * a.npix + i] = n_eq_at(o, c, beta, tau);
    if (a.n_pol) a.n_pol[g * a.npix + i] = n_pol_at(c, Kc, tau);
  }
}

cudaError_t launch_crossings(const CrossingArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  crossings_kernel<<<(unsigned)((a.npix + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// batched images
// ---------------------------------------------------------------------------

// Work-item offsets of the sample kernel: image i has npix * ceil(ngeo / chunk) items.
__global__ void batch_item_offsets_kernel(BatchArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t acc = 0;
  for (int i = 0; i < a.nimg; ++i) {
    a.item_off[i] = acc;
    const int64_t ng = a.img[i].ngeo;
    acc += a.img[i].npix * ((ng + a.chunk - 1) / a.chunk);
  }
  a.item_off[a.nimg] = acc;
}

// The per-ray setup of every image's rays (as ray_setup_kernel); batch_step_kernel
// (kg_samples.cu) follows with the step constants and the bucket counts.
__global__ void __launch_bounds__(128) batch_setup_kernel(BatchArgs a) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned fl = 0;
  int im = 0;
  loop_cap_begin();
  if (r < a.ntot) {
    im = batch_find(a.pix_off, a.nimg, r);
    const BatchImage& B = a.img[im];
    RayRec R;
    int rc = 0, tc = 0;
    fl = ray_setup(B.obs, a.alpha[r], a.beta[r], B.maxtaufrac, &R, &rc, &tc);
    const double* f = R.f;
    if (B.ngeo > 1 && f[F_TAUMAX] / (double)(B.ngeo - 1) == 0.0) fl |= FLAG_ANY_STEP_ZERO;
#pragma unroll
    for (int k = 0; k < NUM_FIELDS; ++k) a.rec[(int64_t)k * a.ntot + r] = f[k];
    a.code[r] = R.code;
    if (a.rclass) a.rclass[r] = rc;
    if (a.thclass) a.thclass[r] = tc;
    if (a.tau_tot) a.tau_tot[r] = f[F_TAUTOT];
  }
  // flags: one atomic per image present in the warp (warp-uniform loop, full-mask reductions)
  const int lane = threadIdx.x & 31;
  unsigned pending = __ballot_sync(0xffffffffu, r < a.ntot);
  while (pending) {
    const int leader = __ffs(pending) - 1;
    const int lim = __shfl_sync(0xffffffffu, im, leader);
    const bool mine = r < a.ntot && im == lim;
    const unsigned in = __ballot_sync(0xffffffffu, mine);
    const unsigned v = __reduce_or_sync(0xffffffffu, mine ? fl : 0u);
    if (lane == leader && v) atomicOr(a.flags + lim, v);
    pending &= ~in;
  }
  batch_loop_cap_end(a);
}

// Per image: exclusive scan of its NBUCKET counts into cursors that start at its first ray.
__global__ void batch_scan_kernel(BatchArgs a) {
  const int im = blockIdx.x, lane = threadIdx.x;
  const uint32_t c = a.counts[im * NBUCKET + lane];
  uint32_t v = c;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  a.counts[(int64_t)a.nimg * NBUCKET + im * NBUCKET + lane] = (uint32_t)a.img[im].pix_off + (v - c);
}

__global__ void __launch_bounds__(128) batch_scatter_kernel(BatchArgs a) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int key = r < a.ntot ? batch_find(a.pix_off, a.nimg, r) * NBUCKET + ray_bucket(a.code[r]) : -1;
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(grp) - 1;
  uint32_t base = 0;
  if (key >= 0 && lane == leader) base = atomicAdd(a.counts + (int64_t)a.nimg * NBUCKET + key, (uint32_t)__popc(grp));
  base = __shfl_sync(grp, base, leader);
  if (key >= 0) a.perm[base + __popc(grp & ((1u << lane) - 1u))] = (int)r;
}

cudaError_t launch_batch_setup(const BatchArgs& a, cudaStream_t s) {
  batch_item_offsets_kernel<<<1, 32, 0, s>>>(a);
  if (a.ntot > 0) {
    const int block = 128;
    const unsigned grid = (unsigned)((a.ntot + block - 1) / block);
    batch_setup_kernel<<<grid, block, 0, s>>>(a);
    if (launch_batch_step(a, s) != cudaSuccess) return cudaGetLastError();
    batch_scan_kernel<<<a.nimg, 32, 0, s>>>(a);
    batch_scatter_kernel<<<grid, block, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace kg

namespace kg {

// Pi(n; phi | m) with the reference adapter's special cases, as the per-ray setup evaluates
// it (ellip_set_at in this translation unit's no-contraction arithmetic), one value per thread.
__global__ void __launch_bounds__(256) ellip_pi_setup_kernel(const double* n, const double* phi, const double* m,
                                                             int64_t N, double* out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    const double ni = n[i], mi = m[i];
    const EllipSet<1> comp = ellip_set_at<1>(HALFPI, mi, &ni, nullptr);
    out[i] = ellip_set_at<1>(phi[i], mi, &ni, &comp).P[0];
  }
}

cudaError_t launch_ellip_pi_setup(const double* n, const double* phi, const double* m, int64_t N, double* out,
                                  cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  int64_t grid = (N + 255) / 256;
  if (grid > 152 * 16) grid = 152 * 16;
  ellip_pi_setup_kernel<<<(unsigned)grid, 256, 0, s>>>(n, phi, m, N, out);
  return cudaGetLastError();
}

}  // namespace kg
