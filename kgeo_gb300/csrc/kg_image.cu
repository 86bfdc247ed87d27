// Equatorial image kernels (unpolarised, and polarised / with path length). Compiled with
// FMA contraction off (-fmad=false), like the per-ray setup: the crossing count Nmax that
// masks each image order is a floor() of elliptic-integral ratios and must round as numpy's
// does. The adjoint is in kg_image_adj.cu (a separate translation unit, compiled in parallel).
#include "kg_launch.h"

namespace kg {

// OPTS: polarisation and / or path length requested (kg_polar.cuh); the plain image keeps
// the shorter kernel.
template <bool OPTS>
__global__ void __launch_bounds__(IMAGE_BLOCK, 1) image_kernel(ImageArgs a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.npix) return;
  const int64_t i = a.perm ? (int64_t)a.perm[t] : t;
  const Observer& o = a.obs;
  const double alpha = a.alpha[i], beta = a.beta[i];
  PixelGeo p;
  for (int m0 = 0; m0 < a.nord; m0 += ORDER_GROUP) {
    const int n = min(ORDER_GROUP, a.nord - m0);
    pixel_geo(o, alpha, beta, a.mbar_lo + m0, n, &p);
    for (int j = 0; j < n; ++j) {
      const int64_t k = i * a.nord + m0 + j;
      PixelOut px{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      if (!image_zero(a.model, o, p, j)) {
        if (OPTS) {
          emission_px_opts(a.model, a.opts, o, p, j, alpha, beta, &px);
        } else {
          emission_px(a.model, o, p, j, &px.I, &px.g);
          px.sinthb = a.model.sinthb;
        }
      }
      a.I[k] = px.I;
      if (a.g) a.g[k] = px.g;
      if (a.r_s) a.r_s[k] = p.r_s[j];
      if (a.Ir) a.Ir[k] = p.Ir[j];
      if (a.sinthb) a.sinthb[k] = px.sinthb;
      if (OPTS) {
        if (a.Q) a.Q[k] = px.Q;
        if (a.U) a.U[k] = px.U;
        if (a.lp) a.lp[k] = px.lp;
        if (a.Ie) a.Ie[k] = px.Ie;
      }
    }
  }
  if (a.imax) a.imax[i] = p.Imax;
  if (a.nmax) a.nmax[i] = p.Nmax;
  if (a.npol) a.npol[i] = p.npol;
}

// ---- pixel order: counting sort by radial class (see launch_pixel_sort) ----

// key of each pixel and the per-block class counts, stored class-major: counts[k * nblk + b]
__global__ void __launch_bounds__(PIX_SORT_BLOCK) pixel_key_kernel(Observer o, const double* alpha,
                                                                   const double* beta, int64_t npix, int* key,
                                                                   uint32_t* counts, int64_t nblk) {
  __shared__ uint32_t cnt[PIX_BUCKETS];
  if (threadIdx.x < PIX_BUCKETS) cnt[threadIdx.x] = 0u;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < npix) {
    const double al = alpha[i], be = beta[i];
    const double lam = -al * o.sin_th;
    const double eta = (al * al - o.a2) * o.cos2 + be * be;
    int k = 0;
    if (eta > 0) k = radial_roots(o, lam, eta).rclass;
    k = k < 0 ? 0 : (k >= PIX_BUCKETS ? PIX_BUCKETS - 1 : k);
    key[i] = k;
    atomicAdd(&cnt[k], 1u);
  }
  __syncthreads();
  if (threadIdx.x < PIX_BUCKETS) counts[(int64_t)threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of the n class-major counts in place (one block, tiles of 1024).
__global__ void __launch_bounds__(1024) pixel_scan_kernel(uint32_t* counts, int64_t n) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0u;
  __syncthreads();
  for (int64_t base = 0; base < n; base += blockDim.x) {
    const int64_t idx = base + threadIdx.x;
    const uint32_t v = idx < n ? counts[idx] : 0u;
    uint32_t x = v;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      const uint32_t t0 = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
      uint32_t y = t0;
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t z = __shfl_up_sync(0xffffffffu, y, off);
        if (lane >= off) y += z;
      }
      if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = y - t0;
    }
    __syncthreads();
    const uint32_t excl = carry + warp_tot[w] + x - v;
    if (idx < n) counts[idx] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
}

// Position of every pixel: its class's offset for this block, the counts of the block's earlier
// warps in that class, its rank among its warp's lanes of that class (no atomics: the order is
// the same in every run).
__global__ void __launch_bounds__(PIX_SORT_BLOCK) pixel_scatter_kernel(const int* key, int64_t npix,
                                                                       const uint32_t* offs, int64_t nblk,
                                                                       int* perm) {
  __shared__ uint32_t wcnt[PIX_SORT_BLOCK / 32][PIX_BUCKETS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < (PIX_SORT_BLOCK / 32) * PIX_BUCKETS; t += blockDim.x) (&wcnt[0][0])[t] = 0u;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = i < npix ? key[i] : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, k);
  const unsigned below = peers & ((1u << lane) - 1u);
  if (k >= 0 && below == 0u) wcnt[w][k] = (uint32_t)__popc(peers);
  __syncthreads();
  if (k >= 0) {
    uint32_t pos = offs[(int64_t)k * nblk + blockIdx.x];
    for (int v = 0; v < w; ++v) pos += wcnt[v][k];
    pos += (uint32_t)__popc(below);
    perm[pos] = (int)i;
  }
}

cudaError_t launch_pixel_sort(const Observer& o, const double* alpha, const double* beta, int64_t npix, void* scratch,
                              const int** perm, cudaStream_t s) {
  *perm = nullptr;
  if (npix <= 0) return cudaSuccess;
  const int64_t nblk = pixel_sort_blocks(npix);
  char* p = static_cast<char*>(scratch);
  int* key = reinterpret_cast<int*>(p);
  int* pm = reinterpret_cast<int*>(p + align_up(sizeof(int) * (size_t)npix, 256));
  uint32_t* counts = reinterpret_cast<uint32_t*>(p + 2 * align_up(sizeof(int) * (size_t)npix, 256));
  pixel_key_kernel<<<(unsigned)nblk, PIX_SORT_BLOCK, 0, s>>>(o, alpha, beta, npix, key, counts, nblk);
  pixel_scan_kernel<<<1, 1024, 0, s>>>(counts, (int64_t)PIX_BUCKETS * nblk);
  pixel_scatter_kernel<<<(unsigned)nblk, PIX_SORT_BLOCK, 0, s>>>(key, npix, counts, nblk, pm);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) *perm = pm;
  return e;
}

cudaError_t launch_image(const ImageArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const unsigned nb = (unsigned)image_adjoint_blocks(a.npix);
  if (a.opts.polarization || a.opts.pathlength)
    image_kernel<true><<<nb, IMAGE_BLOCK, 0, s>>>(a);
  else
    image_kernel<false><<<nb, IMAGE_BLOCK, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
