// Per-sample kernel: one thread per (pixel, Mino sample) item, items ordered pixel-major so
// that the lanes of a warp walk consecutive samples of the same ray and take the same
// branches; stores go to the (nsamp, npix) row-major outputs.
#include "kg_launch.h"
#include "kg_mixed2.cuh"

namespace kg {

__global__ void __launch_bounds__(256) samples_kernel(SampleArgs a) {
  const uint32_t fl = *a.flags;
  loop_cap_begin();
  const bool ordinary_active = (fl & FLAG_ANY_ETA_POS) != 0;
  const bool step_zero = (fl & FLAG_ANY_STEP_ZERO) != 0;
  const int64_t total = a.npix * a.nsamp;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int64_t p = i / a.nsamp;
    const int64_t g = i - p * a.nsamp;
    RecView f{a.rec + p, a.npix};
    double tau = a.tau ? a.tau[g * a.npix + p] : linspace_at(g, a.nsamp, f[F_TAUMAX], step_zero);
    const int code = __ldg(a.code + p);
    const int64_t o = g * a.npix + p;
    if (a.do_phi_t) {
      Sample S = sample_all(a.obs, f, code, tau, ordinary_active);
      if (a.t) a.t[o] = S.t;
      if (a.r) a.r[o] = S.r;
      if (a.th) a.th[o] = S.th;
      if (a.ph) a.ph[o] = S.ph;
      if (a.sig) a.sig[o] = S.sig;
    } else {
      ThetaOut T = sample_theta(f, code, tau, ordinary_active);
      RadialOut R = sample_radial(f, code, tau, false);
      if (a.r) a.r[o] = R.r;
      if (a.th) a.th[o] = T.th;
      // without phi and t the reference's sums reduce to I_t = 4 I_0 = -4 tau, I_phi = I_sig = 0
      if (a.t) a.t[o] = 0 + 4 * (-tau);
      if (a.ph) a.ph[o] = 0.0;
      if (a.sig) a.sig[o] = 0.0;
    }
    if (a.mino) a.mino[o] = tau;
  }
  loop_cap_end(a.flags);
}

// Even Mino grid: one thread per (pixel, chunk of `chunk` consecutive samples), items
// chunk-major over the class-sorted pixels. Each thread evaluates its first sample (and the
// grid's last) directly and the others by the addition-theorem recurrence (kg::ray_chunk).
// Dynamic shared memory of the mixed kernels: one FFRay slot per thread.
extern __shared__ float kg_ffray_smem[];

__device__ __forceinline__ FFRay* ffray_slot() { return reinterpret_cast<FFRay*>(kg_ffray_smem) + threadIdx.x; }

template <bool MIXED, bool RTH>
__global__ void __launch_bounds__(256) stepped_kernel(SampleArgs a) {
  const uint32_t fl = *a.flags;
  loop_cap_begin();
  const bool ordinary_active = (fl & FLAG_ANY_ETA_POS) != 0;
  const bool step_zero = (fl & FLAG_ANY_STEP_ZERO) != 0;
  const int64_t chunk = a.chunk;
  const int64_t nch = (a.nsamp + chunk - 1) / chunk;
  const int64_t c_end = a.c_end < 0 ? nch : a.c_end;
  const int64_t total = a.npix * (c_end - a.c_begin);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    // lanes take consecutive rays of the class-sorted order at the same chunk: uniform
    // branches across the warp and (mostly) contiguous stores
    const int64_t ci = i / a.npix;
    const int64_t c = a.c_begin + ci;
    const int64_t p = __ldg(a.perm + (i - ci * a.npix));
    RecView f{a.rec + p, a.npix};
    const int code = __ldg(a.code + p);
    const int64_t g0 = c * chunk;
    const int64_t g1 = g0 + chunk < a.nsamp ? g0 + chunk : a.nsamp;
    auto emit = [&](int64_t g, double tau, const Sample& S) {
      const int64_t o = (g - a.row0) * a.npix + p;
      if (a.t) a.t[o] = S.t;
      if (a.r) a.r[o] = S.r;
      if (a.th) a.th[o] = S.th;
      if (a.ph) a.ph[o] = S.ph;
      if (a.sig) a.sig[o] = S.sig;
      if (a.mino) a.mino[o] = tau;
    };
    if (MIXED) {
      ray_chunk_ff(a.obs, f, code, g0, g1, a.nsamp, ordinary_active, step_zero, emit, ffray_slot());
    } else if (RTH) {
      ray_chunk_rth(f, code, g0, g1, a.nsamp, ordinary_active, step_zero,
                    [&](int64_t g, double tau, double r, double th) {
                      const int64_t o = (g - a.row0) * a.npix + p;
                      if (a.r) a.r[o] = r;
                      if (a.th) a.th[o] = th;
                      if (a.mino) a.mino[o] = tau;
                    });
    } else {
      ray_chunk(a.obs, f, code, g0, g1, a.nsamp, ordinary_active, step_zero, emit);
    }
  }
  loop_cap_end(a.flags);
}

// Step constants of the even Mino grid (step_constants: the Jacobi values and integral
// increments of one step, the recurrence and precision bits of the code word), after
// ray_setup_kernel wrote the record; in this translation unit FMA contraction is allowed. Counts
// the class buckets of the final code words.
__global__ void __launch_bounds__(128) ray_step_kernel(SetupArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int key = -1;
  loop_cap_begin();
  if (i < a.npix) {
    int code = a.code[i];
    if (a.ngeo > 1) {
      double f[NUM_FIELDS];
#pragma unroll
      for (int k = 0; k < NUM_FIELDS; ++k) f[k] = a.rec[(int64_t)k * a.npix + i];
      code = step_constants<const double*>(f, code, f[F_TAUMAX] / (double)(a.ngeo - 1), f);
#pragma unroll
      for (int k = 0; k < NUM_FIELDS; ++k) a.rec[(int64_t)k * a.npix + i] = f[k];
      a.code[i] = code;
    }
    key = ray_bucket(code);
  }
  // class-bucket counts, one atomic per distinct bucket of the warp
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  if (key >= 0 && (threadIdx.x & 31) == (unsigned)(__ffs(grp) - 1)) atomicAdd(a.counts + key, (uint32_t)__popc(grp));
  loop_cap_end(a.flags);
}

cudaError_t launch_ray_step(const SetupArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  ray_step_kernel<<<(unsigned)((a.npix + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

// The same for every image of a batch.
__global__ void __launch_bounds__(128) batch_step_kernel(BatchArgs a) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int key = -1;
  loop_cap_begin();
  if (r < a.ntot) {
    const int im = batch_find(a.pix_off, a.nimg, r);
    const BatchImage& B = a.img[im];
    int code = a.code[r];
    if (B.ngeo > 1) {
      double f[NUM_FIELDS];
#pragma unroll
      for (int k = 0; k < NUM_FIELDS; ++k) f[k] = a.rec[(int64_t)k * a.ntot + r];
      code = step_constants<const double*>(f, code, f[F_TAUMAX] / (double)(B.ngeo - 1), f);
#pragma unroll
      for (int k = 0; k < NUM_FIELDS; ++k) a.rec[(int64_t)k * a.ntot + r] = f[k];
      a.code[r] = code;
    }
    key = im * NBUCKET + ray_bucket(code);
  }
  // bucket counts: one atomic per distinct (image, bucket) key of the warp
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  if (key >= 0 && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(a.counts + key, (uint32_t)__popc(grp));
  batch_loop_cap_end(a);
}

cudaError_t launch_batch_step(const BatchArgs& a, cudaStream_t s) {
  if (a.ntot <= 0) return cudaSuccess;
  const int block = 128;
  batch_step_kernel<<<(unsigned)((a.ntot + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

// Pi(n; phi | m) as the sample kernels' translation unit compiles it (FMA contraction on):
// form 1 = ellip_set_at (the direct sample evaluators' path), form 2 = ellip_pi_ref.
__global__ void __launch_bounds__(256) ellip_pi_samples_kernel(const double* n, const double* phi, const double* m,
                                                               int64_t N, int form, double* out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    const double ni = n[i], mi = m[i];
    if (form == 2) {
      out[i] = ellip_pi_ref(ni, phi[i], mi);
    } else {
      const EllipSet<1> comp = ellip_set_at<1>(HALFPI, mi, &ni, nullptr);
      out[i] = ellip_set_at<1>(phi[i], mi, &ni, &comp).P[0];
    }
  }
}

cudaError_t launch_ellip_pi_samples(const double* n, const double* phi, const double* m, int64_t N, int form,
                                    double* out, cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  int64_t grid = (N + 255) / 256;
  if (grid > 152 * 16) grid = 152 * 16;
  ellip_pi_samples_kernel<<<(unsigned)grid, 256, 0, s>>>(n, phi, m, N, form, out);
  return cudaGetLastError();
}

cudaError_t launch_samples(const SampleArgs& a, cudaStream_t s) {
  const int64_t total0 = a.npix * a.nsamp;
  if (total0 <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (a.tau == nullptr && a.do_phi_t && a.chunk > 0) {
    const int64_t nch_all = (a.nsamp + a.chunk - 1) / a.chunk;
    const int64_t nch = (a.c_end < 0 ? nch_all : a.c_end) - a.c_begin;
    if (nch <= 0) return cudaSuccess;
    // One item per thread, every item its own thread of the grid (launch shapes measured on
    // GB300 on 512x512 x 400 samples and 5.2 M rays x 256 samples: the FP64 kernels in
    // 128-thread blocks, 7 % faster than 256-thread blocks looping over the items of 64 blocks per
    // SM on the 5.2 M-ray image; the mixed kernel in 256-thread blocks, one per SM, its
    // float-float slots filling the shared memory). The class order of the items puts the
    // costliest first (ray_bucket).
    const int block = a.mixed ? 256 : 128;
    int64_t grid = (a.npix * nch + block - 1) / block;
    const int64_t cap = (int64_t)1 << 30;
    if (grid > cap) grid = cap;
    if (a.mixed) {
      const size_t smem = sizeof(FFRay) * block;
      if (cudaFuncSetAttribute(stepped_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem) != cudaSuccess)
        return cudaGetLastError();
      stepped_kernel<true, false><<<(unsigned)grid, block, smem, s>>>(a);
    } else if (!a.t && !a.ph && !a.sig) {
      // theta and r only: the Jacobi recurrence without E and Pi
      stepped_kernel<false, true><<<(unsigned)grid, block, 0, s>>>(a);
    } else {
      stepped_kernel<false, false><<<(unsigned)grid, block, 0, s>>>(a);
    }
    return cudaGetLastError();
  }
  const int64_t total = total0;
  const int block = 256;
  int64_t grid = (total + block - 1) / block;
  const int64_t cap = (int64_t)sms * 16;  // grid-stride beyond 16 resident-ish blocks per SM
  if (grid > cap) grid = cap;
  samples_kernel<<<(unsigned)grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// batched images: persistent kernel over the work items of every image
// ---------------------------------------------------------------------------

// A block takes tiles of `tile` consecutive work items from a global counter until the items
// run out, so images of different size and cost balance across the SMs without a host-side
// schedule. Inside an image, items are chunk-major over its class-sorted rays (as in
// stepped_kernel); a tile may span two images.
template <bool MIXED>
__global__ void __launch_bounds__(256) batch_samples_kernel(BatchArgs a) {
  __shared__ long long tile_id;
  const int64_t total = a.item_off[a.nimg];
  if (threadIdx.x == 0) kg_loop_cap_word = 0u;  // ordered by the first tile's barrier
  for (;;) {
    if (threadIdx.x == 0) tile_id = (long long)atomicAdd(a.work, 1ull);
    __syncthreads();
    const int64_t base = (int64_t)tile_id * a.tile * a.tile_skip;
    __syncthreads();
    if (base >= total) break;
    for (int64_t k = threadIdx.x; k < a.tile; k += blockDim.x) {
      const int64_t item = base + k;
      if (item >= total) break;
      const int im = batch_find(a.item_off, a.nimg, item);
      const BatchImage& B = a.img[im];
      const int64_t local = item - a.item_off[im];
      const int64_t c = local / B.npix;
      const int64_t p = __ldg(a.perm + B.pix_off + (local - c * B.npix));
      const uint32_t fl = a.flags[im];  // plain load: other blocks may OR FLAG_LOOP_CAP in
      const bool ordinary_active = (fl & FLAG_ANY_ETA_POS) != 0;
      const bool step_zero = (fl & FLAG_ANY_STEP_ZERO) != 0;
      RecView f{a.rec + p, a.ntot};
      const int code = __ldg(a.code + p);
      const int64_t g0 = c * a.chunk;
      const int64_t g1 = g0 + a.chunk < B.ngeo ? g0 + a.chunk : B.ngeo;
      const int64_t obase = B.out_off + (p - B.pix_off);
      const int64_t np = B.npix;
      auto emit = [&](int64_t g, double tau, const Sample& S) {
        const int64_t o = obase + g * np;
        if (a.t) a.t[o] = S.t;
        if (a.r) a.r[o] = S.r;
        if (a.th) a.th[o] = S.th;
        if (a.ph) a.ph[o] = S.ph;
        if (a.sig) a.sig[o] = S.sig;
        if (a.mino) a.mino[o] = tau;
      };
      if (MIXED) ray_chunk_ff(B.obs, f, code, g0, g1, B.ngeo, ordinary_active, step_zero, emit, ffray_slot());
      else ray_chunk(B.obs, f, code, g0, g1, B.ngeo, ordinary_active, step_zero, emit);
    }
    // a capped loop in this tile is charged to the images the tile spans (thread 0 clears the
    // word before the next tile's first barrier)
    __syncthreads();
    if (threadIdx.x == 0 && kg_loop_cap_word) {
      const int64_t last = base + a.tile - 1 < total ? base + a.tile - 1 : total - 1;
      const int i0 = batch_find(a.item_off, a.nimg, base), i1 = batch_find(a.item_off, a.nimg, last);
      for (int j = i0; j <= i1; ++j) atomicOr(a.flags + j, kg_loop_cap_word);
      kg_loop_cap_word = 0u;
    }
  }
}

// The mixed batch kernel's shared-memory allowance, set once per process outside any stream
// capture (kgeo_batch_create calls it).
cudaError_t prepare_batch_kernels() {
  return cudaFuncSetAttribute(batch_samples_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(FFRay) * 256));
}

cudaError_t launch_batch_samples(const BatchArgs& a, int block, int grid, cudaStream_t s) {
  if (a.mixed) batch_samples_kernel<true><<<grid, block, sizeof(FFRay) * block, s>>>(a);
  else batch_samples_kernel<false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
