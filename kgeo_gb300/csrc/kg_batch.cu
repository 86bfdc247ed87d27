// Batched tracing of many images: the plan object of the C ABI, its CUDA-graph replay and
// the autotuner that picks the sample kernel's launch shape (declarations and contracts:
// include/kgeo_gb300.h, kgeo_batch_*).
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/kgeo_gb300.h"
#include "kg_launch.h"

using namespace kg;

struct kgeo_batch_plan {
  int device = 0;
  int sms = 152;
  int precision = KGEO_PRECISION_FP64;
  int nimg = 0;
  int64_t ntot = 0;         // rays
  int64_t nsamp_tot = 0;    // samples of every image (sum of ngeo * npix)
  std::vector<BatchImage> img;
  std::vector<int64_t> pix_off;
  // device copies of the tables (owned)
  BatchImage* d_img = nullptr;
  int64_t* d_pix_off = nullptr;
  // bound buffers (caller-owned)
  BatchArgs args{};
  uint32_t* user_flags = nullptr;  // (nimg) per-image flags words of the caller, or NULL
  bool bound = false;
  // launch shape
  kgeo_batch_config cfg{};
  bool tuned = false;
  // graph of the whole pipeline for the bound buffers and cfg
  cudaGraphExec_t exec = nullptr;
  kgeo_batch_config graph_cfg{};
};

namespace {

int check_obs(double a, double r_o, double th_o) {
  if (!(std::fabs(a) >= 0 && std::fabs(a) < 1)) return KGEO_ERR_SPIN;
  if (!(r_o >= 100)) return KGEO_ERR_R_O;
  if (!(th_o > 0 && th_o < PI && th_o != 0.5 * PI)) return KGEO_ERR_TH_O;
  return KGEO_OK;
}

Observer host_observer(double a, double r_o, double th_o) {
  Observer ob;
  ob.a = a;
  ob.a2 = a * a;
  ob.r_o = r_o;
  ob.th_o = th_o;
  ob.sin_th = std::sin(th_o);
  ob.cos_th = std::cos(th_o);
  ob.cos2 = ob.cos_th * ob.cos_th;
  double root = std::sqrt(1 - ob.a2);
  ob.rplus = 1 + root;
  ob.rminus = 1 - root;
  ob.minspin = std::fabs(a) < MINSPIN;
  ob.r_o_inf = std::isinf(r_o) ? 1 : 0;
  return ob;
}

// Workspace layout of a plan: records, codes, permutation, then the words that every run
// clears with one memset (bucket counts and cursors, per-image flags, the work counter),
// then the item offsets.
struct BatchLayout {
  size_t rec, code, perm, clear, clear_bytes, item_off, total;
};

BatchLayout layout(int64_t ntot, int nimg) {
  BatchLayout L;
  const size_t n = (size_t)(ntot > 0 ? ntot : 1);
  size_t o = 0;
  L.rec = o;
  o += align_up(sizeof(double) * NUM_FIELDS * n, 256);
  L.code = o;
  o += align_up(sizeof(int) * n, 256);
  L.perm = o;
  o += align_up(sizeof(int) * n, 256);
  L.clear = o;
  // counts + cursors (uint32), flags (uint32), padding to 8, work counter (u64)
  L.clear_bytes = align_up(sizeof(uint32_t) * (2 * (size_t)nimg * NBUCKET + nimg), 8) + sizeof(unsigned long long);
  o += align_up(L.clear_bytes, 256);
  L.item_off = o;
  o += align_up(sizeof(int64_t) * ((size_t)nimg + 1), 256);
  L.total = o;
  return L;
}

// Default launch shape: tiles of one item per thread (on the 64-image batch, full runs on GB300:
// mixed 2112 ms with tiles of 256 items against 2452 ms with 1024 and 2614 ms with 2048;
// FP64 2821 ms with two 256-thread blocks per SM against 3028 ms with one and tiles of 1024).
kgeo_batch_config default_config(const kgeo_batch_plan* p) {
  const bool mixed = p->precision == KGEO_PRECISION_MIXED;
  kgeo_batch_config c;
  c.block = 256;
  c.ctas_per_sm = mixed ? 1 : 2;
  c.tile = 256;
  c.chunk = mixed ? DEFAULT_CHUNK_MIXED : DEFAULT_CHUNK;
  return c;
}

bool valid_config(const kgeo_batch_plan* p, const kgeo_batch_config& c) {
  const int maxc = p->precision == KGEO_PRECISION_MIXED ? MAX_CHUNK_MIXED : MAX_CHUNK;
  return (c.block == 128 || c.block == 256) && c.ctas_per_sm >= 1 && c.ctas_per_sm <= 4 && c.tile >= c.block &&
         c.tile % c.block == 0 && c.chunk >= 1 && c.chunk <= maxc;
}

// The autotuner's cache: the only global state of the library (mutex-guarded). Key: device
// SM count, precision and every image's (npix, ngeo).
std::mutex g_tune_mu;
std::map<std::string, kgeo_batch_config> g_tune_cache;

std::string signature(const kgeo_batch_plan* p) {
  std::string s = std::to_string(p->sms) + ":" + std::to_string(p->precision);
  for (const BatchImage& b : p->img) s += ":" + std::to_string(b.npix) + "x" + std::to_string(b.ngeo);
  return s;
}

// The whole pipeline for one launch shape: clear, item offsets, setup, sort, samples.
// tile_skip > 1 runs every tile_skip-th tile of the sample kernel (autotuner timing).
int run_pipeline(kgeo_batch_plan* p, const kgeo_batch_config& c, int tile_skip, cudaStream_t s, bool setup = true) {
  BatchArgs a = p->args;
  a.chunk = c.chunk;
  a.tile = c.tile;
  a.tile_skip = tile_skip;
  a.mixed = p->precision == KGEO_PRECISION_MIXED;
  const size_t words = 2 * (size_t)p->nimg * NBUCKET + p->nimg;
  char* clear = reinterpret_cast<char*>(a.counts);
  const size_t clear_bytes = align_up(sizeof(uint32_t) * words, 8) + sizeof(unsigned long long);
  if (setup) {
    if (cudaMemsetAsync(clear, 0, clear_bytes, s) != cudaSuccess) return KGEO_ERR_CUDA;
    if (launch_batch_setup(a, s) != cudaSuccess) return KGEO_ERR_CUDA;
  } else {
    // re-run of the sample kernel alone: new item offsets for this chunk, work counter reset
    if (cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s) != cudaSuccess) return KGEO_ERR_CUDA;
    BatchArgs b = a;
    b.ntot = 0;  // item offsets only
    if (launch_batch_setup(b, s) != cudaSuccess) return KGEO_ERR_CUDA;
  }
  if (p->nsamp_tot > 0) {
    const int grid = p->sms * c.ctas_per_sm;
    if (launch_batch_samples(a, c.block, grid, s) != cudaSuccess) return KGEO_ERR_CUDA;
  }
  if (tile_skip == 1 && p->user_flags &&
      cudaMemcpyAsync(p->user_flags, a.flags, sizeof(uint32_t) * p->nimg, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return KGEO_ERR_CUDA;
  return KGEO_OK;
}

void drop_graph(kgeo_batch_plan* p) {
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
}

}  // namespace

extern "C" {

int kgeo_batch_create(const kgeo_batch_image* images, int32_t nimg, int32_t precision, kgeo_batch_plan** out) {
  if (!out) return KGEO_ERR_NULL;
  *out = nullptr;
  if (nimg < 0 || nimg > KGEO_BATCH_MAX_IMAGES) return KGEO_ERR_LENGTHS;
  if (nimg > 0 && !images) return KGEO_ERR_NULL;
  if (precision != KGEO_PRECISION_FP64 && precision != KGEO_PRECISION_MIXED) return KGEO_ERR_MODEL;
  if (prepare_batch_kernels() != cudaSuccess) return KGEO_ERR_CUDA;
  kgeo_batch_plan* p = new kgeo_batch_plan();
  p->precision = precision;
  p->nimg = nimg;
  cudaGetDevice(&p->device);
  cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device);
  int64_t off = 0, soff = 0;
  for (int i = 0; i < nimg; ++i) {
    const kgeo_batch_image& m = images[i];
    int st = check_obs(m.a, m.r_o, m.th_o);
    if (!st && m.npix < 0) st = KGEO_ERR_LENGTHS;
    if (!st && m.ngeo < 0) st = KGEO_ERR_NGEO;
    if (st) {
      delete p;
      return st;
    }
    BatchImage b;
    b.obs = host_observer(m.a, m.r_o, m.th_o);
    b.pix_off = off;
    b.npix = m.npix;
    b.ngeo = m.ngeo;
    b.out_off = soff;
    b.maxtaufrac = m.maxtaufrac;
    p->img.push_back(b);
    p->pix_off.push_back(off);
    off += m.npix;
    soff += m.npix * (int64_t)m.ngeo;
  }
  p->pix_off.push_back(off);
  if (off >= ((int64_t)1 << 31)) {
    delete p;
    return KGEO_ERR_LENGTHS;
  }
  p->ntot = off;
  p->nsamp_tot = soff;
  if (nimg > 0) {
    if (cudaMalloc(&p->d_img, sizeof(BatchImage) * nimg) != cudaSuccess ||
        cudaMalloc(&p->d_pix_off, sizeof(int64_t) * (nimg + 1)) != cudaSuccess ||
        cudaMemcpy(p->d_img, p->img.data(), sizeof(BatchImage) * nimg, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->d_pix_off, p->pix_off.data(), sizeof(int64_t) * (nimg + 1), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      kgeo_batch_destroy(p);
      return KGEO_ERR_CUDA;
    }
  }
  p->cfg = default_config(p);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(signature(p));
    if (it != g_tune_cache.end()) {
      p->cfg = it->second;
      p->tuned = true;
    }
  }
  *out = p;
  return KGEO_OK;
}

void kgeo_batch_destroy(kgeo_batch_plan* p) {
  if (!p) return;
  drop_graph(p);
  if (p->d_img) cudaFree(p->d_img);
  if (p->d_pix_off) cudaFree(p->d_pix_off);
  delete p;
}

int kgeo_batch_sizes(const kgeo_batch_plan* p, int64_t* n_rays, int64_t* n_samples, size_t* workspace_bytes) {
  if (!p) return KGEO_ERR_NULL;
  if (n_rays) *n_rays = p->ntot;
  if (n_samples) *n_samples = p->nsamp_tot;
  if (workspace_bytes) *workspace_bytes = layout(p->ntot, p->nimg).total;
  return KGEO_OK;
}

int kgeo_batch_bind(kgeo_batch_plan* p, const double* alpha, const double* beta, kgeo_geodesics* out,
                    void* workspace, size_t workspace_bytes) {
  if (!p || !out) return KGEO_ERR_NULL;
  const BatchLayout L = layout(p->ntot, p->nimg);
  if (!workspace) return KGEO_ERR_NULL;
  if (workspace_bytes < L.total) return KGEO_ERR_WORKSPACE;
  if (p->ntot > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  char* w = static_cast<char*>(workspace);
  BatchArgs& a = p->args;
  a.img = p->d_img;
  a.pix_off = p->d_pix_off;
  a.item_off = reinterpret_cast<int64_t*>(w + L.item_off);
  a.nimg = p->nimg;
  a.ntot = p->ntot;
  a.alpha = alpha;
  a.beta = beta;
  a.rec = reinterpret_cast<double*>(w + L.rec);
  a.code = reinterpret_cast<int*>(w + L.code);
  a.perm = reinterpret_cast<int*>(w + L.perm);
  a.counts = reinterpret_cast<uint32_t*>(w + L.clear);
  a.flags = a.counts + 2 * (size_t)p->nimg * NBUCKET;
  a.work = reinterpret_cast<unsigned long long*>(
      w + L.clear + align_up(sizeof(uint32_t) * (2 * (size_t)p->nimg * NBUCKET + p->nimg), 8));
  a.rclass = out->rclass;
  a.thclass = out->thclass;
  a.tau_tot = out->tau_tot;
  a.t = out->t;
  a.r = out->r;
  a.th = out->th;
  a.ph = out->ph;
  a.sig = out->sig;
  a.mino = out->mino;
  p->user_flags = out->flags;
  p->bound = true;
  drop_graph(p);
  return KGEO_OK;
}

int kgeo_batch_get_config(const kgeo_batch_plan* p, kgeo_batch_config* cfg, int32_t* tuned) {
  if (!p || !cfg) return KGEO_ERR_NULL;
  *cfg = p->cfg;
  if (tuned) *tuned = p->tuned ? 1 : 0;
  return KGEO_OK;
}

int kgeo_batch_set_config(kgeo_batch_plan* p, const kgeo_batch_config* cfg) {
  if (!p || !cfg) return KGEO_ERR_NULL;
  if (!valid_config(p, *cfg)) return KGEO_ERR_MODEL;
  p->cfg = *cfg;
  drop_graph(p);
  return KGEO_OK;
}

int kgeo_batch_run(kgeo_batch_plan* p, void* stream) {
  if (!p) return KGEO_ERR_NULL;
  if (!p->bound) return KGEO_ERR_NULL;
  if (p->nimg == 0) return KGEO_OK;
  return run_pipeline(p, p->cfg, 1, static_cast<cudaStream_t>(stream));
}

int kgeo_batch_autotune(kgeo_batch_plan* p, int32_t budget_ms, void* stream, kgeo_batch_config* best) {
  if (!p) return KGEO_ERR_NULL;
  if (!p->bound) return KGEO_ERR_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->nimg == 0 || p->nsamp_tot == 0) {
    if (best) *best = p->cfg;
    return KGEO_OK;
  }
  // candidates: block size x CTAs per SM x chunk length, tiles of one item per thread. Full
  // runs of the 64-image batch on GB300 set the list: tiles longer than a block were 16-24 %
  // slower; mixed chunks of 64 samples 6 % slower than 128 (every chunk starts with an FP64
  // direct evaluation, which GB300 runs at 1/64 of the FP32 rate), 128 within 2 % of 256; FP64
  // chunks of 50 4 % slower than 64. The tuner's sparse subset of tiles cannot resolve a few per
  // cent, so the list holds only shapes within a few per cent of the best full run.
  std::vector<kgeo_batch_config> cands;
  const bool mixed = p->precision == KGEO_PRECISION_MIXED;
  const int shapes_m[][3] = {{256, 1, 256}, {256, 1, 128}, {128, 2, 256}};
  const int shapes_d[][3] = {{256, 2, 64}, {128, 2, 64}, {128, 4, 64}, {256, 1, 64}};
  const int nshape = mixed ? 3 : 4;
  for (int k = 0; k < nshape; ++k) {
    const int* sh = mixed ? shapes_m[k] : shapes_d[k];
    kgeo_batch_config c;
    c.block = sh[0];
    c.ctas_per_sm = sh[1];
    c.tile = sh[0];
    c.chunk = sh[2];
    if (valid_config(p, c)) cands.push_back(c);
  }
  // setup once; each candidate then times its sample kernel on every S-th tile, S chosen so
  // that a candidate costs about budget / (number of candidates)
  int st = run_pipeline(p, p->cfg, 1 << 20, s);
  if (st) return st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // probe: the default shape on every 64th tile
  int skip = 64;
  float ms = 0.f;
  cudaEventRecord(e0, s);
  st = run_pipeline(p, p->cfg, skip, s, false);
  cudaEventRecord(e1, s);
  if (!st && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  const double per = (budget_ms > 0 ? budget_ms : 2000) / (double)cands.size();
  if (!st && ms > 0) {
    double want = per / ms;  // how much more work than the probe each candidate may do
    int sk = (int)(skip / (want > 1 ? want : 1));
    skip = sk < 1 ? 1 : (sk > 4096 ? 4096 : sk);
  }
  kgeo_batch_config bestc = p->cfg;
  float best_ms = 1e30f;
  for (const kgeo_batch_config& c : cands) {
    if (st) break;
    // warm-up on a sparser subset, then the timed run
    st = run_pipeline(p, c, skip * 4, s, false);
    if (st) break;
    cudaEventRecord(e0, s);
    st = run_pipeline(p, c, skip, s, false);
    cudaEventRecord(e1, s);
    if (st || cudaEventSynchronize(e1) != cudaSuccess) {
      st = st ? st : KGEO_ERR_CUDA;
      break;
    }
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (t < best_ms) {
      best_ms = t;
      bestc = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  p->cfg = bestc;
  p->tuned = true;
  drop_graph(p);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[signature(p)] = bestc;
  }
  if (best) *best = bestc;
  return KGEO_OK;
}

int kgeo_batch_graph_launch(kgeo_batch_plan* p, void* stream) {
  if (!p) return KGEO_ERR_NULL;
  if (!p->bound) return KGEO_ERR_NULL;
  if (p->nimg == 0) return KGEO_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->exec && std::memcmp(&p->graph_cfg, &p->cfg, sizeof(kgeo_batch_config)) != 0) drop_graph(p);
  if (!p->exec) {
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return KGEO_ERR_CUDA;
    cudaGraph_t g = nullptr;
    int st = KGEO_OK;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) st = KGEO_ERR_CUDA;
    if (!st) {
      const int rs = run_pipeline(p, p->cfg, 1, cap);
      if (cudaStreamEndCapture(cap, &g) != cudaSuccess || rs) st = rs ? rs : KGEO_ERR_CUDA;
    }
    if (!st && cudaGraphInstantiate(&p->exec, g, 0) != cudaSuccess) st = KGEO_ERR_CUDA;
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cap);
    if (st) {
      p->exec = nullptr;
      return st;
    }
    p->graph_cfg = p->cfg;
  }
  return cudaGraphLaunch(p->exec, s) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

}  // extern "C"
