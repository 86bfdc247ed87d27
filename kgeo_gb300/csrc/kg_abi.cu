// C ABI of the kgeo GB300 tracer (declarations and contracts: include/kgeo_gb300.h).
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/kgeo_gb300.h"

#include "kg_launch.h"

using namespace kg;

static_assert(KGEO_FLAG_LOOP_CAP == kg::FLAG_LOOP_CAP, "flag bit of the C ABI and the kernels differ");

namespace {

// Observer checks with the reference's rules (kgeo/kerr_raytracing_ana.py:59-65).
int check_observer(const kgeo_observer* o) {
  if (!o) return KGEO_ERR_NULL;
  if (!(std::fabs(o->a) >= 0 && std::fabs(o->a) < 1)) return KGEO_ERR_SPIN;
  if (!(o->r_o >= 100)) return KGEO_ERR_R_O;
  if (!(o->th_o > 0 && o->th_o < PI && o->th_o != 0.5 * PI)) return KGEO_ERR_TH_O;
  return KGEO_OK;
}

// Per-image constants with the host libm, as numpy computes them for a Python float.
Observer make_observer(const kgeo_observer* o) {
  Observer ob;
  ob.a = o->a;
  ob.a2 = o->a * o->a;
  ob.r_o = o->r_o;
  ob.th_o = o->th_o;
  ob.sin_th = std::sin(o->th_o);
  ob.cos_th = std::cos(o->th_o);
  ob.cos2 = ob.cos_th * ob.cos_th;
  double root = std::sqrt(1 - ob.a2);
  ob.rplus = 1 + root;
  ob.rminus = 1 - root;
  ob.minspin = std::fabs(o->a) < MINSPIN;
  ob.r_o_inf = std::isinf(o->r_o) ? 1 : 0;
  return ob;
}

struct Scratch {
  void* ptr = nullptr;
  bool owned = false;
  cudaStream_t s = nullptr;
  ~Scratch() {
    if (owned && ptr) cudaFreeAsync(ptr, s);
  }
};

int get_scratch(Scratch& sc, void* workspace, size_t bytes, int64_t npix, cudaStream_t s) {
  size_t need = workspace_bytes(npix);
  sc.s = s;
  if (workspace) {
    if (bytes < need) return KGEO_ERR_WORKSPACE;
    sc.ptr = workspace;
    return KGEO_OK;
  }
  if (cudaMallocAsync(&sc.ptr, need, s) != cudaSuccess) return KGEO_ERR_CUDA;
  sc.owned = true;
  return KGEO_OK;
}

int setup_common(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix, int64_t ngeo,
                 double maxtaufrac, const Workspace& w, kgeo_geodesics* out, cudaStream_t s) {
  // counters and flags are adjacent: one memset clears both
  if (cudaMemsetAsync(w.counts, 0, sizeof(uint32_t) * (2 * NBUCKET + 1), s) != cudaSuccess) return KGEO_ERR_CUDA;
  if (npix == 0) return KGEO_OK;
  SetupArgs sa;
  sa.obs = make_observer(obs);
  sa.alpha = alpha;
  sa.beta = beta;
  sa.npix = npix;
  sa.ngeo = ngeo;
  sa.maxtaufrac = maxtaufrac;
  sa.rec = w.rec;
  sa.code = w.code;
  sa.rclass = out ? out->rclass : nullptr;
  sa.thclass = out ? out->thclass : nullptr;
  sa.tau_tot = out ? out->tau_tot : nullptr;
  sa.flags = w.flags;
  sa.counts = w.counts;
  sa.perm = w.perm;
  return launch_ray_setup(sa, s) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int samples_common(const kgeo_observer* obs, const Workspace& w, int64_t npix, int64_t nsamp, const double* tau,
                   int do_phi_t, int chunk, int mixed, kgeo_geodesics* out, cudaStream_t s) {
  if (npix > 0) {
    SampleArgs pa;
    pa.obs = make_observer(obs);
    pa.rec = w.rec;
    pa.code = w.code;
    pa.npix = npix;
    pa.nsamp = nsamp;
    pa.tau = tau;
    pa.do_phi_t = do_phi_t;
    if (mixed)
      pa.chunk = chunk < 0 ? DEFAULT_CHUNK_MIXED : (chunk > MAX_CHUNK_MIXED ? MAX_CHUNK_MIXED : chunk);
    else
      pa.chunk = chunk < 0 ? DEFAULT_CHUNK : (chunk > MAX_CHUNK ? MAX_CHUNK : chunk);
    pa.perm = w.perm;
    pa.mixed = mixed;
    pa.c_begin = 0;
    pa.c_end = -1;
    pa.row0 = 0;
    pa.flags = w.flags;
    pa.t = out->t;
    pa.r = out->r;
    pa.th = out->th;
    pa.ph = out->ph;
    pa.sig = out->sig;
    pa.mino = out->mino;
    if (launch_samples(pa, s) != cudaSuccess) return KGEO_ERR_CUDA;
  }
  if (out->flags &&
      cudaMemcpyAsync(out->flags, w.flags, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return KGEO_ERR_CUDA;
  return KGEO_OK;
}

int trace_common(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                 int64_t nsamp, const double* tau, int do_phi_t, double maxtaufrac, kgeo_geodesics* out,
                 void* workspace, size_t workspace_bytes_, void* stream, int mixed = 0) {
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (nsamp < 0) return KGEO_ERR_NGEO;
  if (!out) return KGEO_ERR_NULL;
  if (npix > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch sc;
  st = get_scratch(sc, workspace, workspace_bytes_, npix, s);
  if (st) return st;
  Workspace w = carve_workspace(sc.ptr, npix);
  st = setup_common(obs, alpha, beta, npix, tau ? 0 : nsamp, maxtaufrac, w, out, s);
  if (st) return st;
  return samples_common(obs, w, npix, nsamp, tau, do_phi_t, -1, mixed, out, s);
}

// Emission model with the reference's parameter checks (kgeo/velocities.py:315-317,
// 446-451: fac_subkep, beta_phi, beta_r in [0, 1]).
int make_model(const kgeo_emission* m, EmissionModel* out) {
  if (!m) return KGEO_ERR_NULL;
  if (m->emissivity < KGEO_EMIS_BPL || m->emissivity > KGEO_EMIS_RING) return KGEO_ERR_MODEL;
  if (m->velocity < KGEO_VEL_ZAMO || m->velocity > KGEO_VEL_GENERAL) return KGEO_ERR_MODEL;
  const int nv = m->velocity == KGEO_VEL_SUBKEP ? 1 : (m->velocity == KGEO_VEL_GENERAL ? 3 : 0);
  for (int k = 0; k < nv; ++k)
    if (!(m->vel_p[k] >= 0 && m->vel_p[k] <= 1)) return KGEO_ERR_MODEL;
  out->emis = m->emissivity;
  out->vel = m->velocity;
  out->retrograde = m->retrograde != 0;
  for (int k = 0; k < 2; ++k) out->emis_p[k] = m->emis_p[k];
  for (int k = 0; k < 3; ++k) out->vel_p[k] = m->vel_p[k];
  out->mu_ring = m->mu_ring;
  out->emiscut_in = m->emiscut_in;
  out->emiscut_out = m->emiscut_out;
  out->specind = m->specind;
  out->sinthb = m->sinthb;
  out->sinthb_pow = std::pow(m->sinthb, 1 + m->specind);
  return KGEO_OK;
}

// Image options (NULL: unpolarised, no path length). Field coefficients must be finite;
// 'simple' fields need a non-zero coefficient (kgeo/bfields.py:87-91).
int make_options(const kgeo_image_options* p, ImageOptions* out) {
  out->polarization = 0;
  out->pathlength = 0;
  out->diskangle = 0.1;
  out->field = FieldModel{0, 0, {0.0, 0.0, 0.0}};
  if (!p) return KGEO_OK;
  out->polarization = p->polarization != 0;
  out->pathlength = p->pathlength != 0;
  if (out->pathlength && !std::isfinite(p->diskangle)) return KGEO_ERR_MODEL;
  out->diskangle = p->diskangle;
  if (out->polarization) {
    const kgeo_bfield& b = p->bfield;
    if (b.field < KGEO_BFIELD_SIMPLE || b.field > KGEO_BFIELD_GEN_POWER) return KGEO_ERR_MODEL;
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(b.c[k])) return KGEO_ERR_MODEL;
    if ((b.field == KGEO_BFIELD_SIMPLE || b.field == KGEO_BFIELD_SIMPLE_RM1) && b.c[0] == 0 && b.c[1] == 0 &&
        b.c[2] == 0)
      return KGEO_ERR_MODEL;
    out->field.field = b.field;
    out->field.flag = b.flag != 0;
    for (int k = 0; k < 3; ++k) out->field.c[k] = b.c[k];
  }
  return KGEO_OK;
}

// ---------------------------------------------------------------------------
// host-buffer raytrace: windows of whole recurrence chunks computed into a ring of device
// buffers while the previous windows are copied to the host on a second stream
// ---------------------------------------------------------------------------
constexpr int HOST_RING = 4;      // device window buffers in flight (two computing, two copying)
constexpr int HOST_WINDOWS = 8;   // target number of windows per call

struct HostPlan {
  int64_t chunk, nch, wch, nwin;
  size_t n, base, io, slot, total;
};

HostPlan host_plan(int64_t npix, int64_t ngeo, int mixed) {
  HostPlan h;
  h.chunk = mixed ? DEFAULT_CHUNK_MIXED : DEFAULT_CHUNK;
  h.nch = ngeo > 0 ? (ngeo + h.chunk - 1) / h.chunk : 0;
  h.wch = h.nch > 0 ? (h.nch + HOST_WINDOWS - 1) / HOST_WINDOWS : 1;
  h.nwin = h.nch > 0 ? (h.nch + h.wch - 1) / h.wch : 0;
  h.n = (size_t)(npix > 0 ? npix : 1);
  h.base = workspace_bytes(npix);
  h.io = 2 * align_up(sizeof(double) * h.n, 256) + align_up(sizeof(double) * h.n, 256) +
         2 * align_up(sizeof(int32_t) * h.n, 256);
  h.slot = 6 * align_up(sizeof(double) * h.n * (size_t)(h.wch * h.chunk), 256);
  h.total = h.base + h.io + (size_t)HOST_RING * h.slot;
  return h;
}

// The copy stream, a second compute stream and the ring's events; destroying them while
// work is queued is allowed (the driver releases them when that work completes).
struct HostPipe {
  cudaStream_t cs = nullptr;  // device-to-host copies
  cudaStream_t s2 = nullptr;  // odd windows: a window's last blocks overlap the next window's first
  cudaEvent_t done[HOST_RING] = {}, copied[HOST_RING] = {}, setup = nullptr, s2_end = nullptr;
  bool ok = false;
  HostPipe() {
    ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
         cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&setup, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&s2_end, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < HOST_RING && ok; ++k)
      ok = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&copied[k], cudaEventDisableTiming) == cudaSuccess;
  }
  ~HostPipe() {
    for (int k = 0; k < HOST_RING; ++k) {
      if (done[k]) cudaEventDestroy(done[k]);
      if (copied[k]) cudaEventDestroy(copied[k]);
    }
    if (setup) cudaEventDestroy(setup);
    if (s2_end) cudaEventDestroy(s2_end);
    if (cs) cudaStreamDestroy(cs);
    if (s2) cudaStreamDestroy(s2);
  }
};

// Device address of host memory the device can write directly (page-locked and mapped into the
// unified address space); false for pageable memory (or a pointer the runtime does not know).
bool device_view(const void* host, void** dev) {
  if (!host) {
    *dev = nullptr;
    return true;
  }
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return false;
  *dev = at.devicePointer;
  return true;
}

int raytrace_host(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix, int64_t ngeo,
                  double maxtaufrac, int mixed, kgeo_geodesics* out, void* workspace, size_t workspace_bytes_,
                  cudaStream_t s) {
  const HostPlan h = host_plan(npix, ngeo, mixed);
  Scratch sc;
  sc.s = s;
  if (workspace) {
    if (workspace_bytes_ < h.total) return KGEO_ERR_WORKSPACE;
    sc.ptr = workspace;
  } else {
    if (cudaMallocAsync(&sc.ptr, h.total, s) != cudaSuccess) return KGEO_ERR_CUDA;
    sc.owned = true;
  }
  char* p = static_cast<char*>(sc.ptr);
  Workspace w = carve_workspace(p, npix);
  p += h.base;
  double* al = reinterpret_cast<double*>(p);
  p += align_up(sizeof(double) * h.n, 256);
  double* be = reinterpret_cast<double*>(p);
  p += align_up(sizeof(double) * h.n, 256);
  double* tau_tot = reinterpret_cast<double*>(p);
  p += align_up(sizeof(double) * h.n, 256);
  int32_t* rclass = reinterpret_cast<int32_t*>(p);
  p += align_up(sizeof(int32_t) * h.n, 256);
  int32_t* thclass = reinterpret_cast<int32_t*>(p);
  p += align_up(sizeof(int32_t) * h.n, 256);
  char* ring = p;
  const size_t bytes_px = sizeof(double) * (size_t)npix;
  if (npix > 0) {
    if (cudaMemcpyAsync(al, alpha, bytes_px, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(be, beta, bytes_px, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return KGEO_ERR_CUDA;
  }
  kgeo_geodesics per{};
  per.tau_tot = tau_tot;
  per.rclass = rclass;
  per.thclass = thclass;
  int st = setup_common(obs, al, be, npix, ngeo, maxtaufrac, w, &per, s);
  if (st) return st;
  // the sample outputs as device addresses, when the host buffers allow it
  void* dv[6];
  const double* const hv[6] = {out->t, out->r, out->th, out->ph, out->sig, out->mino};
  bool direct = true;
  for (int j = 0; j < 6; ++j) direct = direct && device_view(hv[j], &dv[j]);
  if (direct) {
    kgeo_geodesics dout{};
    dout.t = static_cast<double*>(dv[0]);
    dout.r = static_cast<double*>(dv[1]);
    dout.th = static_cast<double*>(dv[2]);
    dout.ph = static_cast<double*>(dv[3]);
    dout.sig = static_cast<double*>(dv[4]);
    dout.mino = static_cast<double*>(dv[5]);
    st = samples_common(obs, w, npix, ngeo, nullptr, 1, -1, mixed, &dout, s);
    if (st) return st;
    bool fail = false;
    if (npix > 0)
      fail = (out->tau_tot && cudaMemcpyAsync(out->tau_tot, tau_tot, bytes_px, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
             (out->rclass && cudaMemcpyAsync(out->rclass, rclass, sizeof(int32_t) * (size_t)npix,
                                             cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
             (out->thclass && cudaMemcpyAsync(out->thclass, thclass, sizeof(int32_t) * (size_t)npix,
                                              cudaMemcpyDeviceToHost, s) != cudaSuccess);
    if (!fail && out->flags)
      fail = cudaMemcpyAsync(out->flags, w.flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess;
    return fail ? KGEO_ERR_CUDA : KGEO_OK;
  }
  HostPipe pipe;
  if (!pipe.ok) return KGEO_ERR_CUDA;
  double* const host_out[6] = {out->t, out->r, out->th, out->ph, out->sig, out->mino};
  const size_t slot_arr = align_up(sizeof(double) * h.n * (size_t)(h.wch * h.chunk), 256);
  int last = -1;
  bool fail = cudaEventRecord(pipe.setup, s) != cudaSuccess || cudaStreamWaitEvent(pipe.s2, pipe.setup, 0) != cudaSuccess;
  for (int64_t wi = 0; npix > 0 && wi < h.nwin && !fail; ++wi) {
    const int k = (int)(wi % HOST_RING);
    cudaStream_t cw = (wi & 1) ? pipe.s2 : s;
    const int64_t cb = wi * h.wch;
    const int64_t ce = cb + h.wch < h.nch ? cb + h.wch : h.nch;
    const int64_t g0 = cb * h.chunk;
    const int64_t g1 = ce * h.chunk < ngeo ? ce * h.chunk : ngeo;
    double* slot[6];
    for (int j = 0; j < 6; ++j) slot[j] = reinterpret_cast<double*>(ring + (size_t)k * h.slot + (size_t)j * slot_arr);
    if (wi >= HOST_RING && cudaStreamWaitEvent(cw, pipe.copied[k], 0) != cudaSuccess) {
      fail = true;
      break;
    }
    SampleArgs pa;
    pa.obs = make_observer(obs);
    pa.rec = w.rec;
    pa.code = w.code;
    pa.npix = npix;
    pa.nsamp = ngeo;
    pa.tau = nullptr;
    pa.do_phi_t = 1;
    pa.chunk = (int)h.chunk;
    pa.perm = w.perm;
    pa.mixed = mixed;
    pa.c_begin = cb;
    pa.c_end = ce;
    pa.row0 = g0;
    pa.flags = w.flags;
    pa.t = slot[0];
    pa.r = slot[1];
    pa.th = slot[2];
    pa.ph = slot[3];
    pa.sig = slot[4];
    pa.mino = slot[5];
    if (launch_samples(pa, cw) != cudaSuccess || cudaEventRecord(pipe.done[k], cw) != cudaSuccess ||
        cudaStreamWaitEvent(pipe.cs, pipe.done[k], 0) != cudaSuccess) {
      fail = true;
      break;
    }
    for (int j = 0; j < 6 && !fail; ++j)
      fail = host_out[j] && cudaMemcpyAsync(host_out[j] + g0 * npix, slot[j], bytes_px * (size_t)(g1 - g0),
                                            cudaMemcpyDeviceToHost, pipe.cs) != cudaSuccess;
    if (cudaEventRecord(pipe.copied[k], pipe.cs) != cudaSuccess) fail = true;
    else last = k;
  }
  if (!fail && npix > 0) {
    fail = (out->tau_tot && cudaMemcpyAsync(out->tau_tot, tau_tot, bytes_px, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
           (out->rclass && cudaMemcpyAsync(out->rclass, rclass, sizeof(int32_t) * (size_t)npix,
                                           cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
           (out->thclass && cudaMemcpyAsync(out->thclass, thclass, sizeof(int32_t) * (size_t)npix,
                                            cudaMemcpyDeviceToHost, s) != cudaSuccess);
  }
  if (!fail && out->flags)
    fail = cudaMemcpyAsync(out->flags, w.flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess;
  // join before anything else is queued on s (also on failure, so that the scratch is freed
  // only after the kernels and copies that use it): the copy stream is in order, its last
  // event covers every copy; s2_end covers the odd windows' kernels
  if (cudaEventRecord(pipe.s2_end, pipe.s2) != cudaSuccess || cudaStreamWaitEvent(s, pipe.s2_end, 0) != cudaSuccess)
    fail = true;
  if (last >= 0 && cudaStreamWaitEvent(s, pipe.copied[last], 0) != cudaSuccess) fail = true;
  return fail ? KGEO_ERR_CUDA : KGEO_OK;
}

}  // namespace

extern "C" {

size_t kgeo_workspace_size(int64_t npix) { return workspace_bytes(npix); }

int kgeo_raytrace(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                  int32_t ngeo, double maxtaufrac, kgeo_geodesics* out, void* workspace,
                  size_t workspace_bytes_, void* stream) {
  return trace_common(obs, alpha, beta, npix, ngeo, nullptr, 1, maxtaufrac, out, workspace, workspace_bytes_,
                      stream);
}

size_t kgeo_raytrace_host_workspace_size(int64_t npix, int32_t ngeo, int32_t precision) {
  return host_plan(npix, ngeo, precision == KGEO_PRECISION_MIXED).total;
}

int kgeo_raytrace_host(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                       int32_t ngeo, double maxtaufrac, int32_t precision, kgeo_geodesics* out, void* workspace,
                       size_t workspace_bytes_, void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (ngeo < 0) return KGEO_ERR_NGEO;
  if (precision != KGEO_PRECISION_FP64 && precision != KGEO_PRECISION_MIXED) return KGEO_ERR_MODEL;
  if (!out) return KGEO_ERR_NULL;
  if (npix > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  return raytrace_host(obs, alpha, beta, npix, ngeo, maxtaufrac, precision == KGEO_PRECISION_MIXED, out, workspace,
                       workspace_bytes_, static_cast<cudaStream_t>(stream));
}

int kgeo_raytrace_mixed(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                        int32_t ngeo, double maxtaufrac, kgeo_geodesics* out, void* workspace,
                        size_t workspace_bytes_, void* stream) {
  return trace_common(obs, alpha, beta, npix, ngeo, nullptr, 1, maxtaufrac, out, workspace, workspace_bytes_,
                      stream, 1);
}

int kgeo_coords_at_tau(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                       const double* tau, int32_t ntau, int32_t do_phi_and_t, kgeo_geodesics* out,
                       void* workspace, size_t workspace_bytes_, void* stream) {
  if (ntau > 0 && npix > 0 && !tau) return KGEO_ERR_NULL;
  return trace_common(obs, alpha, beta, npix, ntau, tau, do_phi_and_t ? 1 : 0, 1.0, out, workspace,
                      workspace_bytes_, stream);
}

int kgeo_r_equatorial(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha,
                      const double* beta, int64_t npix, double* r_s, double* Ir, double* Imax, double* Nmax,
                      void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (mbar_lo < 0 || n_orders < 0) return KGEO_ERR_MBAR;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (npix > 0 && (!alpha || !beta || (n_orders > 0 && (!r_s || !Ir)))) return KGEO_ERR_NULL;
  EquatorialArgs ea;
  ea.obs = make_observer(obs);
  ea.alpha = alpha;
  ea.beta = beta;
  ea.npix = npix;
  ea.mbar_lo = mbar_lo;
  ea.nord = n_orders;
  ea.r_s = r_s;
  ea.Ir = Ir;
  ea.Imax = Imax;
  ea.Nmax = Nmax;
  return launch_equatorial(ea, static_cast<cudaStream_t>(stream)) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_rho_of_req(const kgeo_curve* curves, int32_t ncurves, const double* varphi, int32_t nphi, double xtol,
                    double rtol, int32_t maxiter, double* rho, int32_t* status, void* stream) {
  if (ncurves < 0 || nphi < 0) return KGEO_ERR_LENGTHS;
  if (!(xtol > 0) || !(rtol >= 4 * 2.220446049250313e-16) || maxiter < 0) return KGEO_ERR_SOLVER;
  if (ncurves == 0 || nphi == 0) return KGEO_OK;
  if (!curves || !varphi || !rho) return KGEO_ERR_NULL;
  std::vector<CurveSpec> spec((size_t)ncurves);
  for (int32_t c = 0; c < ncurves; ++c) {
    const kgeo_curve& k = curves[c];
    kgeo_observer o{k.a, INFINITY, k.th_o};
    int st = check_observer(&o);
    if (st) return st;
    if (k.mbar < 0) return KGEO_ERR_MBAR;
    spec[c].obs = make_observer(&o);
    spec[c].r_target = k.r_eq;
    spec[c].rho_min = k.rho_min;
    spec[c].rho_max = k.rho_max;
    spec[c].mbar = k.mbar;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CurveSpec* table = nullptr;
  const size_t bytes = sizeof(CurveSpec) * spec.size();
  if (cudaMallocAsync(reinterpret_cast<void**>(&table), bytes, s) != cudaSuccess) return KGEO_ERR_CUDA;
  // a pageable source: the call returns once the table is staged, so `spec` may go
  bool ok = cudaMemcpyAsync(table, spec.data(), bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (ok) {
    CurveArgs ca;
    ca.curves = table;
    ca.ncurves = ncurves;
    ca.varphi = varphi;
    ca.nphi = nphi;
    ca.xtol = xtol;
    ca.rtol = rtol;
    ca.maxiter = maxiter;
    ca.rho = rho;
    ca.status = status;
    ok = launch_curves(ca, s) == cudaSuccess;
  }
  ok = (cudaFreeAsync(table, s) == cudaSuccess) && ok;
  return ok ? KGEO_OK : KGEO_ERR_CUDA;
}

namespace {
int make_jet_field(const kgeo_jet_field* j, double a, JetField* out) {
  if (!j) return KGEO_ERR_NULL;
  if (j->model < KGEO_JET_PARA || j->model > KGEO_JET_POWER) return KGEO_ERR_MODEL;
  if (!std::isfinite(j->psitarget) || !std::isfinite(j->pval)) return KGEO_ERR_MODEL;
  out->model = j->model;
  out->psitarget = j->psitarget;
  out->pval = j->pval;
  out->rp = 1 + std::sqrt(1 - a * a);
  return KGEO_OK;
}
}  // namespace

int kgeo_jet_guesses(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                     const double* r, const double* th, const double* mino, int32_t ngeo,
                     const kgeo_jet_field* field, int32_t neqmax, double* taumax, int32_t* count, double* guesses,
                     int32_t nguess, void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (ngeo < 0 || nguess < 0) return KGEO_ERR_NGEO;
  JetGuessArgs ga;
  st = make_jet_field(field, obs->a, &ga.field);
  if (st) return st;
  if (npix > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  if (npix > 0 && r && (!th || !mino)) return KGEO_ERR_NULL;
  ga.obs = make_observer(obs);
  ga.alpha = alpha;
  ga.beta = beta;
  ga.npix = npix;
  ga.r = r;
  ga.th = th;
  ga.mino = mino;
  ga.ngeo = ngeo;
  ga.neqmax = neqmax;
  ga.taumax = taumax;
  ga.count = count;
  ga.guesses = guesses;
  ga.nguess = nguess;
  return launch_jet_guesses(ga, static_cast<cudaStream_t>(stream)) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_jet_findroot(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                      const double* guesses, int32_t nguess, const kgeo_jet_field* field, double tol, int32_t maxiter,
                      void* workspace, size_t workspace_bytes_, double* tau, double* r, double* th, double* signpr,
                      double* signpth, double* neq, int32_t* status, void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (nguess < 0) return KGEO_ERR_NGEO;
  if (!(tol > 0) || maxiter < 1) return KGEO_ERR_SOLVER;
  JetSolveArgs ja;
  st = make_jet_field(field, obs->a, &ja.field);
  if (st) return st;
  if (npix > 0 && nguess > 0 && (!alpha || !beta || !guesses || !tau)) return KGEO_ERR_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch sc;
  st = get_scratch(sc, workspace, workspace_bytes_, npix, s);
  if (st) return st;
  Workspace w = carve_workspace(sc.ptr, npix);
  st = setup_common(obs, alpha, beta, npix, 0, 1.0 - 1.e-10, w, nullptr, s);
  if (st) return st;
  ja.obs = make_observer(obs);
  ja.rec = w.rec;
  ja.code = w.code;
  ja.flags = w.flags;
  ja.alpha = alpha;
  ja.beta = beta;
  ja.npix = npix;
  ja.guesses = guesses;
  ja.nguess = nguess;
  ja.tol = tol;
  ja.maxiter = maxiter;
  ja.tau = tau;
  ja.r = r;
  ja.th = th;
  ja.signpr = signpr;
  ja.signpth = signpth;
  ja.neq = neq;
  ja.status = status;
  return launch_jet_solve(ja, s) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_jet_stokes(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                    const double* r, const double* th, const double* signpr, const double* signpth,
                    const double* neq, int32_t nguess, const kgeo_jet_emission* em, double* I, double* Q,
                    double* U, double* evpa, double* I_c, double* Q_c, double* U_c, double* stagnation,
                    int32_t* status, void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (nguess < 0) return KGEO_ERR_NGEO;
  if (!em) return KGEO_ERR_NULL;
  if (!(em->model == KGEO_JET_MONO || (em->model == KGEO_JET_POWER && em->pval == 0.0))) return KGEO_ERR_MODEL;
  if (em->neqmax < 1 || !(em->nu_parallel >= -1.0 && em->nu_parallel <= 1.0) || !(em->sigma >= 0.0) ||
      !std::isfinite(em->specind))
    return KGEO_ERR_MODEL;
  if (!I || !Q || !U) return KGEO_ERR_NULL;
  if (npix > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  if (npix > 0 && nguess > 0 && (!r || !th || !signpr || !signpth || !neq)) return KGEO_ERR_NULL;
  JetStokesArgs ja;
  if (jet_bz_table(&ja.tab) != cudaSuccess) return KGEO_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* par = nullptr;
  if (cudaMallocAsync(&par, 4 * sizeof(double), s) != cudaSuccess) return KGEO_ERR_CUDA;
  ja.obs = make_observer(obs);
  ja.p.field = em->model == KGEO_JET_MONO ? JETF_MONO : JETF_POWER0;
  ja.p.nu = em->nu_parallel;
  ja.p.sigma = em->sigma;
  ja.p.r0 = 0.0;
  ja.p.specind = em->specind;
  ja.alpha = alpha;
  ja.beta = beta;
  ja.npix = npix;
  ja.r = r;
  ja.th = th;
  ja.signpr = signpr;
  ja.signpth = signpth;
  ja.neq = neq;
  ja.nguess = nguess;
  ja.neqmax = em->neqmax;
  ja.par = par;
  ja.I = I;
  ja.Q = Q;
  ja.U = U;
  ja.evpa = evpa;
  ja.Ic = I_c;
  ja.Qc = Q_c;
  ja.Uc = U_c;
  ja.stagnation = stagnation;
  ja.status = status;
  const cudaError_t e = launch_jet_stokes(ja, s);
  const cudaError_t f = cudaFreeAsync(par, s);
  return (e == cudaSuccess && f == cudaSuccess) ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_critical_curve(double a, double th_o, int64_t n, double* alpha, double* beta, void* stream) {
  kgeo_observer o{a, INFINITY, th_o};
  int st = check_observer(&o);
  if (st) return st;
  if (n < 0) return KGEO_ERR_LENGTHS;
  if (n == 0) return KGEO_OK;
  if (!alpha || !beta) return KGEO_ERR_NULL;
  CriticalArgs ca;
  ca.a = a;
  ca.sin_th = std::sin(th_o);
  ca.cos_th = std::cos(th_o);
  ca.tan_th = std::tan(th_o);
  ca.rminus = 2 * (1 + std::cos(2. * std::acos(-a) / 3.));
  ca.rplus = 2 * (1 + std::cos(2. * std::acos(a) / 3.));
  ca.n = n;
  ca.alpha = alpha;
  ca.beta = beta;
  return launch_critical(ca, static_cast<cudaStream_t>(stream)) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_image(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha, const double* beta,
               int64_t npix, const kgeo_emission* model, kgeo_image_out* out, void* stream) {
  return kgeo_image_ex(obs, mbar_lo, n_orders, alpha, beta, npix, model, nullptr, out, stream);
}

int kgeo_image_ex(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha,
                  const double* beta, int64_t npix, const kgeo_emission* model, const kgeo_image_options* options,
                  kgeo_image_out* out, void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (mbar_lo < 0 || n_orders < 1) return KGEO_ERR_MBAR;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  ImageArgs ia;
  st = make_model(model, &ia.model);
  if (st) return st;
  st = make_options(options, &ia.opts);
  if (st) return st;
  if (!out) return KGEO_ERR_NULL;
  if (npix > 0 && (!alpha || !beta || !out->I)) return KGEO_ERR_NULL;
  ia.obs = make_observer(obs);
  ia.alpha = alpha;
  ia.beta = beta;
  ia.npix = npix;
  ia.mbar_lo = mbar_lo;
  ia.nord = n_orders;
  ia.I = out->I;
  ia.g = out->g;
  ia.r_s = out->r_s;
  ia.Ir = out->Ir;
  ia.sinthb = out->sinthb;
  ia.imax = out->imax;
  ia.nmax = out->nmax;
  ia.npol = out->npol;
  const bool ex = options != nullptr;
  ia.Q = (ex && ia.opts.polarization) ? out->Q : nullptr;
  ia.U = (ex && ia.opts.polarization) ? out->U : nullptr;
  ia.lp = (ex && ia.opts.pathlength) ? out->lp : nullptr;
  ia.Ie = (ex && ia.opts.pathlength) ? out->Ie : nullptr;
  ia.perm = nullptr;
  if (npix == 0) return KGEO_OK;
  // pixels in radial-class order (stream-ordered scratch, freed after the launch)
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  if (cudaMallocAsync(&scratch, pixel_sort_bytes(npix), s) != cudaSuccess) return KGEO_ERR_CUDA;
  const bool ok = launch_pixel_sort(ia.obs, alpha, beta, npix, scratch, &ia.perm, s) == cudaSuccess &&
                  launch_image(ia, s) == cudaSuccess;
  const bool freed = cudaFreeAsync(scratch, s) == cudaSuccess;
  return ok && freed ? KGEO_OK : KGEO_ERR_CUDA;
}

// per-block partial sums, then the pixel-order scratch
size_t kgeo_image_adjoint_workspace_size(int64_t npix) {
  if (npix <= 0) return 0;
  return align_up((size_t)image_adjoint_blocks(npix) * NQ * sizeof(double), 256) + pixel_sort_bytes(npix);
}

int kgeo_image_adjoint(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha,
                       const double* beta, int64_t npix, const kgeo_emission* model, const double* grad_I,
                       double* grad, void* workspace, size_t workspace_bytes_, void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (mbar_lo < 0 || n_orders < 1) return KGEO_ERR_MBAR;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  ImageAdjointArgs aa;
  st = make_model(model, &aa.model);
  if (st) return st;
  if (!grad) return KGEO_ERR_NULL;
  if (npix > 0 && (!alpha || !beta || !grad_I || !workspace)) return KGEO_ERR_NULL;
  if (workspace_bytes_ < kgeo_image_adjoint_workspace_size(npix)) return KGEO_ERR_WORKSPACE;
  aa.obs = make_observer(obs);
  aa.alpha = alpha;
  aa.beta = beta;
  aa.npix = npix;
  aa.mbar_lo = mbar_lo;
  aa.nord = n_orders;
  aa.grad_I = grad_I;
  aa.partial = static_cast<double*>(workspace);
  aa.grad = grad;
  aa.perm = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (npix > 0) {
    char* sort_scratch = static_cast<char*>(workspace) + align_up((size_t)image_adjoint_blocks(npix) * NQ * sizeof(double), 256);
    if (launch_pixel_sort(aa.obs, alpha, beta, npix, sort_scratch, &aa.perm, s) != cudaSuccess) return KGEO_ERR_CUDA;
  }
  return launch_image_adjoint(aa, s) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_equatorial_crossings(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                              const double* tau, int32_t ntau, double* n_eq, double* n_pol,
                              double* outside_crit, void* stream) {
  if (!obs) return KGEO_ERR_NULL;
  if (!(std::fabs(obs->a) >= 0 && std::fabs(obs->a) < 1)) return KGEO_ERR_SPIN;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (ntau < 0) return KGEO_ERR_NGEO;
  if (npix > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  if (npix > 0 && ntau > 0 && (n_eq || n_pol) && !tau) return KGEO_ERR_NULL;
  CrossingArgs ca;
  ca.obs = make_observer(obs);
  ca.alpha = alpha;
  ca.beta = beta;
  ca.npix = npix;
  ca.tau = tau;
  ca.ntau = ntau;
  ca.n_eq = n_eq;
  ca.n_pol = n_pol;
  ca.outside = outside_crit;
  ca.n_turn = nullptr;
  return launch_crossings(ca, static_cast<cudaStream_t>(stream)) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_angular_turnings(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                          const double* tau, int32_t ntau, double* n_turn, void* stream) {
  if (!obs) return KGEO_ERR_NULL;
  if (!(std::fabs(obs->a) >= 0 && std::fabs(obs->a) < 1)) return KGEO_ERR_SPIN;
  if (!(obs->th_o >= 0 && obs->th_o <= 0.5 * PI)) return KGEO_ERR_TH_O;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (ntau < 0) return KGEO_ERR_NGEO;
  if (npix > 0 && ntau > 0 && (!alpha || !beta || !tau || !n_turn)) return KGEO_ERR_NULL;
  CrossingArgs ca;
  ca.obs = make_observer(obs);
  ca.alpha = alpha;
  ca.beta = beta;
  ca.npix = npix;
  ca.tau = tau;
  ca.ntau = ntau;
  ca.n_eq = nullptr;
  ca.n_pol = nullptr;
  ca.outside = nullptr;
  ca.n_turn = n_turn;
  return launch_crossings(ca, static_cast<cudaStream_t>(stream)) == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_ray_setup(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix, int32_t ngeo,
                   double maxtaufrac, void* workspace, size_t workspace_bytes_, kgeo_geodesics* per_ray,
                   void* stream) {
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (ngeo < 0) return KGEO_ERR_NGEO;
  if (!workspace) return KGEO_ERR_NULL;
  if (workspace_bytes_ < workspace_bytes(npix)) return KGEO_ERR_WORKSPACE;
  if (npix > 0 && (!alpha || !beta)) return KGEO_ERR_NULL;
  Workspace w = carve_workspace(workspace, npix);
  return setup_common(obs, alpha, beta, npix, ngeo, maxtaufrac, w, per_ray, static_cast<cudaStream_t>(stream));
}

int kgeo_ray_samples(const kgeo_observer* obs, const void* workspace, size_t workspace_bytes_, int64_t npix,
                     const double* tau, int32_t nsamp, int32_t do_phi_and_t, int32_t chunk, int32_t precision,
                     kgeo_geodesics* out, void* stream) {
  if (precision != KGEO_PRECISION_FP64 && precision != KGEO_PRECISION_MIXED) return KGEO_ERR_MODEL;
  int st = check_observer(obs);
  if (st) return st;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  if (nsamp < 0) return KGEO_ERR_NGEO;
  if (!workspace || !out) return KGEO_ERR_NULL;
  if (workspace_bytes_ < workspace_bytes(npix)) return KGEO_ERR_WORKSPACE;
  Workspace w = carve_workspace(const_cast<void*>(workspace), npix);
  return samples_common(obs, w, npix, nsamp, tau, do_phi_and_t ? 1 : 0, chunk, precision == KGEO_PRECISION_MIXED,
                        out, static_cast<cudaStream_t>(stream));
}

const char* kgeo_status_string(int status) {
  switch (status) {
    case KGEO_OK: return "ok";
    case KGEO_ERR_SPIN: return "|a| should be a float in range [0,1)";
    case KGEO_ERR_R_O: return "r_o should be a float > 100";
    case KGEO_ERR_TH_O: return "th_o should be a float in range (0,pi/2) or (pi/2,pi)";
    case KGEO_ERR_LENGTHS: return "alpha, beta are different lengths!";
    case KGEO_ERR_NGEO: return "ngeo must be >= 0";
    case KGEO_ERR_MBAR: return "mbar should be an integer >=0!";
    case KGEO_ERR_WORKSPACE: return "workspace too small";
    case KGEO_ERR_NULL: return "a required pointer is NULL";
    case KGEO_ERR_CUDA: return "CUDA runtime error";
    case KGEO_ERR_MODEL: return "emissivity / velocity / B-field model or image option out of range";
    case KGEO_ERR_NOALLOC_SIZE: return "npix exceeds KGEO_NOALLOC_MAX_PIXELS (kgeo_raytrace_noalloc)";
    case KGEO_ERR_SOLVER: return "root solver arguments out of range (xtol > 0, rtol >= 4 eps, maxiter >= 0)";
    default: return "unknown status";
  }
}

int kgeo_ellip_pi(const double* n, const double* phi, const double* m, int64_t N, int32_t form, double* out,
                  void* stream) {
  if (N < 0) return KGEO_ERR_LENGTHS;
  if (form < 0 || form > 2) return KGEO_ERR_MODEL;
  if (N > 0 && (!n || !phi || !m || !out)) return KGEO_ERR_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = form == 0 ? launch_ellip_pi_setup(n, phi, m, N, out, s)
                            : launch_ellip_pi_samples(n, phi, m, N, form, out, s);
  return e == cudaSuccess ? KGEO_OK : KGEO_ERR_CUDA;
}

int kgeo_abi_version(void) { return KGEO_ABI_VERSION; }

}  // extern "C"
