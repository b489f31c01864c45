// C ABI: context, error reporting, BTE plan lifecycle and queries.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <mutex>
#include <string>

#include "internal.h"

namespace obte {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};
static std::atomic<int64_t> g_h2d{0};   // bytes the table uploads copied host -> device

void set_error(const std::string& msg) { g_last_error = msg; }

obte_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
  return e == cudaErrorMemoryAllocation ? OBTE_ERR_OOM : OBTE_ERR_CUDA;
}

void count_launch(int n) { g_launches += n; }

cudaError_t wait_stream(cudaStream_t stream) {
  const char* env = std::getenv("OBTE_BLOCKING_SYNC");   // read per call: a caller may switch modes between phases
  const bool blocking = env && std::atoi(env) != 0;
  if (!blocking) return cudaStreamSynchronize(stream);
  // one blocking-sync event per thread and device, created on first use
  thread_local std::vector<std::pair<int, cudaEvent_t>> events;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaEvent_t ev = nullptr;
  for (auto& de : events)
    if (de.first == dev) ev = de.second;
  if (!ev) {
    e = cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    events.emplace_back(dev, ev);
  }
  e = cudaEventRecord(ev, stream);
  if (e != cudaSuccess) return e;
  return cudaEventSynchronize(ev);
}

// ---- recycled device blocks ---------------------------------------------------------------
namespace {
struct CachedBlock {
  void* p;
  size_t bytes;
  int dev;
};
std::mutex g_cache_mu;
std::vector<CachedBlock> g_cache;     // idle blocks, oldest first
size_t g_cached = 0;
thread_local int g_recycle = 0;

// Most bytes the cache keeps (OBTE_DEVICE_CACHE_MB, default 16 GiB); older blocks beyond it are freed.
size_t cache_cap() {
  static const size_t cap = [] {
    const char* e = std::getenv("OBTE_DEVICE_CACHE_MB");
    return e ? (size_t)std::max(0L, std::atol(e)) << 20 : (size_t)16 << 30;
  }();
  return cap;
}

// Allocation sizes: powers of two up to 1 MiB, multiples of 2 MiB above, so blocks of similar plans fit.
size_t size_class(size_t n) {
  if (n <= ((size_t)1 << 20)) {
    size_t c = 512;
    while (c < n) c <<= 1;
    return c;
  }
  const size_t g = (size_t)2 << 20;
  return (n + g - 1) / g * g;
}

// Free every cached block of `dev` (all devices: -1); returns the bytes freed.
size_t cache_trim(int dev) {
  std::vector<CachedBlock> drop;
  {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    std::vector<CachedBlock> keep;
    for (const auto& b : g_cache) (dev < 0 || b.dev == dev ? drop : keep).push_back(b);
    g_cache.swap(keep);
    for (const auto& b : drop) g_cached -= b.bytes;
  }
  size_t freed = 0;
  int cur = 0;
  cudaGetDevice(&cur);
  for (const auto& b : drop) {
    if (b.dev != cur) cudaSetDevice(b.dev);
    cudaFree(b.p);
    if (b.dev != cur) cudaSetDevice(cur);
    freed += b.bytes;
  }
  return freed;
}
}  // namespace

RecycleScope::RecycleScope() { ++g_recycle; }
RecycleScope::~RecycleScope() { --g_recycle; }

void device_release(void* p, size_t bytes, int dev) {
  if (!g_recycle) {
    cudaFree(p);
    return;
  }
  std::vector<CachedBlock> drop;
  {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    g_cache.push_back({p, bytes, dev});
    g_cached += bytes;
    while (g_cached > cache_cap() && !g_cache.empty()) {   // the oldest blocks go first
      drop.push_back(g_cache.front());
      g_cached -= g_cache.front().bytes;
      g_cache.erase(g_cache.begin());
    }
  }
  for (const auto& b : drop) cudaFree(b.p);   // blocks of this device: the caller's device is current
}

obte_status DevBuf::alloc(size_t n) {
  release();
  if (n == 0) n = 16;
  const size_t want = size_class(n);
  int d = 0;
  OBTE_CUDA(cudaGetDevice(&d));
  {
    // best fit among the cached blocks of this device, at most 1/8 (or one 2 MiB step) larger
    std::lock_guard<std::mutex> lock(g_cache_mu);
    const size_t slack = std::max(want / 8, want > ((size_t)1 << 20) ? ((size_t)2 << 20) : (size_t)0);
    int best = -1;
    for (int i = 0; i < (int)g_cache.size(); ++i) {
      const CachedBlock& b = g_cache[i];
      if (b.dev == d && b.bytes >= want && b.bytes <= want + slack && (best < 0 || b.bytes < g_cache[best].bytes))
        best = i;
    }
    if (best >= 0) {
      p = g_cache[best].p;
      bytes = g_cache[best].bytes;
      dev = d;
      g_cached -= bytes;
      g_cache.erase(g_cache.begin() + best);
      return OBTE_OK;
    }
  }
  cudaError_t e = cudaMalloc(&p, want);
  if (e == cudaErrorMemoryAllocation && cache_trim(d) > 0) {
    (void)cudaGetLastError();
    e = cudaMalloc(&p, want);
  }
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
  }
  bytes = want;
  dev = d;
  return OBTE_OK;
}

namespace {
std::vector<std::pair<void*, size_t>> g_host_cache;   // idle pinned blocks (guarded by g_cache_mu)
constexpr size_t kHostCacheBlocks = 256;
}  // namespace

void host_release(void* p, size_t bytes) {
  if (g_recycle) {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    if (g_host_cache.size() < kHostCacheBlocks) {
      g_host_cache.emplace_back(p, bytes);
      return;
    }
  }
  cudaFreeHost(p);
}

obte_status HostBuf::alloc(size_t n) {
  release();
  if (n == 0) n = 16;
  {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    for (size_t i = 0; i < g_host_cache.size(); ++i)
      if (g_host_cache[i].second >= n && g_host_cache[i].second <= 4 * n + 4096) {
        p = g_host_cache[i].first;
        bytes = g_host_cache[i].second;
        g_host_cache.erase(g_host_cache.begin() + i);
        return OBTE_OK;
      }
  }
  cudaError_t e = cudaMallocHost(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_fail(e, "cudaMallocHost", __FILE__, __LINE__);
  }
  bytes = n;
  return OBTE_OK;
}

// A buffer that already holds an allocation of the needed size class is refilled in place: a re-upload
// (new transmissions of a design loop, every step) then costs no cudaFree / cudaMalloc, which synchronise
// the whole device.
template <typename T>
obte_status upload(DevBuf& b, const std::vector<T>& v, cudaStream_t stream) {
  const size_t need = std::max<size_t>(v.size(), 1) * sizeof(T);
  if (!(b.p && b.bytes == size_class(need))) OBTE_TRY(b.alloc(need));
  if (!v.empty()) {
    OBTE_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
    OBTE_CUDA(wait_stream(stream));
    g_h2d += (int64_t)(v.size() * sizeof(T));
  }
  return OBTE_OK;
}
obte_status upload_bytes(DevBuf& b, const void* p, size_t bytes, cudaStream_t stream) {
  const size_t need = std::max<size_t>(bytes, 1);
  if (!(b.p && b.bytes == size_class(need))) OBTE_TRY(b.alloc(need));
  if (bytes) {
    OBTE_CUDA(cudaMemcpyAsync(b.p, p, bytes, cudaMemcpyHostToDevice, stream));
    OBTE_CUDA(wait_stream(stream));
    g_h2d += (int64_t)bytes;
  }
  return OBTE_OK;
}
template obte_status upload<int32_t>(DevBuf&, const std::vector<int32_t>&, cudaStream_t);
template obte_status upload<int64_t>(DevBuf&, const std::vector<int64_t>&, cudaStream_t);
template obte_status upload<double>(DevBuf&, const std::vector<double>&, cudaStream_t);
template obte_status upload<float>(DevBuf&, const std::vector<float>&, cudaStream_t);
template obte_status upload<int8_t>(DevBuf&, const std::vector<int8_t>&, cudaStream_t);

}  // namespace obte

using namespace obte;

extern "C" const char* obte_status_string(int status) {
  switch (status) {
    case OBTE_OK: return "OK";
    case OBTE_ERR_BAD_ARG: return "BAD_ARG";
    case OBTE_ERR_OOM: return "OOM";
    case OBTE_ERR_ADMISSION: return "ADMISSION_REJECTED";
    case OBTE_ERR_NOT_CONVERGED: return "NOT_CONVERGED";
    case OBTE_ERR_CUDA: return "CUDA_ERROR";
    case OBTE_ERR_CYCLE: return "CYCLE";
    case OBTE_ERR_UNSUPPORTED: return "UNSUPPORTED";
    case OBTE_ERR_DEVICE_TIMEOUT: return "DEVICE_TIMEOUT";
    default: return "UNKNOWN";
  }
}

extern "C" const char* obte_last_error(void) { return g_last_error.c_str(); }

extern "C" int64_t obte_launch_count(void) { return g_launches.load(); }

extern "C" int64_t obte_h2d_bytes(void) { return g_h2d.load(); }

extern "C" obte_status obte_context_create(int device, void* stream, obte_context* out) {
  if (!out) { set_error("null out"); return OBTE_ERR_BAD_ARG; }
  int count = 0;
  OBTE_CUDA(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) { set_error("bad device index"); return OBTE_ERR_BAD_ARG; }
  OBTE_CUDA(cudaSetDevice(device));
  auto* c = new obte_context_s();
  c->device = device;
  c->stream = static_cast<cudaStream_t>(stream);
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaGetDeviceProperties", __FILE__, __LINE__); }
  c->num_sms = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  *out = c;
  return OBTE_OK;
}

extern "C" obte_status obte_context_destroy(obte_context ctx) {
  delete ctx;
  return OBTE_OK;
}

extern "C" obte_status obte_context_set_stream(obte_context ctx, void* stream) {
  if (!ctx) { set_error("null context"); return OBTE_ERR_BAD_ARG; }
  ctx->stream = static_cast<cudaStream_t>(stream);
  return OBTE_OK;
}

// Conserved-offset weights over the full state (zero on the periodic part); returns their sum.
static double offset_weights(const obte_plan p, std::vector<double>& ell) {
  const Schedule& s = p->sched;
  ell.assign(p->nu, 0.0);
  double sum = 0;
  for (int64_t e = 0; e < s.n; ++e) { ell[e] = s.ell_T[e]; sum += s.ell_T[e]; }
  for (int64_t w = 0; w < s.nd; ++w) { ell[s.n + w] = s.ell_B[w]; sum += s.ell_B[w]; }
  return sum;
}

extern "C" obte_status obte_bte_plan_create(obte_context ctx, const obte_problem* prob, const obte_material* mat,
                                            obte_plan* out) {
  if (!out) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (ctx) OBTE_CUDA(cudaSetDevice(ctx->device));
  auto* p = new obte_plan_s();
  p->ctx = ctx;
  obte_status st = build_schedule(prob, mat, p->sched);
  if (st != OBTE_OK) { delete p; return st; }
  const Schedule& s = p->sched;
  p->nx = s.x_base[s.n_dir] * s.n_mfp;
  p->nu = s.n + s.nd + p->nx;
  std::vector<double> ell;
  p->ell_sum = offset_weights(p, ell);
  if (!ctx) { *out = p; return OBTE_OK; }   // host-only plan: schedule queries, no device tables
  auto fail = [&](obte_status code) { delete p; return code; };
  cudaStream_t strm = ctx->stream;
  p->stream = strm;
  if ((st = upload(p->ell, ell, strm)) != OBTE_OK) return fail(st);
  if ((st = upload(p->x_cell, s.x_cell, strm)) != OBTE_OK) return fail(st);
  if ((st = upload(p->diffuse_cell, s.diffuse_cell, strm)) != OBTE_OK) return fail(st);
  if ((st = upload(p->kconst, s.kconst, strm)) != OBTE_OK) return fail(st);
  if ((st = upload(p->kshift, s.kshift, strm)) != OBTE_OK) return fail(st);
  if ((st = upload(p->sshift, s.sshift, strm)) != OBTE_OK) return fail(st);
  if ((st = upload(p->x_base_dev, s.x_base, strm)) != OBTE_OK) return fail(st);
  *out = p;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_plan_set_transmission(obte_plan plan, const double* side_transmission,
                                                      int64_t* upload_bytes) {
  if (!plan || !side_transmission) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (upload_bytes) *upload_bytes = 0;
  // nothing issued earlier may still read the coefficients being replaced
  if (plan->ctx) OBTE_CUDA(cudaStreamSynchronize(plan->stream));
  OBTE_TRY(set_transmission(plan->sched, side_transmission));
  const Schedule& s = plan->sched;
  std::vector<double> ell;
  plan->ell_sum = offset_weights(plan, ell);
  // the preconditioner belongs to the old transmissions; the last solution stays as a warm start
  plan->xprec.reset();
  dsa_join(plan);
  plan->dsa.reset();                       // its interface conductances change with t
  plan->n_solves = 0;
  if (!plan->ctx) return OBTE_OK;
  // the acceleration's operator for the new t is built on a host thread while the tables are refreshed
  dsa_start_async(plan);
  cudaStream_t strm = plan->stream;
  OBTE_TRY(upload(plan->ell, ell, strm));
  OBTE_TRY(upload(plan->kconst, s.kconst, strm));
  OBTE_TRY(upload(plan->kshift, s.kshift, strm));
  int64_t bytes = (int64_t)(ell.size() + s.kconst.size() + s.kshift.size()) * 8;
  OBTE_TRY(refresh_tables(plan, side_transmission, &bytes));
  if (upload_bytes) *upload_bytes = bytes;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_plan_destroy(obte_plan plan) {
  if (!plan) return OBTE_OK;
  dsa_join(plan);
  // every use of the plan's device buffers was on its stream: once it is idle they can be recycled
  const bool idle = plan->ctx && wait_stream(plan->stream) == cudaSuccess;
  if (idle) {
    RecycleScope recycle;
    delete plan;
  } else {
    delete plan;
  }
  return OBTE_OK;
}

extern "C" obte_status obte_device_cache_trim(int64_t* freed_bytes) {
  const size_t f = cache_trim(-1);
  if (freed_bytes) *freed_bytes = (int64_t)f;
  return OBTE_OK;
}

extern "C" obte_status obte_device_cache_bytes(int64_t* cached_bytes) {
  if (!cached_bytes) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  std::lock_guard<std::mutex> lock(g_cache_mu);
  *cached_bytes = (int64_t)g_cached;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_plan_set_stream(obte_plan plan, void* stream) {
  if (!plan || !plan->ctx) { set_error("null or host-only plan"); return OBTE_ERR_BAD_ARG; }
  // finish work issued on the previous stream before switching
  OBTE_CUDA(wait_stream(plan->stream));
  plan->stream = static_cast<cudaStream_t>(stream);
  return OBTE_OK;
}

extern "C" obte_status obte_bte_plan_footprint(obte_plan plan, int32_t precision, int32_t restart,
                                               int64_t* plan_bytes, int64_t* solve_bytes) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  const Schedule& s = plan->sched;
  // table bytes per precision, computed from the host schedule (tables may not be uploaded yet)
  auto tab = [&](size_t rb) {
    size_t b = 0;
    b += (s.cell.size() + s.slot.size() + s.xk.size() + s.wout.size() + s.contact.size() + s.in_idx.size() +
          s.lev_ptr.size() + s.wo_wall.size()) * 4;
    b += (s.in_coef.size() + s.D.size() + s.P.size() + s.mfp.size() + s.tco.size() + s.sig.size() +
          s.wo_wall.size() * 4 + s.kcoef.size() + s.scoef.size() + s.hs.size()) * rb;
    b += (s.lev_ptr.size() + s.in_idx.size()) * 8; // unit tables and periodic prefetch lists (bound)
    return (int64_t)b;
  };
  // tables that are uploaded count with their actual size, the others with an upper estimate
  // FP64 tables before upload: plus the reciprocal table (n_dir x n x the MFPs rounded up to a chunk), unless
  // it is switched off or over its cap
  int64_t rinv_est = (int64_t)s.n_dir * s.n * ((s.n_mfp + 3) & ~3) * 8;
  {
    const char* off = std::getenv("OBTE_SWEEP64_RINV");
    const char* cap = std::getenv("OBTE_SWEEP64_RINV_GB");
    if ((off && std::atoi(off) == 0) || (double)rinv_est > (cap ? std::atof(cap) : 32.0) * 1e9) rinv_est = 0;
  }
  const int64_t t64 = plan->d64.ready ? (int64_t)plan->d64.bytes() : tab(8) + rinv_est;
  const int64_t t32 = plan->d32.ready ? (int64_t)plan->d32.bytes() : tab(4);
  int64_t pb = (int64_t)plan->nu * 8 + (int64_t)s.x_cell.size() * 4 + (int64_t)s.kconst.size() * 24;
  if (precision == OBTE_FP64) pb += t64;
  else if (precision == OBTE_FP32) pb += t32;
  else pb += t64 + t32;
  pb += xprec_resident_bytes(plan->xprec.get());
  if (plan->dsa) {
    pb += plan->dsa->bytes;
  } else if (dsa_default(s)) {
    // the diffusion operator a solve will build: CSR of L, five element vectors and a hierarchy of at
    // most about three times L's size
    const int64_t nnz = s.n + 2 * (int64_t)s.dsa.e1.size();
    pb += 4 * (nnz * 12 + (s.n + 1) * 4) + s.n * 8 * 5;
  }
  if (plan_bytes) *plan_bytes = pb;
  if (solve_bytes) *solve_bytes = plan->ctx ? solve_scratch_bytes(plan, restart > 0 ? restart : 30) : 0;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_state_layout(obte_plan plan, int64_t* n_elems, int64_t* n_diffuse, int64_t* n_x) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  if (n_elems) *n_elems = plan->sched.n;
  if (n_diffuse) *n_diffuse = plan->sched.nd;
  if (n_x) *n_x = plan->nx;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_precond_info(obte_plan plan, int32_t* n_blocks, int32_t* setup_sweeps,
                                             double* setup_ms) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  const XPrec* P = plan->xprec.get();
  if (n_blocks) *n_blocks = P ? P->nblk : 0;
  if (setup_sweeps) *setup_sweeps = P ? P->detect_sweeps + P->probe_sweeps : 0;
  if (setup_ms) *setup_ms = P ? P->setup_ms : 0.0;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_precond_bytes(obte_plan plan, int64_t* resident, int64_t* build_bound) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  if (resident) *resident = xprec_resident_bytes(plan->xprec.get());
  if (build_bound) *build_bound = plan->ctx ? xprec_build_bound(plan) : 0;
  return OBTE_OK;
}

extern "C" obte_status obte_bte_schedule(obte_plan plan, int32_t q, int64_t* order, int64_t* level_ptr,
                                         int64_t* n_levels, int64_t* n_slots) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  const Schedule& s = plan->sched;
  if (q < 0 || q >= s.n_dir) { set_error("direction out of range"); return OBTE_ERR_BAD_ARG; }
  const int nl = s.nlev[q];
  if (n_levels) *n_levels = nl;
  if (n_slots) *n_slots = s.nslots[q];
  if (order)
    for (int64_t p = 0; p < s.n; ++p) order[p] = s.cell[(size_t)q * s.n + p];
  if (level_ptr)
    for (int L = 0; L <= nl; ++L) level_ptr[L] = s.lev_ptr[s.lev_off[q] + L];
  return OBTE_OK;
}

extern "C" obte_status obte_bte_tables_digest(obte_plan plan, int32_t precision, uint64_t* digest) {
  if (!plan || !digest) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  return tables_digest(plan, precision != OBTE_FP64, digest);
}

extern "C" obte_status obte_bte_schedule_coefficients(obte_plan plan, int32_t q, double* in_coef, double* D,
                                                      double* P) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  const Schedule& s = plan->sched;
  if (q < 0 || q >= s.n_dir) { set_error("direction out of range"); return OBTE_ERR_BAD_ARG; }
  const size_t base = (size_t)q * s.n;
  if (in_coef) std::copy(s.in_coef.begin() + base * s.nf, s.in_coef.begin() + (base + s.n) * s.nf, in_coef);
  if (D) std::copy(s.D.begin() + base, s.D.begin() + base + s.n, D);
  if (P) std::copy(s.P.begin() + base, s.P.begin() + base + s.n, P);
  return OBTE_OK;
}

namespace obte {
obte_status ensure_fields_scratch(obte_plan plan) {
  if (plan->fields_J.p) return OBTE_OK;
  const Schedule& s = plan->sched;
  OBTE_TRY(plan->fields_J.alloc((size_t)s.n * s.ds * sizeof(double)));
  OBTE_TRY(plan->fields_K.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
  OBTE_TRY(plan->fields_S.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
  return OBTE_OK;
}
}  // namespace obte

extern "C" obte_status obte_bte_sweep_fields(obte_plan plan, int32_t precision, const double* u_in, double* u_out,
                                             int32_t with_source, void* T) {
  if (!plan || !u_in || !u_out || !T) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (!plan->ctx) { set_error("host-only plan cannot sweep"); return OBTE_ERR_BAD_ARG; }
  if (precision != OBTE_FP64 && precision != OBTE_FP32 && precision != OBTE_FP32_REFINE &&
      precision != OBTE_DOUBLE_FLOAT) {
    set_error("bad precision"); return OBTE_ERR_BAD_ARG;
  }
  if (plan->xstore) { set_error("a gradient solve is using the per-ordinate store"); return OBTE_ERR_BAD_ARG; }
  const bool fp32 = precision == OBTE_FP32 || precision == OBTE_FP32_REFINE;
  // the final-pass kernel also accumulates J, K and S; they go to plan-owned buffers and are discarded
  OBTE_TRY(ensure_fields_scratch(plan));
  if (fp32) plan->xstore = static_cast<float*>(T);
  else plan->xstore64 = static_cast<double*>(T);
  const obte_status st =
      precision == OBTE_DOUBLE_FLOAT
          ? launch_sweep_df(plan, u_in, u_out, with_source != 0, plan->fields_J.as<double>(), plan->fields_K.as<double>(),
                            plan->fields_S.as<double>())
          : launch_sweep(plan, fp32, u_in, u_out, with_source != 0, true, plan->fields_J.as<double>(),
                         plan->fields_K.as<double>(), plan->fields_S.as<double>());
  plan->xstore = nullptr;
  plan->xstore64 = nullptr;
  OBTE_TRY(st);
  OBTE_CUDA(cudaStreamSynchronize(plan->stream));
  return check_device_error(plan);
}

extern "C" obte_status obte_bte_plan_test_wait_timeout(obte_plan plan, int32_t skip_unit, int32_t wait_limit) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  if (skip_unit < -1 || wait_limit < 0) { set_error("skip_unit must be >= -1 and wait_limit >= 0"); return OBTE_ERR_BAD_ARG; }
  plan->test_skip_unit = skip_unit;
  plan->test_wait_limit = wait_limit;
  return OBTE_OK;
}
