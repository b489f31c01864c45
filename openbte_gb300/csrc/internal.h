// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <atomic>
#include <memory>
#include <thread>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/obte.h"

namespace obte {

// ---- error handling ----------------------------------------------------------
void set_error(const std::string& msg);
obte_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define OBTE_CUDA(call)                                                         \
  do {                                                                          \
    cudaError_t _e = (call);                                                    \
    if (_e != cudaSuccess) return ::obte::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define OBTE_TRY(call)                                                          \
  do {                                                                          \
    obte_status _s = (call);                                                    \
    if (_s != OBTE_OK) return _s;                                               \
  } while (0)

// Count of kernel launches issued by this library (instrumentation for the bench).
void count_launch(int n = 1);

// Wait until `stream` has finished its work.  By default this is cudaStreamSynchronize, which spins on a
// core while it waits; with OBTE_BLOCKING_SYNC=1 the calling thread sleeps on a blocking-sync event
// instead (a serving loop with many GPU slots would otherwise keep one host core spinning per slot, taken
// from the threads that build and upload the next requests' plans).
cudaError_t wait_stream(cudaStream_t stream);

// Host worker count: OBTE_HOST_THREADS, else the hardware concurrency (at most 32).
inline int host_threads() {
  int t = (int)std::thread::hardware_concurrency();
  if (const char* env = std::getenv("OBTE_HOST_THREADS")) t = std::atoi(env);
  return std::max(1, std::min(t, 32));
}

// f(i) for i in [0, n) over host threads in contiguous blocks (results must not depend on the split).
template <typename F>
void parallel_for(int64_t n, F&& f) {
  const int nt = (int)std::min<int64_t>(host_threads(), std::max<int64_t>(1, n / 64));
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      for (int64_t i = n * t / nt; i < n * (t + 1) / nt; ++i) f(i);
    });
  for (auto& th : pool) th.join();
}

// f(i) for i in [0, n) where each i is a large task (a direction): one task at a time per host thread,
// handed out in index order from a shared counter (results must not depend on the assignment).
template <typename F>
void parallel_tasks(int64_t n, F&& f) {
  const int nt = (int)std::min<int64_t>(host_threads(), n);
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (int64_t i = next++; i < n; i = next++) f(i);
    });
  for (auto& th : pool) th.join();
}

// Wall time of a host phase, printed to stderr at scope exit when OBTE_TRACE is set.
struct PhaseTimer {
  const char* name;
  std::chrono::steady_clock::time_point t0;
  bool on;
  explicit PhaseTimer(const char* n)
      : name(n), t0(std::chrono::steady_clock::now()), on(std::getenv("OBTE_TRACE") != nullptr) {}
  ~PhaseTimer() {
    if (on)
      std::fprintf(stderr, "[obte trace] %s %.1f ms\n", name,
                   std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  }
};

// ---- device buffer ------------------------------------------------------------
// Device memory is taken from a library-wide cache of recycled blocks when one fits, else from cudaMalloc.
// Blocks return to the cache only where the caller guarantees that no work still uses them (a plan being
// destroyed after its stream was synchronised: RecycleScope); elsewhere release() calls cudaFree.  cudaFree
// synchronises the whole device, which stalled every concurrent solve of a serving loop each time a
// finished request's plan was dropped.
void device_release(void* p, size_t bytes, int dev);
struct RecycleScope {      // while alive on this thread, released device buffers go to the cache
  RecycleScope();
  ~RecycleScope();
};
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int dev = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) device_release(p, bytes, dev);
    p = nullptr;
    bytes = 0;
  }
  obte_status alloc(size_t n);
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// Page-locked host buffer (the solver's small per-iteration device -> host reads).  Recycled like DevBuf
// (cudaFreeHost synchronises the device as cudaFree does).
void host_release(void* p, size_t bytes);
struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  ~HostBuf() { release(); }
  void release() {
    if (p) host_release(p, bytes);
    p = nullptr;
    bytes = 0;
  }
  obte_status alloc(size_t n);
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// Upload a host vector into a fresh device buffer (synchronous on `stream`).
template <typename T>
obte_status upload(DevBuf& b, const std::vector<T>& v, cudaStream_t stream);
obte_status upload_bytes(DevBuf& b, const void* p, size_t bytes, cudaStream_t stream);

// ---- smoothed-aggregation AMG (preconditioner of the Fourier CG, amg.cu) ---------------------------
struct AmgHierarchy;
struct AmgDeleter {
  void operator()(AmgHierarchy* h) const;
};
using AmgPtr = std::unique_ptr<AmgHierarchy, AmgDeleter>;
// Hierarchy of the SPD CSR matrix (rp, ci, val); row `pin` (>= 0) is replaced by the identity.  Coarsening
// stops at `coarse_max` rows or fewer, whose operator is inverted densely (host Gauss-Jordan, O(rows^3)).
obte_status amg_build(int64_t n, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                      const std::vector<double>& val, int pin, int num_sms, cudaStream_t st, AmgPtr& out,
                      int coarse_max = 400);
// Enqueue z = M^-1 r (one symmetric V-cycle) on `st`; with `part`, also the nb_part block partials of
// r . z (launched on exactly nb_part blocks).  Returns the number of kernel launches.
int amg_apply(const AmgHierarchy& H, const double* r, double* z, double* part, int nb_part, cudaStream_t st);
int amg_levels(const AmgHierarchy& H);
int amg_launches(const AmgHierarchy& H, bool with_part);   // kernel launches of one amg_apply

}  // namespace obte

struct obte_context_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  size_t smem_optin = 0;
};

namespace obte {

// Inflow item kinds packed in the top 2 bits of an int32 (index in the low 30 bits).
enum : int32_t { ITEM_NONE = 0, ITEM_CELL = 1, ITEM_PERIODIC = 2, ITEM_WALL = 3 };
constexpr int ITEM_SHIFT = 30;
constexpr int32_t ITEM_MASK = (1 << ITEM_SHIFT) - 1;
inline int32_t pack_item(int kind, int32_t idx) { return (int32_t)((uint32_t)kind << ITEM_SHIFT) | idx; }

// Host-side sweep schedule: one direction per block of n_elems items (level order).
// Allocator whose resize() leaves trivially constructible elements uninitialised: the per-direction
// schedule arrays (hundreds of MB on large meshes) are first written by the parallel direction workers,
// so their pages are touched in parallel instead of by one serial zero fill.
template <typename T>
struct DefaultInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind { using other = DefaultInitAlloc<U>; };
  DefaultInitAlloc() noexcept = default;
  template <typename U>
  DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept {}
  template <typename U>
  void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new (static_cast<void*>(p)) U;
  }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};
template <typename T>
using RawVec = std::vector<T, DefaultInitAlloc<T>>;
template <typename T>
obte_status upload(DevBuf& b, const RawVec<T>& v, cudaStream_t stream) {
  return upload_bytes(b, v.data(), v.size() * sizeof(T), stream);
}

struct Schedule {
  int dim = 2;
  int nf = 3;                      // inflow slots per element (= sides per element)
  int64_t n = 0;                   // elements
  int n_dir = 0, n_mfp = 0, m_pad = 0, n_chunks = 0, ds = 2;
  int64_t nd = 0;                  // diffuse wall sides (T_B entries)
  // per direction, per position (n_dir * n); written by build_schedule's direction workers
  RawVec<int32_t> cell, slot, xk, wout, contact;
  RawVec<int32_t> in_idx;          // n_dir * n * nf
  RawVec<double> in_coef;          // n_dir * n * nf
  RawVec<double> D, P;             // n_dir * n
  // levels
  std::vector<int32_t> lev_ptr;    // concatenated level pointers
  std::vector<int64_t> lev_off;    // [n_dir] start of direction q in lev_ptr
  std::vector<int32_t> nlev;       // [n_dir]
  std::vector<int32_t> nslots;     // [n_dir]
  int max_slots = 0;
  int max_src = 0;                 // largest number of periodic source elements of one direction
  // periodic interface
  std::vector<int64_t> x_base;     // [n_dir+1] source-cell offsets
  std::vector<int32_t> x_cell;     // [x_base[n_dir]] element of each source slot
  // wall outputs: entries (q, wall) with their re-emission weights
  std::vector<int32_t> wo_wall;    // [n_wo]
  std::vector<double> w_db;        // [nd * dim] wall area vector / volume of its element
  std::vector<double> gbm_sum;     // [nd] sum over ordinates of min(sigma . w_db, 0)
  std::vector<int32_t> wo_off;     // [n_dir+1] first wall-output entry of each direction
  int max_wo = 0;                  // most wall-output entries of one direction
  // contact
  std::vector<double> kcoef;       // [n_ce * m_pad]
  std::vector<double> scoef;       // [n_ce]
  std::vector<double> kconst;      // [n_mfp * n_dir]  alpha-term of K
  std::vector<double> kshift;      // [n_mfp * n_dir]  dK/d(offset)
  std::vector<double> sshift;      // [n_mfp * n_dir]  dS/d(offset)
  // per-ordinate tables (padded)
  std::vector<double> mfp;         // [m_pad]
  std::vector<double> tco;         // [n_dir * m_pad]
  std::vector<double> sig;         // [n_dir * m_pad * ds]
  std::vector<double> sig_sum;     // [ds] sum over all ordinates of sigma
  std::vector<double> hs;          // [n] heat_source * coeff (empty if none)
  // offset weights (energy-conservation left null vector)
  std::vector<double> ell_T, ell_B;
  std::vector<int32_t> diffuse_cell;  // [nd] element of each wall side
  // transmission-interface data for dkappa/dt (present when side transmissions were given)
  bool tim = false;
  int64_t n_sides = 0;
  std::vector<double> dirs;                  // [n_dir * dim] unit directions
  std::vector<int32_t> tim_side;             // [ni] side id of internal side k
  std::vector<int32_t> tim_e1, tim_e2;       // [ni] its elements (area vector points from e1)
  std::vector<int32_t> tim_w1, tim_w2;       // [ni] reflecting wall of the e1 / e2 directed face (-1: none)
  std::vector<double> tim_na;                // [ni * dim] area vector
  std::vector<double> tim_jump;              // [ni] periodic jump (0 off periodic sides)
  std::vector<char> tim_contact;             // [ni] 1 = contact side
  double contact_alpha = 0, normalization = 0;
  bool extra_sources = false;                // isothermal walls, heat source or nanowire terms
  bool isothermal = false;                   // isothermal (mixed) walls: they fix the temperature level, so
                                             // I - K has no constant null mode and no offset is applied
  // Diffusion-synthetic acceleration data (dsa.cu): the cell-temperature diffusion operator that the
  // transport operator I - K approaches on smooth temperature errors.
  struct DsaData {
    std::vector<double> vol;                 // [n] element volumes
    std::vector<int32_t> e1, e2;             // [nfc] the two elements of each internal side (periodic too)
    std::vector<int32_t> side;               // [nfc] its side id
    std::vector<double> area, dist;          // [nfc] side area, centre-to-centre distance estimate
    std::vector<double> t;                   // [nfc] side transmission (1: plain side)
    std::vector<int32_t> iso_cell;           // [niso] isothermal walls: element
    std::vector<double> iso_area, iso_dist;  // [niso] area, centre-to-wall distance estimate
    std::vector<double> Dm, Gm;              // [n_mfp] per MFP: sum_q t_coeff (mfp v_q)(mfp v_q)^T / dim
                                             // (isotropic part) and the half-range flux moment
  } dsa;
  // Transmission plans without isothermal walls or nanowire terms keep the transmission-free factor of
  // every coefficient that depends on the side transmissions t: the sweep order, the levels, the slots and
  // the packed table layout depend on the mesh and the directions only, so new transmissions replace
  // coefficients and nothing else (set_transmission).
  struct TransmissionFactors {
    bool ok = false;
    int contact_kind = 0;
    std::vector<double> g0;                  // [n_dir * n * nf] inflow coefficient without t
    std::vector<int32_t> mode;               // same layout: side s (x t_s), -(s + 2) (x (1 - t_s)), -1 (x 1)
    std::vector<int32_t> per_i, per_j, per_side;   // [np] periodic sides: their two elements and side id
    std::vector<double> per_a;               // [n_dir * np * 2] jump terms of P without t
    std::vector<int32_t> c_side;             // [nc] contact sides
    std::vector<double> c_na;                // [nc * dim] their area vectors
    std::vector<int32_t> co_ptr, co_k, co_role;   // element -> (contact side, role 1 = e1 / 2 = e2)
    std::vector<double> ell0;                // [nd] ell_B without the wall's scale
    std::vector<int32_t> w_side;             // [nd] side of a reflecting wall (-1: diffuse wall, scale 1)
  } tf;
};

obte_status build_schedule(const obte_problem* prob, const obte_material* mat, Schedule& s);
// New side transmissions [n_sides] for a plan built with side transmissions (coefficients only).
obte_status set_transmission(Schedule& s, const double* side_transmission);

// Device copy of the schedule in precision Real.
//   rec      packed per-item records (level order, all directions)
//   klev_*   kernel level pointers: levels split into units of at most `cap` items
//   vals     per-sweep (DeltaT + h, perturbation - wall inflow) pairs, level order
//   si/sr    side table of special elements (periodic inflow, wall/periodic/contact outputs)
struct DevSchedule {
  bool ready = false;
  int G = 1, KV = 4, mc = 0, mcp = 0, n_chunks = 0, zero_slot = 0, rows = 0;   // G lanes x KV MFPs per element, mcp per CTA
  int emax = 0, unit_wo = 0, pf_pad = 0, unit_sx = 0;   // periodic bank rows, per-unit staging sizes
  int nbuf = 2;                            // TMA pipeline depth
  size_t smem = 0;
  DevBuf rec, klev_ptr, klev_off, knlev, kwo, kpf, pf, sx, ksx, mfp, tco, sig, wo_wall, wo_geo, kcoef, scoef, hs, vals, cellmap,
      Pq, si, sr, wo_off, spec;
  DevBuf lpt;                              // launch order: CTAs of the directions with the most units first
  // FP64 tables: 1 / (1 + mfp_m D) per (direction, chunk, position, MFP of the chunk), so that the FP64
  // sweep multiplies instead of dividing on GB300's narrow FP64 pipe (null when over its memory cap)
  DevBuf rinv;
  // deterministic reductions (OBTE_DETERMINISTIC=1): per-(direction, chunk) partials and per-position sums
  DevBuf det_d, det_j, det_w, det_k, det_s, det_S, det_SJ;
  // transmission plans: the special-entry index of each item (host), so that new transmissions rewrite
  // the wall coefficients; the records' coefficient words are rewritten on the device (refresh_tables)
  RawVec<int32_t> h_spec;
  bool refreshable = false;
  int64_t n_spec = 0;
  size_t bytes() const;
};

}  // namespace obte

namespace obte {
// Solver scratch, kept with the plan and reused across solves with the same restart length.
struct SolveWork {
  int64_t nu = 0;
  int restart = 0;
  int nb = 1;
  DevBuf u, Fu, r, V, w, tmp, partial, hdev, sdev, Jraw, Kraw, Sraw, delta;
  DevBuf pz;         // preconditioned vector (allocated when the plan has a preconditioner)
  DevBuf rc, Jraw2, Kraw2, Sraw2;   // refinement: correction right-hand side, outputs of the correction
  DevBuf V32, w32;   // FP32 basis and working vector (stages with FP32 sweeps), allocated on first use
  DevBuf gs;         // device Arnoldi step: second-pass coefficients, Hessenberg column, flags
  HostBuf hcol;      // pinned copy of the Hessenberg column
};

// Diffusion-synthetic acceleration (dsa.cu): right preconditioner term E L^-1 R, with R the volume-
// weighted temperature part of a state vector, L the cell diffusion operator of Schedule::DsaData solved
// by `cycles` stationary smoothed-aggregation V-cycle iterations (a fixed linear map, as GMRES needs), and
// E the extension of a cell correction to the temperatures, the wall temperatures of each wall's element
// and the periodic inflow of each source slot's element.
struct DsaOp {
  AmgPtr amg;
  DevBuf rp, ci, val;            // L (CSR, symmetric, volume-weighted)
  DevBuf vol;                    // [n]
  DevBuf b, d, r, e, mean;       // right-hand side, correction, residual, cycle update; partial sums of the
                                 // weighted means (one per block)
  double inv_vol_sum = 0;
  bool project = true;           // L has the constant null vector (no isothermal walls)
  int cycles = 1;
  int levels = 0;
  double setup_ms = 0;
  int64_t bytes = 0;             // device bytes held
};

// Right preconditioner of the GMRES on the periodic-inflow unknowns: for the ordinates whose inflow
// circulates through the periodic cell for many periods, the exact inverse of their one-period
// inflow -> outflow transfer, (I - T_b)^-1 - I, as a dense FP32 block over the direction's source slots.
struct XPrec {
  bool tried = false;            // setup ran (blocks may still be empty)
  int nblk = 0, smax = 0;
  int probe_sweeps = 0, detect_sweeps = 0;
  double setup_ms = 0;
  DevBuf bm, bs, boff, bwoff;    // per block: MFP, size (slots), first entry in bslot, offset of its W block
  DevBuf bslot;                  // source slots of every block, concatenated
  DevBuf W;                      // FP32 row-major blocks
};

// Transmission-interface gradient: per internal side tables, ordinate tables and the final-pass
// per-ordinate temperatures (built on the first gradient call of a plan).
struct TimDevice {
  bool ready = false;
  bool paired = false;  // adjoint fields from a separate plan with the reversed directions
  double kfac = 0;      // adjoint scale nrm * a / jump (sigma = a tau L s)
  DevBuf side, e1, e2, w1, w2, na, jump, contact, dirs, tl, sig, refl, xs, K;
};
}  // namespace obte

struct obte_plan_s {
  obte_context ctx = nullptr;
  cudaStream_t stream = nullptr;    // stream of every call on this plan (set at creation, changeable)
  std::unique_ptr<obte::SolveWork> work;
  obte::Schedule sched;
  obte::DevSchedule d64, d32;       // FP64 and FP32 tables (built lazily)
  obte::DevBuf x_cell, diffuse_cell, kconst, kshift, sshift;
  obte::DevBuf ell;                 // [nu] conserved-offset weights (zero on the periodic part)
  double ell_sum = 0;               // ell . 1
  obte::DevBuf x_base_dev;
  obte::DevBuf err;                 // device error word (bounded waits that gave up)
  int64_t nx = 0;                   // periodic-inflow unknowns (source cells x n_mfp)
  int64_t nu = 0;                   // state length
  bool has_solution = false;        // work->u holds the last converged state
  // deterministic reductions: position of element c in direction q's order [n_dir][n], wall -> wall-output
  // entries (CSR, in entry order), first contact entry of each direction [n_dir + 1]
  obte::DevBuf det_inv, det_wptr, det_went, det_ceoff;
  int64_t det_nce = -1;             // contact entries (-1: tables not built)
  float* xstore = nullptr;          // set during a gradient solve: final-pass per-ordinate temperatures
  bool xstore_add = false;          // the final pass adds its temperatures to xstore (pass at a correction)
  double* xstore64 = nullptr;       // set during obte_bte_sweep_fields in FP64: the same in FP64
  obte::DevBuf fields_J, fields_K, fields_S;   // final-pass outputs of obte_bte_sweep_fields (discarded)
  // bounded-wait test (obte_bte_plan_test_wait_timeout): level unit whose bulk copy the sweeps skip
  // (-1: none) and the poll cap of their copy waits (0: the default)
  int test_skip_unit = -1;
  int test_wait_limit = 0;
  std::unique_ptr<obte::TimDevice> tim;   // transmission-interface gradient tables and scratch
  // non-final sweeps run only these CTAs (direction * n_chunks + chunk) while set (preconditioner setup)
  const int32_t* sweep_cta_map = nullptr;
  int sweep_n_cta = 0;
  int sweep_batch = 1;                    // with the map: that many state vectors, sweep_batch_stride apart
  int64_t sweep_batch_stride = 0;
  std::unique_ptr<obte::XPrec> xprec;     // periodic-inflow block preconditioner
  std::unique_ptr<obte::DsaOp> dsa;       // diffusion-synthetic acceleration (built on first use)
  // set-up of `dsa` for new transmissions, on a host thread beside the refresh of the tables (joined by
  // the next solve or by destroy; a failure is retried there)
  std::thread dsa_build;
  obte_status dsa_build_status = OBTE_OK;
  // transmission plans: per (item, inflow slot) the coefficient without t, its t factor (mode) and the
  // record coefficient word it fills (-1: none), and the current side transmissions, on the device
  obte::DevBuf tf_g0, tf_mode, tf_word, tf_t;
  int n_solves = 0;                       // obte_bte_solve calls on this plan
};

namespace obte {
// One sweep (sweep.cu). final: also accumulate J (into Jraw), K and S.
obte_status launch_sweep(obte_plan plan, bool fp32, const double* u_in, double* u_out, bool with_src,
                         bool final_pass, double* Jraw, double* K, double* S);
obte_status ensure_tables(obte_plan plan, bool fp32);
// The output pass (J, K, S accumulated) in double-float arithmetic on the FP64 tables (sweep.cu).
obte_status launch_sweep_df(obte_plan plan, const double* u_in, double* u_out, bool with_src, double* Jraw,
                            double* K, double* S);
// After set_transmission: the coefficient words of the device tables that exist (bytes uploaded added to *bytes).
obte_status refresh_tables(obte_plan plan, const double* side_transmission, int64_t* bytes);
// Digest of the packed sweep tables of one precision, built on the host.
obte_status tables_digest(obte_plan plan, bool fp32, uint64_t* digest);
// Periodic-inflow preconditioner (xprec.cu): built once per plan.
obte_status ensure_xprec(obte_plan plan, SolveWork& wk);
// out[X blocks] += W in[X blocks] (fp32: FP32 accumulation, for stages with an FP32 Krylov basis)
void xprec_add(obte_plan plan, const double* in, double* out, bool fp32);
int64_t xprec_resident_bytes(const XPrec* P);
// Diffusion-synthetic acceleration (dsa.cu).
obte_status ensure_dsa(obte_plan plan);
void dsa_add(obte_plan plan, const double* in, double* out);    // out += E L^-1 R in
bool dsa_default(const Schedule& s);                            // on by default for this problem?
void dsa_start_async(obte_plan plan);                           // build `dsa` on a host thread
obte_status dsa_join(obte_plan plan);                           // wait for it (OBTE_OK if none ran)
void dsa_matrix(const Schedule& s, std::vector<int32_t>& rp, std::vector<int32_t>& ci, std::vector<double>& val,
                bool& project);                                 // the diffusion operator (host)
int64_t xprec_build_bound(obte_plan plan);   // device bytes a build would allocate (0 once tried)
obte_status check_device_error(obte_plan plan);
// Plan-owned J, K, S buffers for sweeps whose final-pass accumulations are discarded (api.cu).
obte_status ensure_fields_scratch(obte_plan plan);
int64_t solve_scratch_bytes(obte_plan plan, int restart);
}  // namespace obte
