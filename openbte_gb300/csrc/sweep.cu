// Batched upwind transport sweep for sm_103a.
//
// One CTA = one direction q x one chunk of 32 mean free paths (lane = MFP).
// The CTA walks the direction's elements level by level (longest-path layers
// of the upwind DAG, periodic inflow cut); inside a level every warp takes a
// contiguous run of elements, all 32 lanes solving an element for their own MFP:
//
//   T_mq[c] = (DeltaT[c] + h[c] + L_m P_q[c] - L_m sum_in g_f T_up) / (1 + L_m D_q[c])
//
// which is the row of A_mq T = B of openbte/bte.py:183-218 for an element whose
// upwind neighbours are already known.  T_up comes from
//   - the shared-memory slot of an upstream element (ITEM_CELL),
//   - the periodic-inflow part of the state vector (ITEM_PERIODIC),
//   - the wall temperature T_B (ITEM_WALL, openbte/bte.py:200,214).
//
// Data movement per level:
//   - the level's packed item records (geometry, coefficients, slots) arrive in
//     shared memory by a TMA bulk copy (cp.async.bulk + mbarrier) issued one
//     level ahead, so the record stream overlaps the previous level's compute;
//   - DeltaT[c] for a warp's items is gathered by its lanes in one instruction
//     and handed out by shuffles;
//   - T stays in a shared-memory ring of slots (recycled after the last
//     consumer's level); it never goes to HBM.
// Reductions of openbte/bte.py:222-243 are fused:
//   DeltaT'[c] += sum_m t_mq T        (warp shuffle, then one FP64 atomic)
//   T_B'[w]    += sum_m (-GG) T       (walls)
//   x'         = T at periodic source elements (interface unknowns)
//   final pass: J += sum_m sigma_mq T, K_mq / S_mq in registers per lane.
// Every mbarrier wait is bounded; on timeout the CTA raises the device error
// word, stops using the records, waits (bounded) for its own copy in flight
// and leaves at the next block-wide barrier.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "internal.h"

namespace obte {

// ---- packed item records ---------------------------------------------------------
// FP32: 16 words (64 B); FP64: 24 words (96 B). Both multiples of 16 B (TMA).
//   w0 cell  w1 slot  w2 xk  w3 wout  w4 contact  w5..w8 in_idx[4]
//   FP32: w9..w12 in_coef[4]  w13 D  w14 P  w15 pad
//   FP64: w9 pad, w10..w17 in_coef[4], w18..w19 D, w20..w21 P, w22..w23 pad
template <typename Real> struct RecLayout;
template <> struct RecLayout<float> { static constexpr int W = 16; };
template <> struct RecLayout<double> { static constexpr int W = 24; };

template <typename Real>
static void pack_records(const Schedule& s, std::vector<int32_t>& out) {
  constexpr int W = RecLayout<Real>::W;
  const size_t total = (size_t)s.n_dir * s.n;
  out.assign(total * W, 0);
  for (size_t it = 0; it < total; ++it) {
    int32_t* r = out.data() + it * W;
    r[0] = s.cell[it]; r[1] = s.slot[it]; r[2] = s.xk[it]; r[3] = s.wout[it]; r[4] = s.contact[it];
    for (int f = 0; f < 4; ++f) r[5 + f] = f < s.nf ? s.in_idx[it * s.nf + f] : 0;
    if (sizeof(Real) == 4) {
      for (int f = 0; f < 4; ++f) {
        float v = f < s.nf ? (float)s.in_coef[it * s.nf + f] : 0.f;
        std::memcpy(&r[9 + f], &v, 4);
      }
      float d = (float)s.D[it], p = (float)s.P[it];
      std::memcpy(&r[13], &d, 4);
      std::memcpy(&r[14], &p, 4);
    } else {
      for (int f = 0; f < 4; ++f) {
        double v = f < s.nf ? s.in_coef[it * s.nf + f] : 0.0;
        std::memcpy(&r[10 + 2 * f], &v, 8);
      }
      std::memcpy(&r[18], &s.D[it], 8);
      std::memcpy(&r[20], &s.P[it], 8);
    }
  }
}

// ---- PTX helpers (TMA bulk copy + mbarrier) -----------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false if the phase did not complete within the iteration cap.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  for (int i = 0; i < (1 << 22); ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <typename Real>
struct SweepParams {
  int64_t n;
  int64_t nd;
  int n_mfp, m_pad, n_chunks, n_dir, ds, cap;
  const int32_t* __restrict__ rec;       // packed records
  const int32_t* __restrict__ lev_ptr;   // kernel level units
  const int64_t* __restrict__ lev_off;
  const int32_t* __restrict__ nlev;
  const int64_t* __restrict__ x_base;
  const int32_t* __restrict__ wo_wall;
  const Real* __restrict__ mfp;
  const Real* __restrict__ tco;
  const Real* __restrict__ sig;
  const Real* __restrict__ wo_gg;
  const Real* __restrict__ kcoef;
  const Real* __restrict__ scoef;
  const Real* __restrict__ hs;
  const double* __restrict__ u_in;
  double* __restrict__ u_out;
  double* __restrict__ Jraw;
  double* __restrict__ K;
  double* __restrict__ S;
  int* __restrict__ err;
  int with_src;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename Real>
__device__ __forceinline__ Real rec_real(const int32_t* r, int word);
template <>
__device__ __forceinline__ float rec_real<float>(const int32_t* r, int word) {
  return __int_as_float(r[word]);
}
template <>
__device__ __forceinline__ double rec_real<double>(const int32_t* r, int word) {
  return __hiloint2double(r[word + 1], r[word]);
}

template <typename Real, int NF, bool FINAL>
__global__ void __launch_bounds__(256) bte_sweep_kernel(const SweepParams<Real> p) {
  constexpr int W = RecLayout<Real>::W;
  constexpr bool F32 = sizeof(Real) == 4;
  constexpr int OFF_COEF = F32 ? 9 : 10;
  constexpr int STEP = F32 ? 1 : 2;
  constexpr int OFF_D = F32 ? 13 : 18;
  constexpr int OFF_P = F32 ? 14 : 20;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);            // 2 mbarriers
  int* s_abort = reinterpret_cast<int*>(smem_raw + 16);             // [2], by level parity
  int32_t* recbuf0 = reinterpret_cast<int32_t*>(smem_raw + 128);
  int32_t* recbuf1 = recbuf0 + (size_t)p.cap * W;
  Real* buf = reinterpret_cast<Real*>(recbuf1 + (size_t)p.cap * W);  // T ring [slots][32]

  const int q = blockIdx.x / p.n_chunks;
  const int chunk = blockIdx.x - q * p.n_chunks;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int m = chunk * 32 + lane;
  const bool active = m < p.n_mfp;

  const Real lam = p.mfp[m];
  const Real tq = p.tco[(int64_t)q * p.m_pad + m];
  Real sg0 = 0, sg1 = 0, sg2 = 0;
  if (FINAL) {
    const Real* sp = p.sig + ((int64_t)q * p.m_pad + m) * p.ds;
    sg0 = sp[0];
    if (p.ds > 1) sg1 = sp[1];
    if (p.ds > 2) sg2 = sp[2];
  }
  const double* __restrict__ dT = p.u_in;
  const double* __restrict__ TB = p.u_in + p.n;
  const double* __restrict__ X = p.u_in + p.n + p.nd;
  double* __restrict__ dT_out = p.u_out;
  double* __restrict__ TB_out = p.u_out + p.n;
  double* __restrict__ X_out = p.u_out + p.n + p.nd;
  const int64_t xq = p.x_base[q];
  const int32_t* __restrict__ lev = p.lev_ptr + p.lev_off[q];
  const int nlev = p.nlev[q];
  const int32_t* __restrict__ rec_q = p.rec + (int64_t)q * p.n * W;
  const bool src = p.with_src != 0;

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    s_abort[0] = 0;
    s_abort[1] = 0;
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned bytes = (unsigned)(lev[1] - lev[0]) * W * 4u;
    mbar_expect_tx(&bars[0], bytes);
    tma_load_1d(recbuf0, rec_q + (int64_t)lev[0] * W, bytes, &bars[0]);
  }

  Real kacc = 0, sacc = 0;
  bool issued_next = false;
  for (int L = 0; L < nlev; ++L) {
    const int b = lev[L];
    const int e = lev[L + 1];
    const int cur = L & 1;
    issued_next = false;
    if (threadIdx.x == 0 && L + 1 < nlev) {
      // buffer cur^1 was last read during level L-1, finished at the barrier below
      fence_proxy_async();
      const unsigned bytes = (unsigned)(lev[L + 2] - lev[L + 1]) * W * 4u;
      mbar_expect_tx(&bars[cur ^ 1], bytes);
      tma_load_1d(cur ? recbuf0 : recbuf1, rec_q + (int64_t)lev[L + 1] * W, bytes, &bars[cur ^ 1]);
      issued_next = true;
    }
    const bool ready = mbar_wait_bounded(&bars[cur], (unsigned)(L >> 1) & 1u);
    if (!ready) {
      s_abort[cur] = 1;
      if (lane == 0) atomicOr(p.err, 1);
    } else {
      const int32_t* recs = cur ? recbuf1 : recbuf0;
      const int width = e - b;
      const int ipw = (width + nw - 1) / nw;
      const int i0 = warp * ipw;
      const int cnt = max(0, min(ipw, width - i0));
      // gather DeltaT (+ heat source) of this warp's items, one lane per item
      Real my_dT = 0;
      if (lane < cnt) {
        const int c = recs[(i0 + lane) * W];
        my_dT = (Real)dT[c];
        if (src && p.hs) my_dT += p.hs[c];
      }
      for (int k = 0; k < cnt; ++k) {
        const int32_t* r = recs + (i0 + k) * W;
        const int c = r[0];
        const int sl = r[1];
        const int xk = r[2];
        const int wo = r[3];
        const int ce = r[4];
        Real acc = __shfl_sync(0xffffffffu, my_dT, k);
        if (src) acc += lam * rec_real<Real>(r, OFF_P);
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const int32_t code = r[5 + f];
          const int kind = (int)((uint32_t)code >> ITEM_SHIFT);
          if (kind == ITEM_NONE) continue;
          const int idx = code & ITEM_MASK;
          Real v;
          if (kind == ITEM_CELL) {
            v = buf[idx * 32 + lane];
          } else if (kind == ITEM_PERIODIC) {
            v = active ? (Real)X[(xq + idx) * p.n_mfp + m] : Real(0);
          } else {
            v = (Real)TB[idx];
          }
          acc -= lam * rec_real<Real>(r, OFF_COEF + STEP * f) * v;
        }
        const Real T = acc / (Real(1) + lam * rec_real<Real>(r, OFF_D));
        if (sl >= 0) buf[sl * 32 + lane] = T;

        const Real rs = warp_sum(tq * T);
        if (lane == 0) atomicAdd(&dT_out[c], (double)rs);
        if (xk >= 0 && active) X_out[(xq + xk) * p.n_mfp + m] = (double)T;
        if (wo) {
          const int wb = wo >> 3, wn = wo & 7;
          for (int j = 0; j < wn; ++j) {
            const Real rw = warp_sum(p.wo_gg[(int64_t)(wb + j) * p.m_pad + m] * T);
            if (lane == 0) atomicAdd(&TB_out[p.wo_wall[wb + j]], (double)rw);
          }
        }
        if (FINAL) {
          const Real r0 = warp_sum(sg0 * T);
          if (lane == 0) atomicAdd(&p.Jraw[(int64_t)c * p.ds], (double)r0);
          if (p.ds > 1) {
            const Real r1 = warp_sum(sg1 * T);
            if (lane == 0) atomicAdd(&p.Jraw[(int64_t)c * p.ds + 1], (double)r1);
          }
          if (p.ds > 2) {
            const Real r2 = warp_sum(sg2 * T);
            if (lane == 0) atomicAdd(&p.Jraw[(int64_t)c * p.ds + 2], (double)r2);
          }
          if (ce >= 0) {
            kacc += p.kcoef[(int64_t)ce * p.m_pad + m] * T;
            sacc += p.scoef[ce] * T;
          }
        }
      }
    }
    __syncthreads();
    // a flag raised during level L lives in word L&1; level L+1 writes the other word,
    // so a warp still reading this one cannot see a later level's timeout
    if (s_abort[cur]) {
      // leave together; first let the copy this CTA still has in flight land (bounded)
      if (threadIdx.x == 0 && issued_next) mbar_wait_bounded(&bars[cur ^ 1], (unsigned)((L + 1) >> 1) & 1u);
      __syncthreads();
      return;
    }
  }
  if (FINAL) {
    // reduce the per-warp K/S partials (the T ring is free after the last barrier)
    Real* red = buf;
    red[warp * 32 + lane] = kacc;
    red[(nw + warp) * 32 + lane] = sacc;
    __syncthreads();
    if (warp == 0) {
      Real ks = 0, ss = 0;
      for (int w = 0; w < nw; ++w) {
        ks += red[w * 32 + lane];
        ss += red[(nw + w) * 32 + lane];
      }
      if (active) {
        p.K[(int64_t)m * p.n_dir + q] = (double)ks;
        p.S[(int64_t)m * p.n_dir + q] = (double)ss;
      }
    }
  }
}

// ---- table upload ---------------------------------------------------------------

size_t DevSchedule::bytes() const {
  const DevBuf* all[] = {&rec, &klev_ptr, &klev_off, &knlev, &mfp, &tco, &sig, &wo_wall, &wo_gg, &kcoef, &scoef, &hs};
  size_t b = 0;
  for (auto* x : all) b += x->bytes;
  return b;
}

template <typename Real>
static obte_status upload_real(DevBuf& b, const std::vector<double>& v, cudaStream_t st) {
  std::vector<Real> h(v.begin(), v.end());
  if (h.empty()) h.push_back(Real(0));
  return upload(b, h, st);
}

static constexpr int kThreads = 256;

// Shared memory of one CTA for a given level cap.
template <typename Real>
static size_t sweep_smem(const Schedule& s, int cap) {
  const int nw = kThreads / 32;
  return 128 + 2 * (size_t)cap * RecLayout<Real>::W * 4 + (size_t)std::max(s.max_slots, 2 * nw) * 32 * sizeof(Real);
}

template <typename Real>
static obte_status upload_tables(obte_plan plan, DevSchedule& d) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->ctx->stream;
  // level cap: largest of {128, 96, 64, 48, 32} that lets two CTAs share an SM, else the smallest that fits one
  const size_t per_sm = 228 * 1024, reserve = 1024;
  int cap = 0;
  for (int c : {128, 96, 64, 48, 32})
    if (sweep_smem<Real>(s, c) + reserve <= per_sm / 2) { cap = c; break; }
  if (!cap)
    for (int c : {128, 96, 64, 48, 32})
      if (sweep_smem<Real>(s, c) <= plan->ctx->smem_optin) { cap = c; break; }
  if (!cap) {
    set_error("sweep front needs more shared memory than one CTA can have (" + std::to_string(s.max_slots) +
              " slots)");
    return OBTE_ERR_UNSUPPORTED;
  }
  d.cap = cap;
  // split levels into units of at most `cap` items (slots were assigned per level, so this stays valid)
  std::vector<int32_t> kptr;
  std::vector<int64_t> koff(s.n_dir);
  std::vector<int32_t> kn(s.n_dir);
  for (int q = 0; q < s.n_dir; ++q) {
    koff[q] = (int64_t)kptr.size();
    const int32_t* lp = s.lev_ptr.data() + s.lev_off[q];
    int units = 0;
    kptr.push_back(0);
    for (int L = 0; L < s.nlev[q]; ++L) {
      for (int32_t a = lp[L]; a < lp[L + 1]; a += cap) {
        kptr.push_back(std::min(a + cap, lp[L + 1]));
        ++units;
      }
    }
    kn[q] = units;
  }
  std::vector<int32_t> rec;
  pack_records<Real>(s, rec);
  OBTE_TRY(upload(d.rec, rec, st));
  OBTE_TRY(upload(d.klev_ptr, kptr, st));
  OBTE_TRY(upload(d.klev_off, koff, st));
  OBTE_TRY(upload(d.knlev, kn, st));
  std::vector<int32_t> wo = s.wo_wall;
  if (wo.empty()) wo.push_back(0);
  OBTE_TRY(upload(d.wo_wall, wo, st));
  OBTE_TRY(upload_real<Real>(d.mfp, s.mfp, st));
  OBTE_TRY(upload_real<Real>(d.tco, s.tco, st));
  OBTE_TRY(upload_real<Real>(d.sig, s.sig, st));
  OBTE_TRY(upload_real<Real>(d.wo_gg, s.wo_gg, st));
  OBTE_TRY(upload_real<Real>(d.kcoef, s.kcoef, st));
  OBTE_TRY(upload_real<Real>(d.scoef, s.scoef, st));
  if (!s.hs.empty()) OBTE_TRY(upload_real<Real>(d.hs, s.hs, st));
  d.ready = true;
  return OBTE_OK;
}

obte_status ensure_tables(obte_plan plan, bool fp32) {
  if (!plan->err.p) {
    OBTE_TRY(plan->err.alloc(sizeof(int)));
    OBTE_CUDA(cudaMemsetAsync(plan->err.p, 0, sizeof(int), plan->ctx->stream));
  }
  if (fp32) {
    if (!plan->d32.ready) return upload_tables<float>(plan, plan->d32);
  } else {
    if (!plan->d64.ready) return upload_tables<double>(plan, plan->d64);
  }
  return OBTE_OK;
}

// ---- launch -----------------------------------------------------------------------

template <typename Real, int NF, bool FINAL>
static obte_status launch_impl(obte_plan plan, const DevSchedule& d, const double* u_in, double* u_out,
                               bool with_src, double* Jraw, double* K, double* S) {
  const Schedule& s = plan->sched;
  const size_t smem = sweep_smem<Real>(s, d.cap);
  auto kern = bte_sweep_kernel<Real, NF, FINAL>;
  OBTE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SweepParams<Real> p;
  p.n = s.n; p.nd = s.nd; p.n_mfp = s.n_mfp; p.m_pad = s.m_pad; p.n_chunks = s.n_chunks; p.n_dir = s.n_dir;
  p.ds = s.ds; p.cap = d.cap;
  p.rec = d.rec.as<int32_t>();
  p.lev_ptr = d.klev_ptr.as<int32_t>();
  p.lev_off = d.klev_off.as<int64_t>();
  p.nlev = d.knlev.as<int32_t>();
  p.x_base = plan->x_base_dev.as<int64_t>();
  p.wo_wall = d.wo_wall.as<int32_t>();
  p.mfp = d.mfp.as<Real>(); p.tco = d.tco.as<Real>(); p.sig = d.sig.as<Real>(); p.wo_gg = d.wo_gg.as<Real>();
  p.kcoef = d.kcoef.as<Real>(); p.scoef = d.scoef.as<Real>();
  p.hs = s.hs.empty() ? nullptr : d.hs.as<Real>();
  p.u_in = u_in; p.u_out = u_out; p.Jraw = Jraw; p.K = K; p.S = S; p.with_src = with_src ? 1 : 0;
  p.err = plan->err.as<int>();
  const int grid = s.n_dir * s.n_chunks;
  kern<<<grid, kThreads, smem, plan->ctx->stream>>>(p);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  return OBTE_OK;
}

obte_status launch_sweep(obte_plan plan, bool fp32, const double* u_in, double* u_out, bool with_src,
                         bool final_pass, double* Jraw, double* K, double* S) {
  OBTE_TRY(ensure_tables(plan, fp32));
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->ctx->stream;
  if (s.ds > 3) { set_error("sigma with more than 3 components"); return OBTE_ERR_UNSUPPORTED; }
  if (s.nf > 4) { set_error("elements with more than 4 sides are not supported"); return OBTE_ERR_UNSUPPORTED; }
  OBTE_CUDA(cudaMemsetAsync(u_out, 0, (size_t)(s.n + s.nd) * sizeof(double), st));
  if (final_pass) OBTE_CUDA(cudaMemsetAsync(Jraw, 0, (size_t)s.n * s.ds * sizeof(double), st));
#define OBTE_DISPATCH(R, DS)                                                                        \
  do {                                                                                              \
    if (s.nf == 3) {                                                                                \
      if (final_pass) return launch_impl<R, 3, true>(plan, DS, u_in, u_out, with_src, Jraw, K, S);  \
      return launch_impl<R, 3, false>(plan, DS, u_in, u_out, with_src, Jraw, K, S);                 \
    } else {                                                                                        \
      if (final_pass) return launch_impl<R, 4, true>(plan, DS, u_in, u_out, with_src, Jraw, K, S);  \
      return launch_impl<R, 4, false>(plan, DS, u_in, u_out, with_src, Jraw, K, S);                 \
    }                                                                                               \
  } while (0)
  if (fp32) OBTE_DISPATCH(float, plan->d32);
  else OBTE_DISPATCH(double, plan->d64);
#undef OBTE_DISPATCH
}

// Device error word: nonzero after a bounded wait gave up (cleared on read).
obte_status check_device_error(obte_plan plan) {
  if (!plan->err.p) return OBTE_OK;
  int h = 0;
  OBTE_CUDA(cudaMemcpyAsync(&h, plan->err.p, sizeof(int), cudaMemcpyDeviceToHost, plan->ctx->stream));
  OBTE_CUDA(cudaStreamSynchronize(plan->ctx->stream));
  if (h) {
    OBTE_CUDA(cudaMemsetAsync(plan->err.p, 0, sizeof(int), plan->ctx->stream));
    set_error("a device-side wait timed out in the sweep kernel");
    return OBTE_ERR_DEVICE_TIMEOUT;
  }
  return OBTE_OK;
}

}  // namespace obte
