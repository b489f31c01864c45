// Batched upwind transport sweep for sm_103a.
//
// One CTA = one direction q x one chunk of 32 mean free paths (lane = MFP).
// The CTA walks the direction's elements level by level (longest-path layers
// of the upwind DAG, periodic inflow cut); inside a level every warp takes one
// element at a time, all 32 lanes solving that element for their own MFP:
//
//   T_mq[c] = (DeltaT[c] + h[c] + L_m P_q[c] - L_m sum_in g_f T_up) / (1 + L_m D_q[c])
//
// which is the row of A_mq T = B of openbte/bte.py:183-218 for an element whose
// upwind neighbours are already known.  T_up comes from
//   - the shared-memory slot of an upstream element (ITEM_CELL),
//   - the periodic-inflow part of the state vector (ITEM_PERIODIC),
//   - the wall temperature T_B (ITEM_WALL, openbte/bte.py:200,214).
// Values of T never leave the SM except where the path needs them; the
// reductions of openbte/bte.py:222-243 are fused:
//   DeltaT'[c] += sum_m t_mq T        (warp shuffle, then one FP64 atomic)
//   T_B'[w]    += sum_m (-GG) T       (walls)
//   x'         = T at periodic source elements (interface unknowns)
//   final pass: J += sum_m sigma_mq T, K_mq / S_mq in registers per lane.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"

namespace obte {

template <typename Real>
struct SweepParams {
  int64_t n;
  int64_t nd;
  int n_mfp, m_pad, n_chunks, n_dir, ds;
  const int32_t* __restrict__ cell;
  const int32_t* __restrict__ slot;
  const int32_t* __restrict__ xk;
  const int32_t* __restrict__ wout;
  const int32_t* __restrict__ contact;
  const int32_t* __restrict__ in_idx;
  const int32_t* __restrict__ lev_ptr;
  const int64_t* __restrict__ lev_off;
  const int32_t* __restrict__ nlev;
  const int64_t* __restrict__ x_base;
  const int32_t* __restrict__ wo_wall;
  const Real* __restrict__ in_coef;
  const Real* __restrict__ D;
  const Real* __restrict__ P;
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
  int with_src;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename Real, int NF, bool FINAL>
__global__ void __launch_bounds__(256) bte_sweep_kernel(const SweepParams<Real> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* buf = reinterpret_cast<Real*>(smem_raw);  // [slots][32]

  const int q = blockIdx.x / p.n_chunks;
  const int chunk = blockIdx.x - q * p.n_chunks;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int m = chunk * 32 + lane;
  const bool active = m < p.n_mfp;

  const Real lam = p.mfp[m];
  const Real tq = p.tco[(int64_t)q * p.m_pad + m];
  Real sg[3] = {0, 0, 0};
  if (FINAL) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (d < p.ds) sg[d] = p.sig[((int64_t)q * p.m_pad + m) * p.ds + d];
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
  const int64_t base = (int64_t)q * p.n;
  const bool src = p.with_src != 0;

  Real kacc = 0, sacc = 0;
  for (int L = 0; L < nlev; ++L) {
    const int b = lev[L];
    const int e = lev[L + 1];
    for (int pos = b + warp; pos < e; pos += nw) {
      const int64_t it = base + pos;
      const int c = p.cell[it];
      Real acc = (Real)dT[c];
      if (src) {
        acc += lam * p.P[it];
        if (p.hs) acc += p.hs[c];
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const int32_t code = p.in_idx[it * NF + f];
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
        acc -= lam * p.in_coef[it * NF + f] * v;
      }
      const Real T = acc / (Real(1) + lam * p.D[it]);
      const int sl = p.slot[it];
      if (sl >= 0) buf[sl * 32 + lane] = T;

      const Real r = warp_sum(tq * T);
      if (lane == 0) atomicAdd(&dT_out[c], (double)r);
      const int xk = p.xk[it];
      if (xk >= 0 && active) X_out[(xq + xk) * p.n_mfp + m] = (double)T;
      const int wo = p.wout[it];
      if (wo) {
        const int wb = wo >> 3, wn = wo & 7;
        for (int k = 0; k < wn; ++k) {
          const Real rw = warp_sum(p.wo_gg[(int64_t)(wb + k) * p.m_pad + m] * T);
          if (lane == 0) atomicAdd(&TB_out[p.wo_wall[wb + k]], (double)rw);
        }
      }
      if (FINAL) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (d < p.ds) {
            const Real rj = warp_sum(sg[d] * T);
            if (lane == 0) atomicAdd(&p.Jraw[(int64_t)c * p.ds + d], (double)rj);
          }
        }
        const int ce = p.contact[it];
        if (ce >= 0) {
          kacc += p.kcoef[(int64_t)ce * p.m_pad + m] * T;
          sacc += p.scoef[ce] * T;
        }
      }
    }
    __syncthreads();
  }
  if (FINAL) {
    // reduce the per-warp K/S partials (buf is free after the last barrier)
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
  const DevBuf* all[] = {&cell, &slot, &xk, &wout, &contact, &in_idx, &in_coef, &D, &P, &lev_ptr,
                         &mfp, &tco, &sig, &wo_wall, &wo_gg, &kcoef, &scoef, &hs};
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

template <typename Real>
static obte_status upload_tables(obte_plan plan, DevSchedule& d) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->ctx->stream;
  OBTE_TRY(upload(d.cell, s.cell, st));
  OBTE_TRY(upload(d.slot, s.slot, st));
  OBTE_TRY(upload(d.xk, s.xk, st));
  OBTE_TRY(upload(d.wout, s.wout, st));
  OBTE_TRY(upload(d.contact, s.contact, st));
  OBTE_TRY(upload(d.in_idx, s.in_idx, st));
  OBTE_TRY(upload(d.lev_ptr, s.lev_ptr, st));
  std::vector<int32_t> wo = s.wo_wall;
  if (wo.empty()) wo.push_back(0);
  OBTE_TRY(upload(d.wo_wall, wo, st));
  OBTE_TRY(upload_real<Real>(d.in_coef, s.in_coef, st));
  OBTE_TRY(upload_real<Real>(d.D, s.D, st));
  OBTE_TRY(upload_real<Real>(d.P, s.P, st));
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
  const int threads = 256;
  const int nw = threads / 32;
  size_t smem = (size_t)std::max(s.max_slots, 2 * nw) * 32 * sizeof(Real);
  if (smem > plan->ctx->smem_optin) {
    set_error("sweep front needs " + std::to_string(smem) + " B of shared memory, above the per-CTA limit");
    return OBTE_ERR_UNSUPPORTED;
  }
  auto kern = bte_sweep_kernel<Real, NF, FINAL>;
  OBTE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SweepParams<Real> p;
  p.n = s.n; p.nd = s.nd; p.n_mfp = s.n_mfp; p.m_pad = s.m_pad; p.n_chunks = s.n_chunks; p.n_dir = s.n_dir;
  p.ds = s.ds;
  p.cell = d.cell.as<int32_t>(); p.slot = d.slot.as<int32_t>(); p.xk = d.xk.as<int32_t>();
  p.wout = d.wout.as<int32_t>(); p.contact = d.contact.as<int32_t>(); p.in_idx = d.in_idx.as<int32_t>();
  p.lev_ptr = d.lev_ptr.as<int32_t>();
  p.lev_off = plan->lev_off_dev.as<int64_t>(); p.nlev = plan->nlev_dev.as<int32_t>();
  p.x_base = plan->x_base_dev.as<int64_t>();
  p.wo_wall = d.wo_wall.as<int32_t>();
  p.in_coef = d.in_coef.as<Real>(); p.D = d.D.as<Real>(); p.P = d.P.as<Real>(); p.mfp = d.mfp.as<Real>();
  p.tco = d.tco.as<Real>(); p.sig = d.sig.as<Real>(); p.wo_gg = d.wo_gg.as<Real>();
  p.kcoef = d.kcoef.as<Real>(); p.scoef = d.scoef.as<Real>();
  p.hs = s.hs.empty() ? nullptr : d.hs.as<Real>();
  p.u_in = u_in; p.u_out = u_out; p.Jraw = Jraw; p.K = K; p.S = S; p.with_src = with_src ? 1 : 0;
  const int grid = s.n_dir * s.n_chunks;
  kern<<<grid, threads, smem, plan->ctx->stream>>>(p);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  return OBTE_OK;
}

obte_status launch_sweep(obte_plan plan, bool fp32, const double* u_in, double* u_out, bool with_src,
                         bool final_pass, double* Jraw, double* K, double* S) {
  OBTE_TRY(ensure_tables(plan, fp32));
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->ctx->stream;
  OBTE_CUDA(cudaMemsetAsync(u_out, 0, (size_t)(s.n + s.nd) * sizeof(double), st));
  if (final_pass) OBTE_CUDA(cudaMemsetAsync(Jraw, 0, (size_t)s.n * s.ds * sizeof(double), st));
  if (s.ds > 3) { set_error("sigma with more than 3 components"); return OBTE_ERR_UNSUPPORTED; }
#define OBTE_DISPATCH(R, DS)                                                                        \
  do {                                                                                              \
    if (s.nf == 3) {                                                                                \
      if (final_pass) return launch_impl<R, 3, true>(plan, DS, u_in, u_out, with_src, Jraw, K, S);  \
      return launch_impl<R, 3, false>(plan, DS, u_in, u_out, with_src, Jraw, K, S);                 \
    } else if (s.nf == 4) {                                                                         \
      if (final_pass) return launch_impl<R, 4, true>(plan, DS, u_in, u_out, with_src, Jraw, K, S);  \
      return launch_impl<R, 4, false>(plan, DS, u_in, u_out, with_src, Jraw, K, S);                 \
    }                                                                                               \
  } while (0)
  if (fp32) OBTE_DISPATCH(float, plan->d32);
  else OBTE_DISPATCH(double, plan->d64);
#undef OBTE_DISPATCH
  set_error("elements with this many sides are not supported");
  return OBTE_ERR_UNSUPPORTED;
}

}  // namespace obte
