// Periodic-inflow block preconditioner of the GMRES on the sweep fixed point.
//
// The state carries, per ordinate, the temperatures entering the cell across the cut periodic faces
// (openbte/bte.py:99-110 couples the two sides of each periodic pair inside one sparse solve; here
// that coupling is an unknown of the fixed point, see krylov.cu).  One sweep carries an inflow one
// period further.  An ordinate whose rays run through the cell without meeting a wall — a direction
// along a lattice axis of the periodic cell, beside the pore — at a mean free path much longer than
// the cell keeps most of its inflow after a period: its one-period transfer T (source slots ->
// source slots) has a spectral radius near exp(-L / mfp) ~ 0.99, and GMRES spends an iteration on
// almost every such ordinate.  The right preconditioner M^-1 = I + sum_b E_b ((I - T_b)^-1 - I) E_b^T
// applies the exact inverse of those blocks, so (I - K) M^-1 is close to the identity on them.
//
// Setup, once per plan (by default on its second solve: a plan solved once does not pay for it), with
// FP32 sweeps of zero temperature and wall inputs, which isolate the inflow -> outflow map:
//   1. detection: ten applications of the map to an all-ones inflow; an ordinate is slow when the
//      last application kept more than 35 % of its inflow norm (and had not underflowed); its block
//      covers the source slots that iterate reached;
//   2. probing: for slot j of every slow ordinate's direction, a sweep of the unit inflow e_j gives
//      column j of every slow block at once (the ordinates do not interact); only the CTAs of the
//      slow (direction, MFP chunk) pairs run;
//   3. one CTA per block inverts I - T in place by Gauss-Jordan in FP32: T >= 0 with row sums below
//      one makes I - T strictly diagonally dominant, so no pivoting is needed; a block whose pivot
//      falls below 1e-5 is dropped.
// The preconditioner only changes the Krylov space, not the fixed point: the convergence test stays
// on the true residual ‖F(u) - u‖.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "internal.h"

namespace obte {

namespace {

constexpr int XT = 256;
constexpr int kDetect = 10;        // applications of the inflow map in the detection (OBTE_XPREC_DETECT)
constexpr double kSlow = 0.35;     // norm kept by the last application above which an ordinate is slow
                                   // (OBTE_XPREC_SLOW)
constexpr int kMaxSlots = 1024;    // largest block (OBTE_XPREC_MAX_SLOTS, at most kSlotsCap)
constexpr int kSlotsCap = 4096;    // the inversion kernel's column buffer
constexpr double kActive = 0.0;    // slots of a block: detection iterate above this fraction of its largest
                                   // (OBTE_XPREC_ACTIVE; 1e-3 took the largest block 348 -> 298 slots and
                                   // the setup 400 -> 294 ms but cost a sweep per solve on the 60k cell)
constexpr double kMaxBytes = 1.0e9;  // dense blocks' memory (OBTE_XPREC_MAX_GB)

int max_slots() {
  int v = kMaxSlots;
  if (const char* e = std::getenv("OBTE_XPREC_MAX_SLOTS")) v = std::atoi(e);
  return std::max(1, std::min(v, kSlotsCap));
}

double max_bytes() {
  double v = kMaxBytes;
  if (const char* e = std::getenv("OBTE_XPREC_MAX_GB")) v = std::atof(e) * 1e9;
  return v > 0 ? v : kMaxBytes;
}

// per-ordinate sum of squares of the inflow part: out[q * n_mfp + m]
__global__ void xnorm_kernel(const double* __restrict__ x, int64_t xoff, const int64_t* __restrict__ x_base,
                             int n_mfp, double* __restrict__ out) {
  const int q = blockIdx.x;
  const int64_t b0 = x_base[q], b1 = x_base[q + 1];
  for (int m = threadIdx.x; m < n_mfp; m += blockDim.x) {
    double s = 0;
    for (int64_t slot = b0; slot < b1; ++slot) {
      const double v = x[xoff + slot * n_mfp + m];
      s += v * v;
    }
    out[(int64_t)q * n_mfp + m] = s;
  }
}

__global__ void fill_kernel(double* __restrict__ x, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * XT + threadIdx.x; i < n; i += (int64_t)gridDim.x * XT) x[i] = v;
}

// Block b covers MFP m_b and the s_b source slots slot[off_b .. off_b + s_b) of its direction:
// X(b, i) = xoff + slot[off_b + i] n_mfp + m_b.
// probes j0 .. j0 + nj - 1 on the state vectors x + t stride (t = j - j0): x_t[X(b, j)] = v for every block
// with j < s_b
__global__ void xprobe_set_kernel(int nblk, const int32_t* __restrict__ bm, const int32_t* __restrict__ bs,
                                  const int64_t* __restrict__ boff, const int32_t* __restrict__ bslot, int n_mfp,
                                  int64_t xoff, int j0, int nj, int64_t stride, double v, double* __restrict__ x) {
  for (int e = blockIdx.x * XT + threadIdx.x; e < nblk * nj; e += gridDim.x * XT) {
    const int b = e / nj, t = e - b * nj;
    if (j0 + t < bs[b]) x[(int64_t)t * stride + xoff + (int64_t)bslot[boff[b] + j0 + t] * n_mfp + bm[b]] = v;
  }
}

// W blocks are row-major with rows padded to a multiple of 4 floats (16-byte rows for vector loads);
// the padding stays zero
__host__ __device__ __forceinline__ int row_stride(int s) { return (s + 3) & ~3; }

// column j = j0 + blockIdx.y of every block (blockIdx.x) from the state y + blockIdx.y stride:
// W_b[i][j] = y[X(b, i)]
__global__ void xprobe_get_kernel(const int32_t* __restrict__ bm, const int32_t* __restrict__ bs,
                                  const int64_t* __restrict__ boff, const int32_t* __restrict__ bslot,
                                  const int64_t* __restrict__ bwoff, int n_mfp, int64_t xoff, int j0, int64_t stride,
                                  const double* __restrict__ ybase, float* __restrict__ W) {
  const int b = blockIdx.x;
  const int s = bs[b], sp = row_stride(s);
  const int j = j0 + (int)blockIdx.y;
  const double* __restrict__ y = ybase + (int64_t)blockIdx.y * stride;
  if (j >= s) return;
  float* Wb = W + bwoff[b];
  const int32_t* sl = bslot + boff[b];
  const int64_t mb = xoff + bm[b];
  for (int i = threadIdx.x; i < s; i += blockDim.x) Wb[(int64_t)i * sp + j] = (float)y[mb + (int64_t)sl[i] * n_mfp];
}

// In place: W_b holds T_b on entry and (I - T_b)^-1 - I on exit (Gauss-Jordan without pivoting, FP32).
// A block whose pivot falls below 1e-5 is zeroed (no preconditioning on it) and flagged in bad[b].
__global__ void __launch_bounds__(1024) xprec_invert_kernel(const int32_t* __restrict__ bs,
                                                            const int64_t* __restrict__ bwoff, float* __restrict__ W,
                                                            int* __restrict__ bad) {
  __shared__ float colk[kSlotsCap];
  const int b = blockIdx.x;
  const int s = bs[b], sp = row_stride(s);
  float* A = W + bwoff[b];
  const int64_t ss = (int64_t)s * s;
  for (int64_t e = threadIdx.x; e < ss; e += blockDim.x) {
    const int i = (int)(e / s), j = (int)(e - (int64_t)i * s);
    A[(int64_t)i * sp + j] = (i == j ? 1.0f : 0.0f) - A[(int64_t)i * sp + j];
  }
  __syncthreads();
  for (int k = 0; k < s; ++k) {
    for (int i = threadIdx.x; i < s; i += blockDim.x) colk[i] = A[(int64_t)i * sp + k];
    __syncthreads();
    const float piv = colk[k];
    if (!(piv > 1e-5f)) {                       // same value in every thread: a uniform exit
      for (int64_t e = threadIdx.x; e < (int64_t)s * sp; e += blockDim.x) A[e] = 0.0f;
      if (threadIdx.x == 0) bad[b] = 1;
      return;
    }
    const float p = 1.0f / piv;
    for (int j = threadIdx.x; j < s; j += blockDim.x) A[(int64_t)k * sp + j] = (j == k) ? p : A[(int64_t)k * sp + j] * p;
    __syncthreads();
    for (int64_t e = threadIdx.x; e < ss; e += blockDim.x) {
      const int i = (int)(e / s);
      if (i == k) continue;
      const int j = (int)(e - (int64_t)i * s);
      A[(int64_t)i * sp + j] = (j == k) ? -colk[i] * p : A[(int64_t)i * sp + j] - colk[i] * A[(int64_t)k * sp + j];
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < s; i += blockDim.x) A[(int64_t)i * sp + i] -= 1.0f;
}

// out[X(b, i)] += sum_j W_b[i][j] in[X(b, j)]: one CTA per block, the block's inflow staged in shared
// memory (zero-padded to the row stride), one warp per pair of rows, 16-byte loads of W (fixed summation
// order).  Acc = float for stages whose Krylov basis is FP32 (GB300's FP64 pipe would bound the FP64
// form), double otherwise.
template <typename Acc>
__global__ void xprec_apply_kernel(const int32_t* __restrict__ bm, const int32_t* __restrict__ bs,
                                   const int64_t* __restrict__ boff, const int32_t* __restrict__ bslot,
                                   const int64_t* __restrict__ bwoff, const float* __restrict__ W, int n_mfp,
                                   int64_t xoff, const double* __restrict__ in, double* __restrict__ out) {
  extern __shared__ double xin_raw[];
  Acc* xin = reinterpret_cast<Acc*>(xin_raw);
  const int b = blockIdx.x;
  const int s = bs[b], sp = row_stride(s);
  const int32_t* sl = bslot + boff[b];
  const int64_t mb = xoff + bm[b];
  for (int i = threadIdx.x; i < sp; i += blockDim.x) xin[i] = i < s ? (Acc)in[mb + (int64_t)sl[i] * n_mfp] : Acc(0);
  __syncthreads();
  const float* Wb = W + bwoff[b];
  const int lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int q4 = sp >> 2;                                  // float4 per row
  for (int r0 = 2 * (threadIdx.x >> 5); r0 < s; r0 += 2 * nw) {
    const bool two = r0 + 1 < s;
    const float4* w0 = reinterpret_cast<const float4*>(Wb + (int64_t)r0 * sp);
    const float4* w1 = reinterpret_cast<const float4*>(Wb + (int64_t)(two ? r0 + 1 : r0) * sp);
    Acc a0 = 0, a1 = 0;
    for (int c = lane; c < q4; c += 32) {
      const float4 u = w0[c], v = w1[c];
      const Acc x0 = xin[4 * c], x1 = xin[4 * c + 1], x2 = xin[4 * c + 2], x3 = xin[4 * c + 3];
      a0 += (Acc)u.x * x0 + (Acc)u.y * x1 + (Acc)u.z * x2 + (Acc)u.w * x3;
      a1 += (Acc)v.x * x0 + (Acc)v.y * x1 + (Acc)v.z * x2 + (Acc)v.w * x3;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    if (lane == 0) {
      out[mb + (int64_t)sl[r0] * n_mfp] += (double)a0;
      if (two) out[mb + (int64_t)sl[r0 + 1] * n_mfp] += (double)a1;
    }
  }
}

int blocks_for(int64_t n, int num_sms) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + XT - 1) / XT, (int64_t)num_sms * 8));
}

}  // namespace

void xprec_add(obte_plan plan, const double* in, double* out, bool fp32) {
  const XPrec& P = *plan->xprec;
  if (P.nblk == 0) return;
  const Schedule& s = plan->sched;
  auto kern = fp32 ? xprec_apply_kernel<float> : xprec_apply_kernel<double>;
  kern<<<P.nblk, XT, (size_t)row_stride(P.smax) * sizeof(double), plan->stream>>>(
      P.bm.as<int32_t>(), P.bs.as<int32_t>(), P.boff.as<int64_t>(), P.bslot.as<int32_t>(), P.bwoff.as<int64_t>(),
      P.W.as<float>(), s.n_mfp, s.n + s.nd, in, out);
  count_launch();
}

int64_t xprec_resident_bytes(const XPrec* P) {
  if (!P) return 0;
  return (int64_t)(P->bm.bytes + P->bs.bytes + P->boff.bytes + P->bwoff.bytes + P->bslot.bytes + P->W.bytes);
}

int64_t xprec_build_bound(obte_plan plan) {
  if (plan->xprec && plan->xprec->tried) return 0;
  const Schedule& s = plan->sched;
  const int64_t nsrc = s.x_base.empty() ? 0 : s.x_base[s.n_dir];
  bool any_fits = false;
  for (int q = 0; q < s.n_dir && !any_fits; ++q) {
    const int64_t nsl = s.x_base[q + 1] - s.x_base[q];
    any_fits = nsl > 0 && nsl <= max_slots();
  }
  if (nsrc == 0 || s.n_mfp == 0 || !any_fits) return 0;
  const int64_t nord = (int64_t)s.n_dir * s.n_mfp;
  const int64_t nu = plan->nu;
  // W (capped), per-block tables (at most one block per ordinate, every block's slots at most its
  // direction's), detection norms, CTA map, the batched probe vectors (16 pairs or 2 GB at most)
  const int64_t probes = std::min<int64_t>(16 * 2 * nu * (int64_t)sizeof(double), (int64_t)2e9);
  return (int64_t)max_bytes() + nord * (4 + 4 + 8 + 8 + 4 + 16 + 4) + nsrc * s.n_mfp * 4 + probes;
}

obte_status ensure_xprec(obte_plan plan, SolveWork& wk) {
  if (plan->xprec && plan->xprec->tried) return OBTE_OK;
  plan->xprec.reset(new XPrec());
  XPrec& P = *plan->xprec;
  P.tried = true;
  const Schedule& s = plan->sched;
  const int64_t nsrc = s.x_base[s.n_dir];
  if (nsrc == 0 || s.n_mfp == 0) return OBTE_OK;
  // a block spans at most all source slots of its direction: nothing to build where every direction has
  // more than kMaxSlots (the 3D meshes' periodic faces)
  bool any_fits = false;
  for (int q = 0; q < s.n_dir && !any_fits; ++q) {
    const int64_t nsl = s.x_base[q + 1] - s.x_base[q];
    any_fits = nsl > 0 && nsl <= max_slots();
  }
  if (!any_fits) return OBTE_OK;
  OBTE_TRY(ensure_tables(plan, true));
  PhaseTimer timer("xprec setup");
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = plan->stream;
  const int num_sms = plan->ctx->num_sms;
  const int64_t xoff = s.n + s.nd;
  const int64_t nu = plan->nu;
  double* x = wk.tmp.as<double>();
  double* y = wk.w.as<double>();
  // 1. detection: inflow map applied to an all-ones inflow
  OBTE_CUDA(cudaMemsetAsync(x, 0, (size_t)xoff * sizeof(double), st));
  fill_kernel<<<blocks_for(nu - xoff, num_sms), XT, 0, st>>>(x + xoff, nu - xoff, 1.0);
  count_launch();
  int n_detect = kDetect;
  double slow = kSlow;
  if (const char* e = std::getenv("OBTE_XPREC_DETECT")) n_detect = std::max(2, std::atoi(e));
  if (const char* e = std::getenv("OBTE_XPREC_SLOW")) slow = std::atof(e);
  double active = kActive;
  if (const char* e = std::getenv("OBTE_XPREC_ACTIVE")) active = std::atof(e);
  const int64_t nord = (int64_t)s.n_dir * s.n_mfp;
  DevBuf nrm;
  OBTE_TRY(nrm.alloc((size_t)nord * 2 * sizeof(double)));
  for (int it = 0; it < n_detect; ++it) {
    if (it == n_detect - 1) {
      xnorm_kernel<<<s.n_dir, XT, 0, st>>>(x, xoff, plan->x_base_dev.as<int64_t>(), s.n_mfp, nrm.as<double>());
      count_launch();
    }
    OBTE_TRY(launch_sweep(plan, true, x, y, false, false, nullptr, nullptr, nullptr));
    OBTE_CUDA(cudaMemsetAsync(y, 0, (size_t)xoff * sizeof(double), st));
    std::swap(x, y);
  }
  xnorm_kernel<<<s.n_dir, XT, 0, st>>>(x, xoff, plan->x_base_dev.as<int64_t>(), s.n_mfp, nrm.as<double>() + nord);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  std::vector<double> hn((size_t)nord * 2);
  OBTE_CUDA(cudaMemcpyAsync(hn.data(), nrm.p, hn.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  OBTE_CUDA(wait_stream(st));
  P.detect_sweeps = n_detect;
  struct Cand { int q, m; double ratio; std::vector<int32_t> slots; };
  std::vector<Cand> cand;
  std::vector<double> hx;
  for (int q = 0; q < s.n_dir; ++q) {
    const int64_t nsl = s.x_base[q + 1] - s.x_base[q];
    if (nsl == 0) continue;
    std::vector<int> ms;
    for (int m = 0; m < s.n_mfp; ++m) {
      const double a = hn[(size_t)q * s.n_mfp + m], b = hn[(size_t)nord + (size_t)q * s.n_mfp + m];
      const double ratio = a > 0 ? std::sqrt(b / a) : 0.0;
      // fast ordinates' FP32 iterates underflow into denormals, where they stop shrinking (ratio ~1):
      // only an inflow that kept more than 1e-12 of its initial norm (sum of squares = slots) counts
      if (ratio > slow && b > 1e-24 * (double)nsl) ms.push_back(m);
    }
    if (ms.empty()) continue;
    // the block covers the slots where the detection iterate (>= 0, near the slowest mode) is above
    // `active` of its largest value (by default every slot it reached)
    hx.resize((size_t)nsl * s.n_mfp);
    OBTE_CUDA(cudaMemcpyAsync(hx.data(), x + xoff + s.x_base[q] * s.n_mfp, hx.size() * sizeof(double),
                              cudaMemcpyDeviceToHost, st));
    OBTE_CUDA(wait_stream(st));
    for (int m : ms) {
      double vmax = 0;
      for (int64_t i = 0; i < nsl; ++i) vmax = std::max(vmax, hx[(size_t)i * s.n_mfp + m]);
      Cand c{q, m, 0.0, {}};
      const double a = hn[(size_t)q * s.n_mfp + m], b = hn[(size_t)nord + (size_t)q * s.n_mfp + m];
      c.ratio = std::sqrt(b / a);
      for (int64_t i = 0; i < nsl; ++i)
        if (hx[(size_t)i * s.n_mfp + m] > active * vmax) c.slots.push_back((int32_t)(s.x_base[q] + i));
      if (!c.slots.empty() && (int)c.slots.size() <= max_slots()) cand.push_back(std::move(c));
    }
  }
  // memory cap: keep the slowest blocks
  std::stable_sort(cand.begin(), cand.end(), [](const Cand& a, const Cand& b) { return a.ratio > b.ratio; });
  double bytes = 0;
  size_t keep = 0;
  for (; keep < cand.size(); ++keep) {
    const int sz = (int)cand[keep].slots.size();
    const double bb = (double)sz * row_stride(sz) * sizeof(float);
    if (bytes + bb > max_bytes()) break;
    bytes += bb;
  }
  cand.resize(keep);
  std::stable_sort(cand.begin(), cand.end(), [](const Cand& a, const Cand& b) { return a.q != b.q ? a.q < b.q : a.m < b.m; });
  if (cand.empty()) {
    P.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return OBTE_OK;
  }
  const int nblk = (int)cand.size();
  std::vector<int32_t> bm(nblk), bsz(nblk), bslot;
  std::vector<int64_t> boff(nblk), bwoff(nblk);
  int64_t woff = 0;
  int smax = 0;
  for (int b = 0; b < nblk; ++b) {
    const int sz = (int)cand[b].slots.size();
    bm[b] = cand[b].m;
    bsz[b] = sz;
    boff[b] = (int64_t)bslot.size();
    bslot.insert(bslot.end(), cand[b].slots.begin(), cand[b].slots.end());
    bwoff[b] = woff;
    woff += (int64_t)sz * row_stride(sz);
    smax = std::max(smax, sz);
  }
  OBTE_TRY(upload(P.bm, bm, st));
  OBTE_TRY(upload(P.bs, bsz, st));
  OBTE_TRY(upload(P.boff, boff, st));
  OBTE_TRY(upload(P.bslot, bslot, st));
  OBTE_TRY(upload(P.bwoff, bwoff, st));
  OBTE_TRY(P.W.alloc((size_t)woff * sizeof(float)));
  OBTE_CUDA(cudaMemsetAsync(P.W.p, 0, (size_t)woff * sizeof(float), st));   // row padding stays zero
  // 2. probing on the CTAs of the slow (direction, MFP chunk) pairs
  const DevSchedule& d = plan->d32;
  std::vector<int32_t> ctas;
  for (const Cand& c : cand) {
    const int id = c.q * d.n_chunks + c.m / d.mc;
    if (ctas.empty() || ctas.back() != id) ctas.push_back(id);
  }
  ctas.erase(std::unique(ctas.begin(), ctas.end()), ctas.end());
  DevBuf cmap;
  OBTE_TRY(upload(cmap, ctas, st));
  // a probe sweep runs only these CTAs (one chain each, a small part of the GPU): `nbat` probes share a
  // launch, each on its own pair of state vectors (all with zero DeltaT and T_B, as batching requires)
  const int nbat = (int)std::max<int64_t>(
      1, std::min<int64_t>({16, (int64_t)num_sms * 4 / (int64_t)ctas.size(), (int64_t)(2e9 / (16.0 * (double)nu))}));
  DevBuf xb, yb;
  OBTE_TRY(xb.alloc((size_t)nbat * nu * sizeof(double)));
  OBTE_TRY(yb.alloc((size_t)nbat * nu * sizeof(double)));
  OBTE_CUDA(cudaMemsetAsync(xb.p, 0, (size_t)nbat * nu * sizeof(double), st));
  plan->sweep_cta_map = cmap.as<int32_t>();
  plan->sweep_n_cta = (int)ctas.size();
  plan->sweep_batch_stride = nu;
  obte_status ps = OBTE_OK;
  int launches = 0;
  for (int j0 = 0; j0 < smax && ps == OBTE_OK; j0 += nbat) {
    const int nj = std::min(nbat, smax - j0);
    const int sb = blocks_for((int64_t)nblk * nj, num_sms);
    plan->sweep_batch = nj;
    xprobe_set_kernel<<<sb, XT, 0, st>>>(nblk, P.bm.as<int32_t>(), P.bs.as<int32_t>(), P.boff.as<int64_t>(),
                                         P.bslot.as<int32_t>(), s.n_mfp, xoff, j0, nj, nu, 1.0, xb.as<double>());
    ps = launch_sweep(plan, true, xb.as<double>(), yb.as<double>(), false, false, nullptr, nullptr, nullptr);
    if (ps != OBTE_OK) break;
    ++launches;
    xprobe_get_kernel<<<dim3(nblk, nj), XT, 0, st>>>(P.bm.as<int32_t>(), P.bs.as<int32_t>(), P.boff.as<int64_t>(),
                                                     P.bslot.as<int32_t>(), P.bwoff.as<int64_t>(), s.n_mfp, xoff, j0,
                                                     nu, yb.as<double>(), P.W.as<float>());
    xprobe_set_kernel<<<sb, XT, 0, st>>>(nblk, P.bm.as<int32_t>(), P.bs.as<int32_t>(), P.boff.as<int64_t>(),
                                         P.bslot.as<int32_t>(), s.n_mfp, xoff, j0, nj, nu, 0.0, xb.as<double>());
    count_launch(3);
  }
  plan->sweep_cta_map = nullptr;
  plan->sweep_n_cta = 0;
  plan->sweep_batch = 1;
  plan->sweep_batch_stride = 0;
  OBTE_TRY(ps);
  P.probe_sweeps = launches;
  // 3. (I - T)^-1 - I per block
  DevBuf bad;
  OBTE_TRY(bad.alloc((size_t)nblk * sizeof(int)));
  OBTE_CUDA(cudaMemsetAsync(bad.p, 0, (size_t)nblk * sizeof(int), st));
  xprec_invert_kernel<<<nblk, 1024, 0, st>>>(P.bs.as<int32_t>(), P.bwoff.as<int64_t>(), P.W.as<float>(), bad.as<int>());
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  OBTE_CUDA(wait_stream(st));
  OBTE_TRY(check_device_error(plan));
  P.nblk = nblk;
  P.smax = smax;
  P.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (timer.on)
    std::fprintf(stderr, "[obte trace] xprec: %d blocks (largest %d slots), %zu CTAs per probe, %d probes in %d "
                 "batched sweeps of %d\n", nblk, smax, ctas.size(), smax, P.probe_sweeps, nbat);
  return OBTE_OK;
}

}  // namespace obte
