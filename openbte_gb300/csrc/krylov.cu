// Source iteration driver: GMRES on the sweep fixed point.
//
// The reference iterates u <- F(u) with exact per-ordinate solves
// (openbte/bte.py:196-256), u = (DeltaT, T_B).  Here the state also carries
// the periodic inflow of every ordinate, so that one sweep evaluates F
// exactly without a sparse factorisation.  F is affine, F(u) = K u + f, and
// the fixed point solves (I - K) u = f, done with restarted GMRES (one sweep
// per Krylov vector, classical Gram-Schmidt with one re-orthogonalisation).
//
// I - K is singular along the constant mode (a uniform shift of every
// temperature is a fixed point of the homogeneous map).  The reference's
// Jacobi iteration conserves ell.u with ell = (element volumes, wall weights
// A_w sum_mq t_mq L_m |min(s_q.n_w, 0)|), the left null vector of I - K; the
// converged state is therefore shifted by a constant so that ell.u equals its
// value at the initial guess, reproducing the reference's temperature level.
// Isothermal (mixed) walls emit at a fixed temperature: the constant mode is
// then not a fixed point, the solution is unique and no shift is applied.
//
// Precision modes: FP64 sweeps; FP32 sweeps; FP32 sweeps inside an iterative
// refinement whose residual F(u) - u is evaluated with FP64 sweeps.  The
// solution, residuals, cross-block reductions and the Hessenberg system are
// FP64 in every mode; the Krylov basis is FP32 in stages that sweep in FP32 to a
// relative tolerance of 1e-6 or looser (the inner solves of the refinement),
// FP64 otherwise.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "internal.h"

namespace obte {

namespace {

constexpr int VT = 256;       // threads per vector block
constexpr int DOT_TILE = 8;   // vectors per multidot pass

int vec_blocks(const obte_plan plan, int64_t n) {
  const int64_t want = (n + VT - 1) / VT;
  const int64_t cap = (int64_t)plan->ctx->num_sms * 4;
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

// partial[b * kk + j] = sum over block b's range of V[j*ld + i] * w[i] for j < k, and w.w for
// j == k when self != 0 (kk = k + self)
__global__ void __launch_bounds__(VT) multidot_kernel(const double* __restrict__ V, int64_t ld, int k, int self,
                                                      const double* __restrict__ w, int64_t n,
                                                      double* __restrict__ partial, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[VT / 32][DOT_TILE];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int kk = k + self;
  for (int jt = 0; jt < kk; jt += DOT_TILE) {
    double acc[DOT_TILE];
#pragma unroll
    for (int t = 0; t < DOT_TILE; ++t) acc[t] = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x; i < n; i += (int64_t)gridDim.x * VT) {
      const double wi = w[i];
#pragma unroll
      for (int t = 0; t < DOT_TILE; ++t) {
        const int j = jt + t;
        if (j < k) acc[t] += V[(int64_t)j * ld + i] * wi;
        else if (j < kk) acc[t] += wi * wi;
      }
    }
#pragma unroll
    for (int t = 0; t < DOT_TILE; ++t) {
      double v = acc[t];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < DOT_TILE && jt + (int)threadIdx.x < kk) {
      double v = 0;
      for (int w2 = 0; w2 < VT / 32; ++w2) v += red[w2][threadIdx.x];
      partial[(int64_t)blockIdx.x * kk + jt + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

// out[j] = sum_b partial[b * k + j]: one block per output, fixed summation tree (deterministic)
__global__ void __launch_bounds__(VT) reduce_partials_kernel(const double* __restrict__ partial, int nb, int k,
                                                             double* __restrict__ out) {
  __shared__ double red[VT / 32];
  const int j = blockIdx.x;
  double v = 0;
  for (int b = threadIdx.x; b < nb; b += VT) v += partial[(int64_t)b * k + j];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < VT / 32; ++w) t += red[w];
    out[j] = t;
  }
}

// w -= sum_j h[j] V[j]; partial[b] = sum over block b of the new w^2.  The coefficients sit in
// shared memory and the basis is read eight vectors at a time, so each thread keeps eight
// independent loads in flight instead of one load per dependent FMA.
constexpr int MAX_BASIS = 256;
__global__ void __launch_bounds__(VT) update_kernel(double* __restrict__ w, const double* __restrict__ V, int64_t ld,
                                                    int k, const double* __restrict__ h, int64_t n,
                                                    double* __restrict__ partial, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[VT / 32];
  __shared__ double hs[MAX_BASIS];
  for (int j = threadIdx.x; j < k; j += VT) hs[j] = h[j];
  __syncthreads();
  double ss = 0;
  for (int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x; i < n; i += (int64_t)gridDim.x * VT) {
    double acc = w[i];
    int j = 0;
    for (; j + 8 <= k; j += 8) {
      double v[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) v[t] = V[(int64_t)(j + t) * ld + i];
      double s = 0;
#pragma unroll
      for (int t = 0; t < 8; ++t) s += hs[j + t] * v[t];
      acc -= s;
    }
    for (; j < k; ++j) acc -= hs[j] * V[(int64_t)j * ld + i];
    w[i] = acc;
    ss += acc * acc;
  }
  if (partial) {
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w2 = 0; w2 < VT / 32; ++w2) t += red[w2];
      partial[blockIdx.x] = t;
    }
  }
}

// ---- FP32 Krylov basis (stages whose sweeps are FP32) ------------------------------------------
// On GB300 the FP64 pipe cannot keep up with HBM for one FMA per 8 loaded bytes, so the Gram-Schmidt
// passes of the FP32 stages keep the basis V and the new vector w in FP32: FP32 products and
// per-thread sums, FP64 across threads and blocks.  The sweep still takes FP64 input (one widening
// pass per Krylov vector) and the solution x stays FP64.

// The two Gram-Schmidt products read 16 bytes per load: V's rows (stride ld) and w must be 16-byte
// aligned (the FP32 basis rows are padded to a multiple of 4 floats); the n % 4 tail goes through
// block 0.  They run on fewer blocks than the elementwise kernels so that each thread streams several
// float4 per tile: with small states (0.9M entries) one scalar per thread and 8-vector tile left the
// per-tile reductions and barriers dominant.  Warp sums are FP32 (32 partial sums of a few elements
// each), FP64 from the warp level up: FP64 shuffles kept these kernels on the FP64 pipe.

// partial[b * kk + j] = block b's part of V[j] . w (j < k) and of w . w (j == k when self)
constexpr int DOT_TILE4 = 16;
__global__ void __launch_bounds__(VT) multidot32v_kernel(const float* __restrict__ V, int64_t ld, int k, int self,
                                                         const float* __restrict__ w, int64_t n,
                                                         double* __restrict__ partial, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[VT / 32][DOT_TILE4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int kk = k + self;
  const int64_t n4 = n >> 2;
  const float4* w4 = reinterpret_cast<const float4*>(w);
  for (int jt = 0; jt < kk; jt += DOT_TILE4) {
    const float* vp[DOT_TILE4];
#pragma unroll
    for (int t = 0; t < DOT_TILE4; ++t) vp[t] = jt + t < k ? V + (int64_t)(jt + t) * ld : w;   // self / padding read w
    float acc[DOT_TILE4];
#pragma unroll
    for (int t = 0; t < DOT_TILE4; ++t) acc[t] = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x; i < n4; i += (int64_t)gridDim.x * VT) {
      const float4 b = w4[i];
#pragma unroll
      for (int t = 0; t < DOT_TILE4; ++t) {
        const float4 a = reinterpret_cast<const float4*>(vp[t])[i];
        acc[t] = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, acc[t]))));
      }
    }
    if (blockIdx.x == 0)
      for (int64_t i = 4 * n4 + threadIdx.x; i < n; i += VT) {
        const float b = w[i];
#pragma unroll
        for (int t = 0; t < DOT_TILE4; ++t) acc[t] = fmaf(vp[t][i], b, acc[t]);
      }
#pragma unroll
    for (int t = 0; t < DOT_TILE4; ++t) {
      float v = acc[t];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][t] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < DOT_TILE4 && jt + (int)threadIdx.x < kk) {
      double v = 0;
      for (int w2 = 0; w2 < VT / 32; ++w2) v += red[w2][threadIdx.x];
      partial[(int64_t)blockIdx.x * kk + jt + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

// w -= sum_j h[j] V[j] (FP32); partial[b] = block b's part of the new w . w
__global__ void __launch_bounds__(VT) update32v_kernel(float* __restrict__ w, const float* __restrict__ V, int64_t ld,
                                                       int k, const double* __restrict__ h, int64_t n,
                                                       double* __restrict__ partial, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[VT / 32];
  __shared__ float hs[MAX_BASIS];
  for (int j = threadIdx.x; j < k; j += VT) hs[j] = (float)h[j];
  __syncthreads();
  const int64_t n4 = n >> 2;
  float4* w4 = reinterpret_cast<float4*>(w);
  float ss = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x; i < n4; i += (int64_t)gridDim.x * VT) {
    float4 acc = w4[i];
#pragma unroll 4
    for (int j = 0; j < k; ++j) {
      const float4 v = reinterpret_cast<const float4*>(V + (int64_t)j * ld)[i];
      const float c = -hs[j];
      acc.x = fmaf(c, v.x, acc.x);
      acc.y = fmaf(c, v.y, acc.y);
      acc.z = fmaf(c, v.z, acc.z);
      acc.w = fmaf(c, v.w, acc.w);
    }
    w4[i] = acc;
    ss = fmaf(acc.x, acc.x, fmaf(acc.y, acc.y, fmaf(acc.z, acc.z, fmaf(acc.w, acc.w, ss))));
  }
  if (blockIdx.x == 0)
    for (int64_t i = 4 * n4 + threadIdx.x; i < n; i += VT) {
      float acc = w[i];
      for (int j = 0; j < k; ++j) acc = fmaf(-hs[j], V[(int64_t)j * ld + i], acc);
      w[i] = acc;
      ss = fmaf(acc, acc, ss);
    }
  double sd = (double)ss;
  for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sd;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w2 = 0; w2 < VT / 32; ++w2) t += red[w2];
    partial[blockIdx.x] = t;
  }
}

// Device side of the Arnoldi step (no host round trip between the Gram-Schmidt passes).
// DGKS test after the first pass: skip[0] = 1 (no second pass) unless the projection left less than
// 0.7 of the norm w had before it (h[k] = w . w before, s[0] = w . w after).
__global__ void gs_check_kernel(const double* __restrict__ h, int k, const double* __restrict__ s,
                                int* __restrict__ skip) {
  if (threadIdx.x == 0) skip[0] = sqrt(fmax(s[0], 0.0)) < 0.7 * sqrt(fmax(h[k], 0.0)) ? 0 : 1;
}

// Hessenberg column of the step: col[i] = h[i] (+ h2[i] after a second pass) for i < k, col[k] = ‖w‖,
// col[k + 1] = 1 when the second pass ran; inv[0] = 1 / ‖w‖ in FP32 and inv64[0] in FP64 (0 for a zero
// vector).
__global__ void gs_finish_kernel(const double* __restrict__ h, const double* __restrict__ h2, int k,
                                 const double* __restrict__ s, const int* __restrict__ skip,
                                 double* __restrict__ col, float* __restrict__ inv, double* __restrict__ inv64) {
  const bool two = skip[0] == 0;
  for (int i = threadIdx.x; i < k; i += blockDim.x) col[i] = two ? h[i] + h2[i] : h[i];
  if (threadIdx.x == 0) {
    const double hn = sqrt(fmax(two ? s[1] : s[0], 0.0));
    col[k] = hn;
    col[k + 1] = two ? 1.0 : 0.0;
    inv[0] = hn > 0 ? (float)(1.0 / hn) : 0.f;
    inv64[0] = hn > 0 ? 1.0 / hn : 0.0;
  }
}

// y = a[0] x (scale read from the device)
__global__ void scaled_kernel(const double* __restrict__ a, const double* __restrict__ x, double* __restrict__ y,
                              int64_t n) {
  const double s = *a;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = s * x[i];
}
__global__ void scale32d_kernel(const float* __restrict__ a, const float* __restrict__ x, float* __restrict__ y,
                                int64_t n) {
  const float s = *a;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = s * x[i];
}

// x += sum_j y[j] V[j] (FP32 combination, FP64 accumulate into x)
__global__ void __launch_bounds__(VT) xupdate32_kernel(double* __restrict__ x, const float* __restrict__ V, int64_t ld,
                                                       int k, const double* __restrict__ y, int64_t n) {
  __shared__ float ys[MAX_BASIS];
  for (int j = threadIdx.x; j < k; j += VT) ys[j] = (float)y[j];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x; i < n; i += (int64_t)gridDim.x * VT) {
    float s = 0.f;
    for (int j = 0; j < k; ++j) s = fmaf(ys[j], V[(int64_t)j * ld + i], s);
    x[i] += (double)s;
  }
}

// y = (float)(a * x)
__global__ void scale_to_f32_kernel(double a, const double* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)(a * x[i]);
}
// y = (double)x
__global__ void widen_kernel(const float* __restrict__ x, double* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}
// w = (float)(a - b)
__global__ void diff_to_f32_kernel(const double* __restrict__ a, const double* __restrict__ b, float* __restrict__ w,
                                   int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = (float)(a[i] - b[i]);
}

// y = a*x + b*y
// y += x
__global__ void add_kernel(double* __restrict__ y, const double* __restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += x[i];
}

__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, double* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

// z = a*x + b*y
__global__ void lincomb_kernel(double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                               double* __restrict__ z, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = a * x[i] + b * y[i];
}

// u0 = (dT0, dT0[wall elements], dT0[periodic source elements] for every MFP)
__global__ void init_state_kernel(const double* __restrict__ dT0, int64_t n, const int32_t* __restrict__ wall_cell,
                                  int64_t nd, const int32_t* __restrict__ x_cell, int64_t nsrc, int n_mfp,
                                  double* __restrict__ u) {
  const int64_t total = n + nd + nsrc * n_mfp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    double v;
    if (i < n) v = dT0[i];
    else if (i < n + nd) v = dT0[wall_cell[i - n]];
    else v = dT0[x_cell[(i - n - nd) / n_mfp]];
    u[i] = v;
  }
}

// outputs: dT = Fu_T + c; J = Jraw - dT_in * sig_sum; K = Kraw + kconst + c*kshift; S = Sraw + c*sshift
__global__ void finalize_kernel(const double* __restrict__ Fu, const double* __restrict__ u, int64_t n, double c,
                                const double* __restrict__ Jraw, int ds, double s0, double s1, double s2,
                                const double* __restrict__ Kraw, const double* __restrict__ Sraw,
                                const double* __restrict__ kconst, const double* __restrict__ kshift,
                                const double* __restrict__ sshift, int64_t nks, double* __restrict__ dT,
                                double* __restrict__ J, double* __restrict__ K, double* __restrict__ S) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (dT) dT[i] = Fu[i] + c;
    if (J) {
      const double ss[3] = {s0, s1, s2};
      for (int d = 0; d < ds; ++d) J[i * ds + d] = Jraw[i * ds + d] - u[i] * ss[d];
    }
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nks; i += stride) {
    if (K) K[i] = Kraw[i] + kconst[i] + c * kshift[i];
    if (S) S[i] = Sraw[i] + c * sshift[i];
  }
}

using Work = SolveWork;

struct Solver {
  obte_plan plan;
  Work& wk;
  int sweeps = 0, sweeps64 = 0, sweeps_df = 0;
  int max_sweeps;
  cudaStream_t st;

  Solver(obte_plan p, Work& w, int ms) : plan(p), wk(w), max_sweeps(ms), st(p->stream) {
    trace = std::getenv("OBTE_TRACE") != nullptr;
    if (trace)
      for (auto& e : ev) cudaEventCreate(&e);
  }
  ~Solver() {
    if (trace) {
      std::fprintf(stderr, "[obte trace] iterations %d: sweep %.1f ms, orthogonalisation %.1f ms (GPU), wall %.1f ms\n",
                   t_iters, t_sweep, t_gs, t_wall);
      for (auto& e : ev) cudaEventDestroy(e);
    }
  }
  // optional per-iteration timing (OBTE_TRACE): GPU time of the sweep and of the Gram-Schmidt work
  bool trace = false;
  cudaEvent_t ev[3] = {};
  float t_sweep = 0, t_gs = 0;
  double t_wall = 0;
  int t_iters = 0;

  // right preconditioner (periodic-inflow blocks and / or diffusion-synthetic acceleration), or off
  bool xp = false;
  bool xblocks = false;     // periodic-inflow blocks
  bool dsa = false;         // diffusion-synthetic acceleration
  // the next gmres call starts from x = 0 (its initial residual is the right-hand side: no sweep)
  bool x_zero = false;
  // a final pass that recomputes the true residual follows every gmres call: end a cycle whose Arnoldi
  // estimate met the tolerance without the confirming sweep
  bool estimate_exit = false;
  // out += (M^-1 - I) in: W in on the slow inflow blocks, E L^-1 R in of the diffusion correction
  void prec_add(const double* in, double* out, bool fp32) {
    if (xblocks) xprec_add(plan, in, out, fp32);
    if (dsa) dsa_add(plan, in, out);
  }
  // out = M^-1 in
  obte_status prec(const double* in, double* out, bool fp32) {
    OBTE_CUDA(cudaMemcpyAsync(out, in, (size_t)wk.nu * sizeof(double), cudaMemcpyDeviceToDevice, st));
    prec_add(in, out, fp32);
    OBTE_CUDA(cudaGetLastError());
    return OBTE_OK;
  }

  obte_status sweep(bool fp32, const double* in, double* out, bool src, bool fin = false) {
    ++sweeps;
    if (!fp32) ++sweeps64;
    return launch_sweep(plan, fp32, in, out, src, fin, wk.Jraw.as<double>(), wk.Kraw.as<double>(),
                        wk.Sraw.as<double>());
  }
  // the output pass in double-float arithmetic (with source, J, K, S accumulated)
  obte_status sweep_df(const double* in, double* out) {
    ++sweeps;
    ++sweeps_df;
    return launch_sweep_df(plan, in, out, true, wk.Jraw.as<double>(), wk.Kraw.as<double>(), wk.Sraw.as<double>());
  }
  // h[0..k) = V[0..k)^T w (and h[k] = w.w when self), copied to host
  obte_status multidot(const double* V, int k, const double* w, std::vector<double>& h, bool self = false) {
    const int64_t n = wk.nu;
    const int kk = k + (self ? 1 : 0);
    multidot_kernel<<<wk.nb, VT, 0, st>>>(V, n, k, self ? 1 : 0, w, n, wk.partial.as<double>(), nullptr);
    reduce_partials_kernel<<<kk, VT, 0, st>>>(wk.partial.as<double>(), wk.nb, kk, wk.hdev.as<double>());
    count_launch(2);
    OBTE_CUDA(cudaGetLastError());
    h.resize(kk);
    OBTE_CUDA(cudaMemcpyAsync(h.data(), wk.hdev.p, kk * sizeof(double), cudaMemcpyDeviceToHost, st));
    OBTE_CUDA(wait_stream(st));
    return OBTE_OK;
  }
  obte_status norm(const double* x, double& out) {
    std::vector<double> h;
    OBTE_TRY(multidot(x, 1, x, h));
    out = std::sqrt(std::max(h[0], 0.0));
    return OBTE_OK;
  }
  obte_status lincomb(double a, const double* x, double b, const double* y, double* z) {
    lincomb_kernel<<<wk.nb, VT, 0, st>>>(a, x, b, y, z, wk.nu);
    count_launch();
    OBTE_CUDA(cudaGetLastError());
    return OBTE_OK;
  }
  obte_status axpby(double a, const double* x, double b, double* y) {
    axpby_kernel<<<wk.nb, VT, 0, st>>>(a, x, b, y, wk.nu);
    count_launch();
    OBTE_CUDA(cudaGetLastError());
    return OBTE_OK;
  }

  // residual of the correction equation (I-K) x = rhs:   r = rhs - x + K x   (rhs == nullptr: r = F(x) - x)
  obte_status residual(bool fp32, const double* rhs, const double* x, double* r) {
    if (rhs) {
      OBTE_TRY(sweep(fp32, x, wk.tmp.as<double>(), false));
      OBTE_TRY(lincomb(1.0, rhs, -1.0, x, r));
      OBTE_TRY(axpby(1.0, wk.tmp.as<double>(), 1.0, r));
    } else {
      OBTE_TRY(sweep(fp32, x, wk.tmp.as<double>(), true));
      OBTE_TRY(lincomb(1.0, wk.tmp.as<double>(), -1.0, x, r));
    }
    return OBTE_OK;
  }

  // Device Arnoldi scratch: second-pass coefficients [m+1], Hessenberg column [m+3], norms [2], DGKS flag,
  // 1/‖w‖ in FP32 and FP64; and the pinned host copy of the column.
  struct GsScratch {
    double *h2, *col, *s, *inv64;
    int* skip;
    float* inv;
  };
  obte_status gs_scratch(GsScratch& g) {
    const int m = wk.restart;
    if (!wk.gs.p) OBTE_TRY(wk.gs.alloc((size_t)(2 * m + 9) * sizeof(double)));
    if (!wk.hcol.p) OBTE_TRY(wk.hcol.alloc((size_t)(m + 3) * sizeof(double)));
    g.h2 = wk.gs.as<double>();
    g.col = g.h2 + (m + 1);
    g.s = g.col + (m + 3);
    g.skip = reinterpret_cast<int*>(g.s + 2);
    g.inv = reinterpret_cast<float*>(g.s + 3);
    g.inv64 = g.s + 4;
    return OBTE_OK;
  }

  // Restarted GMRES with the FP32 basis (see multidot32v_kernel); same contract as gmres().
  obte_status gmres32(const double* rhs, double* x, double tol_rel, double tol_abs, double& res_out, bool& ok) {
    const int64_t n = wk.nu;
    const int m = wk.restart;
    const int64_t ld = (n + 3) & ~(int64_t)3;   // basis rows padded to 16 bytes
    if (!wk.V32.p) {
      OBTE_TRY(wk.V32.alloc((size_t)ld * (m + 1) * sizeof(float)));
      OBTE_TRY(wk.w32.alloc((size_t)ld * sizeof(float)));
    }
    float* V = wk.V32.as<float>();
    float* w = wk.w32.as<float>();
    double* vj64 = wk.w.as<double>();
    double* r = wk.r.as<double>();
    const int nb = wk.nb;
    // Gram-Schmidt kernels: about 4 float4 per thread and tile, at most the elementwise grid
    const int nbg = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (n / 4 + 4 * VT - 1) / (4 * VT)));
    GsScratch gsd;
    OBTE_TRY(gs_scratch(gsd));
    double* h2d = gsd.h2;
    double* cold = gsd.col;
    double* sd = gsd.s;
    int* skipd = gsd.skip;
    float* invd = gsd.inv;
    const double* hc = wk.hcol.as<double>();
    double* hdev = wk.hdev.as<double>();
    double* part = wk.partial.as<double>();
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    ok = false;
    if (x_zero && rhs) OBTE_TRY(lincomb(1.0, rhs, 0.0, rhs, r));
    else OBTE_TRY(residual(true, rhs, x, r));
    x_zero = false;
    double beta;
    OBTE_TRY(norm(r, beta));
    res_out = beta;
    while (true) {
      double xn;
      OBTE_TRY(norm(x, xn));
      const double tol = std::max(tol_abs, tol_rel * std::max(xn, beta));
      if (beta <= tol) { ok = true; return OBTE_OK; }
      if (sweeps >= max_sweeps) return OBTE_OK;
      scale_to_f32_kernel<<<nb, VT, 0, st>>>(1.0 / beta, r, V, n);
      count_launch();
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      double est = beta;
      for (; j < m && sweeps < max_sweeps; ++j) {
        const auto w0 = std::chrono::steady_clock::now();
        if (trace) cudaEventRecord(ev[0], st);
        widen_kernel<<<nb, VT, 0, st>>>(V + (int64_t)j * ld, vj64, n);
        count_launch();
        const double* zj = vj64;              // z_j = M^-1 v_j
        if (xp) {
          OBTE_TRY(prec(vj64, wk.pz.as<double>(), true));
          zj = wk.pz.as<double>();
        }
        OBTE_TRY(sweep(true, zj, wk.tmp.as<double>(), false));
        if (trace) cudaEventRecord(ev[1], st);
        diff_to_f32_kernel<<<nb, VT, 0, st>>>(zj, wk.tmp.as<double>(), w, n);
        count_launch();
        OBTE_CUDA(cudaGetLastError());
        // classical Gram-Schmidt with one conditional re-orthogonalisation (as in gmres()), all on the
        // device: the second pass's kernels return at once when the DGKS test declines it, and the
        // host reads the finished Hessenberg column once per step
        const int k = j + 1;
        multidot32v_kernel<<<nbg, VT, 0, st>>>(V, ld, k, 1, w, n, part, nullptr);
        reduce_partials_kernel<<<k + 1, VT, 0, st>>>(part, nbg, k + 1, hdev);
        update32v_kernel<<<nbg, VT, 0, st>>>(w, V, ld, k, hdev, n, part, nullptr);
        reduce_partials_kernel<<<1, VT, 0, st>>>(part, nbg, 1, sd);
        gs_check_kernel<<<1, 32, 0, st>>>(hdev, k, sd, skipd);
        multidot32v_kernel<<<nbg, VT, 0, st>>>(V, ld, k, 0, w, n, part, skipd);
        reduce_partials_kernel<<<k, VT, 0, st>>>(part, nbg, k, h2d);
        update32v_kernel<<<nbg, VT, 0, st>>>(w, V, ld, k, h2d, n, part, skipd);
        reduce_partials_kernel<<<1, VT, 0, st>>>(part, nbg, 1, sd + 1);
        gs_finish_kernel<<<1, 128, 0, st>>>(hdev, h2d, k, sd, skipd, cold, invd, gsd.inv64);
        scale32d_kernel<<<nb, VT, 0, st>>>(invd, w, V + (int64_t)k * ld, n);
        count_launch(11);
        OBTE_CUDA(cudaGetLastError());
        OBTE_CUDA(cudaMemcpyAsync(wk.hcol.p, cold, (size_t)(k + 2) * sizeof(double), cudaMemcpyDeviceToHost, st));
        OBTE_CUDA(wait_stream(st));
        const double hn = hc[k];
        for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hc[i];
        H[(size_t)(j + 1) * m + j] = hn;
        for (int i = 0; i < j; ++i) {
          const double a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
          H[(size_t)i * m + j] = cs[i] * a + sn[i] * b;
          H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
        }
        const double a = H[(size_t)j * m + j], b = H[(size_t)(j + 1) * m + j];
        const double rr = std::hypot(a, b);
        cs[j] = rr > 0 ? a / rr : 1.0;
        sn[j] = rr > 0 ? b / rr : 0.0;
        H[(size_t)j * m + j] = rr;
        H[(size_t)(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        est = std::fabs(g[j + 1]);
        if (trace) {
          cudaEventRecord(ev[2], st);
          cudaEventSynchronize(ev[2]);
          float ta = 0, tb = 0;
          cudaEventElapsedTime(&ta, ev[0], ev[1]);
          cudaEventElapsedTime(&tb, ev[1], ev[2]);
          t_sweep += ta;
          t_gs += tb;
          t_wall += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
          ++t_iters;
        }
        if (est <= tol || hn == 0) { ++j; break; }
      }
      std::vector<double> y(j, 0.0);
      for (int i = j - 1; i >= 0; --i) {
        double acc = g[i];
        for (int k = i + 1; k < j; ++k) acc -= H[(size_t)i * m + k] * y[k];
        y[i] = H[(size_t)i * m + i] != 0 ? acc / H[(size_t)i * m + i] : 0.0;
      }
      if (j > 0) {
        OBTE_CUDA(cudaMemcpyAsync(wk.hdev.p, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, st));
        if (xp) {                             // x += M^-1 (V y)
          double* z = wk.pz.as<double>();
          OBTE_CUDA(cudaMemsetAsync(z, 0, (size_t)n * sizeof(double), st));
          xupdate32_kernel<<<nb, VT, 0, st>>>(z, V, ld, j, wk.hdev.as<double>(), n);
          count_launch();
          OBTE_TRY(axpby(1.0, z, 1.0, x));
          prec_add(z, x, true);
        } else {
          xupdate32_kernel<<<nb, VT, 0, st>>>(x, V, ld, j, wk.hdev.as<double>(), n);
          count_launch();
        }
        OBTE_CUDA(cudaGetLastError());
      }
      if (estimate_exit && est <= tol) { res_out = est; ok = true; return OBTE_OK; }
      const double beta_prev = beta;
      OBTE_TRY(residual(true, rhs, x, r));
      OBTE_TRY(norm(r, beta));
      res_out = beta;
      if (beta <= tol) { ok = true; return OBTE_OK; }
      if (sweeps >= max_sweeps) return OBTE_OK;
      // a whole cycle that no longer reduces the true residual near the FP32 sweeps' rounding floor
      // (~5e-7 of ‖x‖): stop instead of spinning to the sweep cap
      if (beta > 0.9 * beta_prev && beta < 1e-5 * xn) return OBTE_OK;
    }
  }

  // Restarted GMRES on (I - K) x = rhs, FP64 vectors, sweeps in the given precision.
  // Stops when the residual norm <= max(tol_abs, tol_rel * scale) with scale = max(‖x‖, ‖r‖)
  // taken at each (re)start, or when the sweep cap is hit.
  obte_status gmres(bool fp32, const double* rhs, double* x, double tol_rel, double tol_abs, double& res_out,
                    bool& ok) {
    // stages with FP32 sweeps and a tolerance no tighter than 1e-6 run on the FP32 basis
    if (fp32 && !std::getenv("OBTE_FP64_BASIS") && (tol_rel >= 1e-6 || (tol_rel == 0 && tol_abs > 0)))
      return gmres32(rhs, x, tol_rel, tol_abs, res_out, ok);
    const int64_t n = wk.nu;
    const int m = wk.restart;
    // the FP64 basis is allocated on first use: FP32-refine solves at the usual tolerances never need it
    if (!wk.V.p) OBTE_TRY(wk.V.alloc((size_t)n * sizeof(double) * (m + 1)));
    double* V = wk.V.as<double>();
    double* w = wk.w.as<double>();
    double* r = wk.r.as<double>();
    GsScratch gsd;
    OBTE_TRY(gs_scratch(gsd));
    const double* hc = wk.hcol.as<double>();
    double* hdev = wk.hdev.as<double>();
    double* part = wk.partial.as<double>();
    const int nb = wk.nb;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    ok = false;
    if (x_zero && rhs) OBTE_TRY(lincomb(1.0, rhs, 0.0, rhs, r));
    else OBTE_TRY(residual(fp32, rhs, x, r));
    x_zero = false;
    double beta;
    OBTE_TRY(norm(r, beta));
    res_out = beta;
    while (true) {
      double xn;
      OBTE_TRY(norm(x, xn));
      const double tol = std::max(tol_abs, tol_rel * std::max(xn, beta));
      if (beta <= tol) { ok = true; return OBTE_OK; }
      if (sweeps >= max_sweeps) return OBTE_OK;
      OBTE_TRY(lincomb(1.0 / beta, r, 0.0, r, V));
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      double est = beta;
      for (; j < m && sweeps < max_sweeps; ++j) {
        double* vj = V + (int64_t)j * n;
        const auto w0 = std::chrono::steady_clock::now();
        if (trace) cudaEventRecord(ev[0], st);
        const double* zj = vj;                // z_j = M^-1 v_j
        if (xp) {
          OBTE_TRY(prec(vj, wk.pz.as<double>(), false));
          zj = wk.pz.as<double>();
        }
        OBTE_TRY(sweep(fp32, zj, wk.tmp.as<double>(), false));
        if (trace) cudaEventRecord(ev[1], st);
        OBTE_TRY(lincomb(1.0, zj, -1.0, wk.tmp.as<double>(), w));
        // classical Gram-Schmidt; a second pass only when the first one cancelled most of w
        // (Daniel-Gragg-Kaufman-Stewart criterion, ‖w‖ after < 0.7 ‖w‖ before).  The whole step runs on
        // the device (the second pass's kernels return at once when the test declines it) and the host
        // reads the Hessenberg column once.
        const int k = j + 1;
        multidot_kernel<<<nb, VT, 0, st>>>(V, n, k, 1, w, n, part, nullptr);   // h[0..j] and w.w in one pass
        reduce_partials_kernel<<<k + 1, VT, 0, st>>>(part, nb, k + 1, hdev);
        update_kernel<<<nb, VT, 0, st>>>(w, V, n, k, hdev, n, part, nullptr);
        reduce_partials_kernel<<<1, VT, 0, st>>>(part, nb, 1, gsd.s);
        gs_check_kernel<<<1, 32, 0, st>>>(hdev, k, gsd.s, gsd.skip);
        multidot_kernel<<<nb, VT, 0, st>>>(V, n, k, 0, w, n, part, gsd.skip);
        reduce_partials_kernel<<<k, VT, 0, st>>>(part, nb, k, gsd.h2);
        update_kernel<<<nb, VT, 0, st>>>(w, V, n, k, gsd.h2, n, part, gsd.skip);
        reduce_partials_kernel<<<1, VT, 0, st>>>(part, nb, 1, gsd.s + 1);
        gs_finish_kernel<<<1, 128, 0, st>>>(hdev, gsd.h2, k, gsd.s, gsd.skip, gsd.col, gsd.inv, gsd.inv64);
        scaled_kernel<<<nb, VT, 0, st>>>(gsd.inv64, w, V + (int64_t)k * n, n);
        count_launch(11);
        OBTE_CUDA(cudaGetLastError());
        OBTE_CUDA(cudaMemcpyAsync(wk.hcol.p, gsd.col, (size_t)(k + 2) * sizeof(double), cudaMemcpyDeviceToHost, st));
        OBTE_CUDA(wait_stream(st));
        const double hn = hc[k];
        // Hessenberg column j
        for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hc[i];
        H[(size_t)(j + 1) * m + j] = hn;
        for (int i = 0; i < j; ++i) {
          const double a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
          H[(size_t)i * m + j] = cs[i] * a + sn[i] * b;
          H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
        }
        const double a = H[(size_t)j * m + j], b = H[(size_t)(j + 1) * m + j];
        const double rr = std::hypot(a, b);
        cs[j] = rr > 0 ? a / rr : 1.0;
        sn[j] = rr > 0 ? b / rr : 0.0;
        H[(size_t)j * m + j] = rr;
        H[(size_t)(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        est = std::fabs(g[j + 1]);
        if (trace) {
          cudaEventRecord(ev[2], st);
          cudaEventSynchronize(ev[2]);
          float a = 0, b = 0;
          cudaEventElapsedTime(&a, ev[0], ev[1]);
          cudaEventElapsedTime(&b, ev[1], ev[2]);
          t_sweep += a;
          t_gs += b;
          t_wall += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
          ++t_iters;
        }
        if (est <= tol || hn == 0) { ++j; break; }
      }
      // y = H^-1 g (upper triangular j x j), x += V y
      std::vector<double> y(j, 0.0);
      for (int i = j - 1; i >= 0; --i) {
        double acc = g[i];
        for (int k = i + 1; k < j; ++k) acc -= H[(size_t)i * m + k] * y[k];
        y[i] = H[(size_t)i * m + i] != 0 ? acc / H[(size_t)i * m + i] : 0.0;
      }
      for (double& v : y) v = -v;   // update_kernel subtracts
      if (j > 0) {
        OBTE_CUDA(cudaMemcpyAsync(wk.hdev.p, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, st));
        if (xp) {                             // x += M^-1 (V y)
          double* z = wk.pz.as<double>();
          OBTE_CUDA(cudaMemsetAsync(z, 0, (size_t)n * sizeof(double), st));
          update_kernel<<<wk.nb, VT, 0, st>>>(z, V, n, j, wk.hdev.as<double>(), n, nullptr, nullptr);
          count_launch();
          OBTE_TRY(axpby(1.0, z, 1.0, x));
          prec_add(z, x, false);
        } else {
          update_kernel<<<wk.nb, VT, 0, st>>>(x, V, n, j, wk.hdev.as<double>(), n, nullptr, nullptr);
          count_launch();
        }
        OBTE_CUDA(cudaGetLastError());
      }
      if (estimate_exit && est <= tol) { res_out = est; ok = true; return OBTE_OK; }
      // true residual for the restart
      const double beta_prev = beta;
      OBTE_TRY(residual(fp32, rhs, x, r));
      OBTE_TRY(norm(r, beta));
      res_out = beta;
      if (beta <= tol) { ok = true; return OBTE_OK; }
      if (sweeps >= max_sweeps) return OBTE_OK;
      // FP32 sweeps: a cycle that no longer reduces the true residual near their rounding floor
      if (fp32 && beta > 0.9 * beta_prev && beta < 1e-5 * xn) return OBTE_OK;
    }
  }
};

}  // namespace

static obte_status alloc_work(obte_plan plan, Work& wk, int restart) {
  PhaseTimer timer("alloc_work");
  const Schedule& s = plan->sched;
  wk.nu = plan->nu;
  wk.restart = restart;
  wk.nb = vec_blocks(plan, wk.nu);
  const size_t vb = (size_t)wk.nu * sizeof(double);
  OBTE_TRY(wk.u.alloc(vb));
  OBTE_TRY(wk.Fu.alloc(vb));
  OBTE_TRY(wk.r.alloc(vb));
  OBTE_TRY(wk.w.alloc(vb));
  OBTE_TRY(wk.tmp.alloc(vb));
  OBTE_TRY(wk.delta.alloc(vb));
  OBTE_TRY(wk.partial.alloc((size_t)wk.nb * (restart + 1) * sizeof(double)));
  OBTE_TRY(wk.hdev.alloc((size_t)(restart + 2) * sizeof(double)));
  OBTE_TRY(wk.sdev.alloc(8 * sizeof(double)));
  OBTE_TRY(wk.Jraw.alloc((size_t)s.n * s.ds * sizeof(double)));
  OBTE_TRY(wk.Kraw.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
  OBTE_TRY(wk.Sraw.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
  return OBTE_OK;
}

int64_t solve_scratch_bytes(obte_plan plan, int restart) {
  const Schedule& s = plan->sched;
  const int64_t vb = plan->nu * (int64_t)sizeof(double);
  // u Fu r w tmp delta pz rc, the FP64 and FP32 bases, two sets of J/K/S accumulators, partials, Arnoldi scratch
  return vb * (8 + restart + 1) + ((plan->nu + 3) & ~3LL) * 4LL * (restart + 2) + 2 * ((int64_t)s.n * s.ds * 8 + 2LL * s.n_mfp * s.n_dir * 8) +
         (int64_t)plan->ctx->num_sms * 4 * (restart + 1) * 8 + (2LL * restart + 9) * 8;
}

}  // namespace obte

using namespace obte;

extern "C" obte_status obte_bte_sweep(obte_plan plan, int32_t precision, const double* u_in, double* u_out,
                                      int32_t with_source) {
  if (!plan || !u_in || !u_out) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (!plan->ctx) { set_error("host-only plan cannot sweep"); return OBTE_ERR_BAD_ARG; }
  if (precision != OBTE_FP64 && precision != OBTE_FP32 && precision != OBTE_FP32_REFINE &&
      precision != OBTE_DOUBLE_FLOAT) {
    set_error("bad precision"); return OBTE_ERR_BAD_ARG;
  }
  if (precision == OBTE_DOUBLE_FLOAT) {
    // the double-float kernel is an output pass: its J, K, S accumulations go to discarded plan scratch
    OBTE_TRY(ensure_fields_scratch(plan));
    OBTE_TRY(launch_sweep_df(plan, u_in, u_out, with_source != 0, plan->fields_J.as<double>(),
                             plan->fields_K.as<double>(), plan->fields_S.as<double>()));
  } else {
    // scratch for the final-pass outputs is not needed for a plain sweep
    OBTE_TRY(launch_sweep(plan, precision != OBTE_FP64, u_in, u_out, with_source != 0, false, nullptr, nullptr,
                          nullptr));
  }
  OBTE_CUDA(wait_stream(plan->stream));
  return check_device_error(plan);
}

extern "C" obte_status obte_bte_plan_prepare(obte_plan plan, int32_t precision, int32_t restart) {
  if (!plan) { set_error("null plan"); return OBTE_ERR_BAD_ARG; }
  if (!plan->ctx) { set_error("host-only plan cannot be prepared"); return OBTE_ERR_BAD_ARG; }
  if (precision != OBTE_FP64 && precision != OBTE_FP32 && precision != OBTE_FP32_REFINE) {
    set_error("bad precision"); return OBTE_ERR_BAD_ARG;
  }
  const Schedule& s = plan->sched;
  restart = restart > 0 ? std::min(restart, 200) : 30;
  // tables of the sweep precisions the solve will use (FP32_REFINE: FP32 sweeps and one FP64 pass)
  if (precision != OBTE_FP64) OBTE_TRY(ensure_tables(plan, true));
  if (precision != OBTE_FP32) OBTE_TRY(ensure_tables(plan, false));
  if (!plan->work || plan->work->restart != restart || plan->work->nu != plan->nu) {
    plan->work.reset(new Work());
    plan->has_solution = false;
    obte_status ast = alloc_work(plan, *plan->work, restart);
    if (ast != OBTE_OK) { plan->work.reset(); return ast; }
  }
  Work& wk = *plan->work;
  if (precision != OBTE_FP64 && !wk.V32.p) {
    const int64_t ld = (wk.nu + 3) & ~(int64_t)3;
    OBTE_TRY(wk.V32.alloc((size_t)ld * (restart + 1) * sizeof(float)));
    OBTE_TRY(wk.w32.alloc((size_t)ld * sizeof(float)));
  }
  if (precision == OBTE_FP32_REFINE && !wk.rc.p) {
    OBTE_TRY(wk.rc.alloc((size_t)wk.nu * sizeof(double)));
    OBTE_TRY(wk.Jraw2.alloc((size_t)s.n * s.ds * sizeof(double)));
    OBTE_TRY(wk.Kraw2.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
    OBTE_TRY(wk.Sraw2.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
  }
  OBTE_CUDA(wait_stream(plan->stream));
  return OBTE_OK;
}

extern "C" obte_status obte_bte_solve(obte_plan plan, const obte_solve_opts* opts, const double* dT0, double* dT,
                                      double* J, double* K, double* S, obte_solve_info* info) {
  if (!plan || !opts || !dT0) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (!plan->ctx) { set_error("host-only plan cannot solve"); return OBTE_ERR_BAD_ARG; }
  const Schedule& s = plan->sched;
  const int prec = opts->precision;
  if (prec != OBTE_FP64 && prec != OBTE_FP32 && prec != OBTE_FP32_REFINE) {
    set_error("bad precision"); return OBTE_ERR_BAD_ARG;
  }
  const int restart = opts->restart > 0 ? std::min(opts->restart, 200) : 30;
  const int max_sweeps = opts->max_sweeps > 0 ? opts->max_sweeps : 1000;
  const double rtol = opts->rtol > 0 ? opts->rtol : 1e-10;
  cudaStream_t st = plan->stream;
  if (!plan->work || plan->work->restart != restart || plan->work->nu != plan->nu) {
    plan->work.reset(new Work());
    plan->has_solution = false;
    obte_status ast = alloc_work(plan, *plan->work, restart);
    if (ast != OBTE_OK) { plan->work.reset(); return ast; }
  }
  Work& wk = *plan->work;
  const bool warm = opts->warm_start && plan->has_solution;
  // the preconditioner's setup sweeps use the work vectors, so it runs before the state is set up
  // (a warm start keeps its previous state in wk.u, which the setup does not touch)
  int pmode = (opts->precond >= -1 && opts->precond <= 1) ? opts->precond : 0;
  if (const char* e = std::getenv("OBTE_XPREC")) pmode = std::atoi(e) == 0 ? -1 : 1;
  const bool build_xp = pmode == 1 || (pmode == 0 && plan->n_solves >= 1);
  ++plan->n_solves;
  if (build_xp) {
    // a preconditioner that does not fit in device memory is left out: the solve runs without it
    const obte_status xs = ensure_xprec(plan, wk);
    if (xs == OBTE_ERR_OOM) {
      plan->xprec->nblk = 0;
      plan->xprec->W.release();
      plan->sweep_cta_map = nullptr;
      plan->sweep_n_cta = 0;
      plan->sweep_batch = 1;
      plan->sweep_batch_stride = 0;
    } else {
      OBTE_TRY(xs);
    }
  }
  const bool use_xp = pmode >= 0 && plan->xprec && plan->xprec->nblk > 0;
  // diffusion-synthetic acceleration: opts->dsa 1 on, -1 off, 0 (other values) the problem's default;
  // OBTE_DSA=0 / 1 overrides
  int dmode = (opts->dsa >= -1 && opts->dsa <= 1) ? opts->dsa : 0;
  if (const char* e = std::getenv("OBTE_DSA")) dmode = std::atoi(e) == 0 ? -1 : 1;
  const bool use_dsa = dmode == 1 || (dmode == 0 && dsa_default(s));
  dsa_join(plan);                 // a set-up started by new transmissions
  if (use_dsa) OBTE_TRY(ensure_dsa(plan));
  if ((use_xp || use_dsa) && !wk.pz.p) OBTE_TRY(wk.pz.alloc((size_t)wk.nu * sizeof(double)));
  plan->has_solution = false;
  Solver sv(plan, wk, max_sweeps);
  sv.xp = use_xp || use_dsa;
  sv.xblocks = use_xp;
  sv.dsa = use_dsa;
  sv.estimate_exit = true;   // every GMRES call below is followed by a final pass
  double* u = wk.u.as<double>();
  const int64_t nsrc = s.x_base[s.n_dir];
  // the state implied by dT0 fixes the conserved temperature level; a warm start keeps the
  // previous converged state as the iterate
  double* u0 = warm ? wk.tmp.as<double>() : u;
  init_state_kernel<<<wk.nb, VT, 0, st>>>(dT0, s.n, plan->diffuse_cell.as<int32_t>(), s.nd,
                                          plan->x_cell.as<int32_t>(), nsrc, s.n_mfp, u0);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  // conserved ell.u of the initial state (DeltaT and T_B parts)
  std::vector<double> h;
  OBTE_TRY(sv.multidot(u0, 1, plan->ell.as<double>(), h));
  const double ell0 = h[0];

  double unorm;
  OBTE_TRY(sv.norm(u, unorm));
  double res = 0;
  bool ok = false;
  // Krylov solve in the sweep precision (FP32 for both reduced modes).  FP32 sweeps carry a
  // relative rounding floor of a few 1e-7, so the FP32 stage stops at the inner tolerance (refine)
  // or no tighter than 5e-7 (plain FP32), and a restart cycle that stalls near the floor ends it.
  const double inner_tol = opts->inner_rtol > 0 ? opts->inner_rtol : 1e-5;
  const double tol1 = prec == OBTE_FP64 ? rtol : prec == OBTE_FP32_REFINE ? std::max(rtol, inner_tol)
                                                                         : std::max(rtol, 5e-7);
  OBTE_TRY(sv.gmres(prec != OBTE_FP64, nullptr, u, tol1, 0.0, res, ok));
  // Final pass at u: F(u) with J, K, S.  In FP32_REFINE it runs in FP64 and doubles as the
  // convergence check of the iterative refinement: while ‖F(u) - u‖ > rtol ‖u‖, solve the
  // correction (I - K) d = F(u) - u with FP32 sweeps and repeat.
  //
  // F is affine and the outputs (F(u), J, K, S) are affine in u, so after a correction d the pass at
  // u + d is the pass at u plus the source-free pass at d.  d is small (the correction of a residual
  // near the FP32 stage tolerance), so the source-free pass runs in FP32: its rounding is ~1e-7 of
  // ‖K d‖, i.e. ~1e-12 of ‖u‖, far below any tolerance this mode accepts.  This replaces the second
  // FP64 pass (FP64 sweeps run on GB300's narrow FP64 pipe, ~10x the time of an FP32 sweep).  The
  // per-ordinate temperatures a gradient solve keeps are affine in u as well: the pass at d adds its
  // own to them.  A correction that is not small (‖d‖ > 1e-3 ‖u‖) gets a full FP64 pass instead.
  constexpr double kPass32Rtol = 5e-6;
  const bool fin32 = prec == OBTE_FP32;
  double* Fu = wk.Fu.as<double>();
  double* r = wk.r.as<double>();
  double* d = wk.delta.as<double>();
  const int steps = prec == OBTE_FP32_REFINE ? std::max(1, opts->refine_steps) : 0;
  const double inner = inner_tol;
  const bool split = prec == OBTE_FP32_REFINE;
  if (split && !wk.rc.p) {
    OBTE_TRY(wk.rc.alloc((size_t)wk.nu * sizeof(double)));
    OBTE_TRY(wk.Jraw2.alloc((size_t)s.n * s.ds * sizeof(double)));
    OBTE_TRY(wk.Kraw2.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
    OBTE_TRY(wk.Sraw2.alloc((size_t)s.n_mfp * s.n_dir * sizeof(double)));
  }
  const int64_t nks = (int64_t)s.n_mfp * s.n_dir;
  bool full_pass = true;
  // With OBTE_REFINE_DF=1, FP32_REFINE runs its full output passes in double-float arithmetic on the FP32 pipe
  // (~44 significant bits: rounding about 1e-13 of the state, below the tolerances down to 1e-11 it
  // certifies; a tighter tolerance and gradient solves keep the FP64 pass).  It is off by default: on GB300
  // the double-float sweep measured slower than the FP64 one (60k triangles x 9,600 ordinates: 23.7 against
  // 16.3 ms; 110k tetrahedra x 15,360: 153 against 62 ms): its chains of dependent FP32 operations cost the
  // latency-bound sweep more than the FP64 pipe does.
  const char* rdf = std::getenv("OBTE_REFINE_DF");
  const bool df_pass = prec == OBTE_FP32_REFINE && plan->xstore == nullptr && rtol >= 1e-11 &&
                       rdf && std::atoi(rdf) != 0;
  // A tolerance of at least kPass32Rtol (10x the FP32 sweep's rounding floor of a few 1e-7 of ‖u‖) is
  // certified by an FP32 output pass: the residual it measures is off by less than a tenth of the
  // tolerance, and J, K, S by ~1e-7 relative.  Such a solve (the served form at 1e-5) runs no FP64 sweep.
  // OBTE_REFINE_FP64_PASS=1 keeps the FP64 pass at every tolerance.
  const char* rfp = std::getenv("OBTE_REFINE_FP64_PASS");
  const bool pass32 = prec == OBTE_FP32_REFINE && plan->xstore == nullptr && rtol >= kPass32Rtol &&
                      !(rfp && std::atoi(rfp) != 0);
  for (int k = 0;; ++k) {
    if (full_pass) {
      if (df_pass && !pass32) OBTE_TRY(sv.sweep_df(u, Fu));
      else OBTE_TRY(sv.sweep(fin32 || pass32, u, Fu, true, true));
    }
    OBTE_TRY(sv.lincomb(1.0, Fu, -1.0, u, r));
    double rn;
    OBTE_TRY(sv.norm(r, rn));
    OBTE_TRY(sv.norm(u, unorm));
    res = rn / std::max(unorm, 1e-300);
    ok = res <= rtol * (prec == OBTE_FP32_REFINE ? 1.0 : 10.0);
    if (ok || k >= steps || sv.sweeps >= max_sweeps) break;
    // GMRES uses wk.r as its own residual workspace: hand it the FP64 residual in a copy
    double* rhs = split ? wk.rc.as<double>() : Fu;
    OBTE_TRY(sv.lincomb(1.0, r, 0.0, r, rhs));
    OBTE_CUDA(cudaMemsetAsync(d, 0, wk.nu * sizeof(double), st));
    sv.x_zero = true;
    bool iok;
    double ires;
    OBTE_TRY(sv.gmres(true, rhs, d, 0.0, std::max(inner * rn, rtol * unorm * 0.5), ires, iok));
    double dn = 0;
    if (split) OBTE_TRY(sv.norm(d, dn));
    OBTE_TRY(sv.axpby(1.0, d, 1.0, u));
    full_pass = !split || dn > 1e-3 * unorm;
    if (!full_pass) {
      // F(u + d) = F(u) + K d; outputs likewise (source-free FP32 final pass at d)
      plan->xstore_add = true;
      const obte_status ds = launch_sweep(plan, true, d, wk.tmp.as<double>(), false, true, wk.Jraw2.as<double>(),
                                          wk.Kraw2.as<double>(), wk.Sraw2.as<double>());
      plan->xstore_add = false;
      OBTE_TRY(ds);
      ++sv.sweeps;
      OBTE_TRY(sv.axpby(1.0, wk.tmp.as<double>(), 1.0, Fu));
      add_kernel<<<wk.nb, VT, 0, st>>>(wk.Jraw.as<double>(), wk.Jraw2.as<double>(), s.n * s.ds);
      add_kernel<<<wk.nb, VT, 0, st>>>(wk.Kraw.as<double>(), wk.Kraw2.as<double>(), nks);
      add_kernel<<<wk.nb, VT, 0, st>>>(wk.Sraw.as<double>(), wk.Sraw2.as<double>(), nks);
      count_launch(3);
      OBTE_CUDA(cudaGetLastError());
    }
  }
  // offset: ell.(Fu + c) = ell0 (none with isothermal walls, whose fixed point is unique)
  double c = 0;
  if (!s.isothermal) {
    OBTE_TRY(sv.multidot(Fu, 1, plan->ell.as<double>(), h));
    c = (ell0 - h[0]) / plan->ell_sum;
  }
  const double s0 = s.ds > 0 ? s.sig_sum[0] : 0, s1 = s.ds > 1 ? s.sig_sum[1] : 0, s2 = s.ds > 2 ? s.sig_sum[2] : 0;
  finalize_kernel<<<wk.nb, VT, 0, st>>>(Fu, u, s.n, c, wk.Jraw.as<double>(), s.ds, s0, s1, s2,
                                        wk.Kraw.as<double>(), wk.Sraw.as<double>(), plan->kconst.as<double>(),
                                        plan->kshift.as<double>(), plan->sshift.as<double>(),
                                        (int64_t)s.n_mfp * s.n_dir, dT, J, K, S);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  double kappa = 0;
  if (K) {
    std::vector<double> kh((size_t)s.n_mfp * s.n_dir);
    OBTE_CUDA(cudaMemcpyAsync(kh.data(), K, kh.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    OBTE_CUDA(wait_stream(st));
    for (double v : kh) kappa += v;
  }
  OBTE_CUDA(wait_stream(st));
  OBTE_TRY(check_device_error(plan));
  plan->has_solution = true;
  if (info) {
    info->kappa_eff = kappa;
    info->n_sweeps = sv.sweeps;
    info->n_sweeps_fp64 = sv.sweeps64;
    info->n_sweeps_df = sv.sweeps_df;
    info->residual = res;
    info->offset = c;
    info->converged = ok ? 1 : 0;
  }
  return ok ? OBTE_OK : OBTE_ERR_NOT_CONVERGED;
}
