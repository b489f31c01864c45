// Fourier first guess on the device (openbte/fourier.py:15-185).
//
// The reference assembles the orthogonal part of the finite-volume diffusion
// operator (fourier.py:51-63), factorises it with SuperLU and runs a
// deferred non-orthogonal correction (fourier.py:149-178):
//   T = F^-1 (B + C);  T -= (max T + min T)/2;  grad = LS gradient(T);
//   C = div(w grad_i + (1-w) grad_j) . v_nonorth;  stop when |‖C‖-‖C_old‖|/‖C‖ <= rtol.
// Here F = V^-1 L with L the symmetric volume-weighted Laplacian (plus Robin
// terms of mixed walls), so each T is a conjugate-gradient solve of
// L T = V (B + C) on the device.  Without mixed walls the reference replaces
// row N = 10 by the identity (fourier.py:115-118), i.e. T_N = (B + C)_N; that
// value is moved to the right-hand side and CG runs on the remaining SPD
// system.  The least-squares gradient (openbte/objects.py:322-405), the
// correction gather and the diffusive kappa (openbte/objects.py:139-172) are
// kernels; CG keeps alpha/beta on the device and the host only reads the
// residual every few iterations.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "internal.h"

namespace obte {
namespace {

constexpr int FT = 256;

__global__ void spmv_kernel(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y,
                            double* __restrict__ part) {
  __shared__ double red[FT / 32];
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    double s = 0;
    for (int k = rp[i]; k < rp[i + 1]; ++k) s += v[k] * x[ci[k]];
    y[i] = s;
    acc += s * x[i];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < FT / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// scalars: [0] rz  [1] pAp  [2] rz_new  [3] rr
__global__ void reduce_kernel(const double* __restrict__ part, int nb, double* __restrict__ dst) {
  __shared__ double red[FT / 32];
  double acc = 0;
  for (int b = threadIdx.x; b < nb; b += FT) acc += part[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < FT / 32; ++w) t += red[w];
    *dst = t;
  }
}

// x += a p; r -= a Ap; z = r * dinv; partials of r.z and r.r
__global__ void cg_update_kernel(int64_t n, const double* __restrict__ sc, double* __restrict__ x,
                                 double* __restrict__ r, double* __restrict__ z, const double* __restrict__ p,
                                 const double* __restrict__ Ap, const double* __restrict__ dinv,
                                 double* __restrict__ part_rz, double* __restrict__ part_rr) {
  __shared__ double red[2][FT / 32];
  const double pap = sc[1];
  const double a = pap != 0 ? sc[0] / pap : 0.0;
  double rz = 0, rr = 0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    x[i] += a * p[i];
    const double ri = r[i] - a * Ap[i];
    r[i] = ri;
    const double zi = ri * dinv[i];
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  for (int o = 16; o > 0; o >>= 1) {
    rz += __shfl_xor_sync(0xffffffffu, rz, o);
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = rz;
    red[1][threadIdx.x >> 5] = rr;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0;
    for (int w = 0; w < FT / 32; ++w) { t0 += red[0][w]; t1 += red[1][w]; }
    part_rz[blockIdx.x] = t0;
    part_rr[blockIdx.x] = t1;
  }
}

// p = z + (rz_new / rz) p ; rz = rz_new
__global__ void cg_direction_kernel(int64_t n, double* __restrict__ sc, double* __restrict__ p,
                                    const double* __restrict__ z) {
  const double rz = sc[0];
  const double b = rz != 0 ? sc[2] / rz : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) p[i] = z[i] + b * p[i];
}

__global__ void copy_scalar_kernel(double* __restrict__ sc, int dst, int src) { sc[dst] = sc[src]; }

// Sum of per-block partials in a fixed order; every block computes the same value, so a
// kernel can use a grid-wide reduction of the previous kernel without another launch.
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int nb) {
  __shared__ double red[FT / 32];
  __shared__ double total;
  double acc = 0;
  for (int b = threadIdx.x; b < nb; b += FT) acc += part[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < FT / 32; ++w) t += red[w];
    total = t;
  }
  __syncthreads();
  return total;
}

// one CG step after the SpMV: alpha = rz / sum(pAp partials); x += a p; r -= a Ap; z = r dinv;
// partials of r.z (next rz) and r.r.  rz is read from sc[cur].  z == nullptr: another preconditioner
// writes z and the r.z partials.
__global__ void cg_step_kernel(int64_t n, const double* __restrict__ part_pap, int nb, const double* __restrict__ sc,
                               int cur, double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
                               const double* __restrict__ p, const double* __restrict__ Ap,
                               const double* __restrict__ dinv, double* __restrict__ part_rz,
                               double* __restrict__ part_rr) {
  __shared__ double red[2][FT / 32];
  const double pap = sum_partials(part_pap, nb);
  const double a = pap != 0 ? sc[cur] / pap : 0.0;
  double rz = 0, rr = 0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    x[i] += a * p[i];
    const double ri = r[i] - a * Ap[i];
    r[i] = ri;
    const double zi = ri * dinv[i];
    if (z) z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  for (int o = 16; o > 0; o >>= 1) {
    rz += __shfl_xor_sync(0xffffffffu, rz, o);
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = rz;
    red[1][threadIdx.x >> 5] = rr;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0;
    for (int w = 0; w < FT / 32; ++w) { t0 += red[0][w]; t1 += red[1][w]; }
    if (z) part_rz[blockIdx.x] = t0;
    part_rr[blockIdx.x] = t1;
  }
}

// p = z + (rz_new / rz) p with rz_new = sum(rz partials); block 0 stores rz_new in sc[cur^1]
// and r.r in sc[3] (read by the host between batches)
__global__ void cg_dir_kernel(int64_t n, const double* __restrict__ part_rz, const double* __restrict__ part_rr,
                              int nb, double* __restrict__ sc, int cur, double* __restrict__ p,
                              const double* __restrict__ z) {
  const double rzn = sum_partials(part_rz, nb);
  const double rz = sc[cur];
  const double b = rz != 0 ? rzn / rz : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) p[i] = z[i] + b * p[i];
  if (blockIdx.x == 0) {
    const double rr = sum_partials(part_rr, nb);
    if (threadIdx.x == 0) {
      sc[cur ^ 1] = rzn;
      sc[3] = rr;
    }
  }
}

// partials of r.z (the preconditioned residual product); p = z as well when p is given
__global__ void rz_kernel(int64_t n, const double* __restrict__ r, const double* __restrict__ z, double* __restrict__ p,
                          double* __restrict__ part) {
  __shared__ double red[FT / 32];
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    const double zi = z[i];
    acc += r[i] * zi;
    if (p) p[i] = zi;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < FT / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// warm start consistent with the pin: T += (B + C)_N - T_N  (two launches: read, then shift)
__global__ void pin_delta_kernel(const double* __restrict__ T, const double* __restrict__ B,
                                 const double* __restrict__ C, int pin, double* __restrict__ out) {
  *out = B[pin] + C[pin] - T[pin];
}
__global__ void shift_by_kernel(int64_t n, double* __restrict__ T, const double* __restrict__ d) {
  const double v = *d;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) T[i] += v;
}

// r = rhs - Ap; z = r dinv; p = z; partials of r.z, r.r and rhs.rhs
__global__ void cg_init_kernel(int64_t n, const double* __restrict__ rhs, const double* __restrict__ Ap,
                               const double* __restrict__ dinv, double* __restrict__ r, double* __restrict__ z,
                               double* __restrict__ p, double* __restrict__ part_rz, double* __restrict__ part_rr,
                               double* __restrict__ part_bb) {
  __shared__ double red[3][FT / 32];
  double rz = 0, rr = 0, bb = 0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    const double ri = rhs[i] - Ap[i];
    const double zi = ri * dinv[i];
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
    bb += rhs[i] * rhs[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    rz += __shfl_xor_sync(0xffffffffu, rz, o);
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    bb += __shfl_xor_sync(0xffffffffu, bb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = rz;
    red[1][threadIdx.x >> 5] = rr;
    red[2][threadIdx.x >> 5] = bb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int w = 0; w < FT / 32; ++w) { t0 += red[0][w]; t1 += red[1][w]; t2 += red[2][w]; }
    part_rz[blockIdx.x] = t0;
    part_rr[blockIdx.x] = t1;
    part_bb[blockIdx.x] = t2;
  }
}

// rhs_i = V_i (B_i + C_i) - L_iN (B_N + C_N) for i != N; rhs_N = 0;  T_N fixed to (B+C)_N
__global__ void cg_rhs_kernel(int64_t n, const double* __restrict__ vol, const double* __restrict__ B,
                              const double* __restrict__ C, int pin, const double* __restrict__ colpin,
                              double* __restrict__ rhs) {
  const double tn = pin >= 0 ? B[pin] + C[pin] : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    double v = vol[i] * (B[i] + C[i]);
    if (pin >= 0) v = (i == pin) ? 0.0 : v - colpin[i] * tn;
    rhs[i] = v;
  }
}

__global__ void set_pin_kernel(double* __restrict__ T, const double* __restrict__ B, const double* __restrict__ C,
                               int pin) {
  T[pin] = B[pin] + C[pin];
}

// block partial max/min
__global__ void minmax_kernel(int64_t n, const double* __restrict__ T, double* __restrict__ pmax,
                              double* __restrict__ pmin) {
  __shared__ double rmx[FT / 32], rmn[FT / 32];
  double mx = -INFINITY, mn = INFINITY;
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) {
    mx = fmax(mx, T[i]);
    mn = fmin(mn, T[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  }
  if ((threadIdx.x & 31) == 0) { rmx[threadIdx.x >> 5] = mx; rmn[threadIdx.x >> 5] = mn; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < FT / 32; ++w) { mx = fmax(mx, rmx[w]); mn = fmin(mn, rmn[w]); }
    mx = rmx[0] > mx ? rmx[0] : mx;
    mn = rmn[0] < mn ? rmn[0] : mn;
    pmax[blockIdx.x] = mx;
    pmin[blockIdx.x] = mn;
  }
}

__global__ void shift_kernel(int64_t n, double* __restrict__ T, double s) {
  for (int64_t i = (int64_t)blockIdx.x * FT + threadIdx.x; i < n; i += (int64_t)gridDim.x * FT) T[i] -= s;
}

// least-squares gradient: grad[c] = sum_k gw[c][:, k] * diff[c][k]
//   diff = T[nb] - T[c] + off   (nb >= 0),   off (nb < 0, no mixed),   value - T[c] (mixed)
__global__ void gradient_kernel(int64_t n, int nv, int dim, const int32_t* __restrict__ nb,
                                const double* __restrict__ off, const unsigned char* __restrict__ mixed,
                                const double* __restrict__ gw, const double* __restrict__ T, double* __restrict__ grad) {
  for (int64_t c = (int64_t)blockIdx.x * FT + threadIdx.x; c < n; c += (int64_t)gridDim.x * FT) {
    const double tc = T[c];
    double g[3] = {0, 0, 0};
    for (int k = 0; k < nv; ++k) {
      const int j = nb[c * nv + k];
      double d;
      if (mixed[c * nv + k]) d = off[c * nv + k] - tc;
      else d = (j >= 0 ? T[j] - tc : 0.0) + off[c * nv + k];
      for (int a = 0; a < dim; ++a) g[a] += gw[(c * dim + a) * nv + k] * d;
    }
    for (int a = 0; a < dim; ++a) grad[c * dim + a] = g[a];
  }
}

// per internal side: tmp = (w grad_i + (1-w) grad_j) . vnon
__global__ void side_flux_kernel(int64_t ns, int dim, const int32_t* __restrict__ si, const int32_t* __restrict__ sj,
                                 const double* __restrict__ w, const double* __restrict__ vnon,
                                 const double* __restrict__ grad, double* __restrict__ tmp) {
  for (int64_t s = (int64_t)blockIdx.x * FT + threadIdx.x; s < ns; s += (int64_t)gridDim.x * FT) {
    const int i = si[s], j = sj[s];
    double t = 0;
    for (int a = 0; a < dim; ++a) t += (w[s] * grad[i * dim + a] + (1.0 - w[s]) * grad[j * dim + a]) * vnon[s * dim + a];
    tmp[s] = t;
  }
}

// C[c] = sum over its internal sides of +-tmp / V_c  (gather, fixed order); partial ‖C‖^2
__global__ void correction_kernel(int64_t n, const int32_t* __restrict__ cp, const int32_t* __restrict__ cs,
                                  const double* __restrict__ tmp, const double* __restrict__ vol,
                                  double* __restrict__ C, double* __restrict__ part) {
  __shared__ double red[FT / 32];
  double acc = 0;
  for (int64_t c = (int64_t)blockIdx.x * FT + threadIdx.x; c < n; c += (int64_t)gridDim.x * FT) {
    double v = 0;
    for (int k = cp[c]; k < cp[c + 1]; ++k) {
      const int e = cs[k];
      v += e >= 0 ? tmp[e] : -tmp[-e - 1];
    }
    v /= vol[c];
    C[c] = v;
    acc += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < FT / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// diffusive kappa terms per contact side (objects.py:152-170)
__global__ void contact_kernel(int64_t nc, const int32_t* __restrict__ e1, const int32_t* __restrict__ e2,
                               const double* __restrict__ coef, double t2const, const double* __restrict__ T,
                               double* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * FT + threadIdx.x; k < nc; k += (int64_t)gridDim.x * FT) {
    const double t2 = e2[k] >= 0 ? T[e2[k]] + t2const : t2const;
    out[k] = (T[e1[k]] - t2) * coef[k];
  }
}

// J = -kappa . grad
__global__ void flux_kernel(int64_t n, int dim, const double* __restrict__ kap, const double* __restrict__ grad,
                            double* __restrict__ J) {
  for (int64_t c = (int64_t)blockIdx.x * FT + threadIdx.x; c < n; c += (int64_t)gridDim.x * FT)
    for (int a = 0; a < dim; ++a) {
      double s = 0;
      for (int b = 0; b < dim; ++b) s += kap[a * dim + b] * grad[c * dim + b];
      J[c * dim + a] = -s;
    }
}

}  // namespace
}  // namespace obte

struct obte_fourier_plan_s {
  obte_context ctx = nullptr;
  int64_t n = 0, ns_int = 0, nc = 0;
  int dim = 2, nv = 3, pin = -1;
  int nb = 1;
  double normalization = 0, contact_t2 = 0;
  std::vector<double> kappa;
  obte::DevBuf rp, ci, val, dinv, vol, B, colpin, g_nb, g_off, g_mixed, gw, s_i, s_j, s_w, s_vnon, c_ptr, c_side,
      k_e1, k_e2, k_coef, kap;
  // work
  obte::DevBuf C, rhs, r, z, p, Ap, part, part2, part3, sc, grad, tmp, kout, pmx, pmn;
  // CG iterations between two convergence checks as one CUDA graph (captured per solution pointer)
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t cg_exec = nullptr;
  const double* cg_exec_T = nullptr;
  // smoothed-aggregation AMG V-cycle as the CG preconditioner (null: Jacobi)
  obte::AmgPtr amg;
  ~obte_fourier_plan_s() {
    if (cg_exec) cudaGraphExecDestroy(cg_exec);
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }
};

using namespace obte;

extern "C" obte_status obte_fourier_plan_create(obte_context ctx, const obte_fourier_problem* pb,
                                                obte_fourier_plan* out) {
  if (!ctx || !pb || !out) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  const int dim = pb->dim;
  const int64_t n = pb->n_elems, ns = pb->n_sides;
  const int nv = pb->elem_nv;
  if ((dim != 2 && dim != 3) || n <= 0 || ns <= 0 || nv < dim + 1 || nv > 8 || !pb->side_elem_map ||
      !pb->normal_areas || !pb->dists || !pb->elem_volumes || !pb->interp_weights || !pb->gradient_weights ||
      !pb->elem_side_map || !pb->kappa) {
    set_error("bad Fourier problem");
    return OBTE_ERR_BAD_ARG;
  }
  OBTE_CUDA(cudaSetDevice(ctx->device));
  const int64_t* sem = pb->side_elem_map;
  const double* na = pb->normal_areas;
  const double* vol = pb->elem_volumes;
  auto inr = [&](int64_t v, int64_t m) { return v >= 0 && v < m; };
  // v_orth, v_nonorth (objects.py:312-319)
  std::vector<double> vo(ns), vn(ns * dim);
  const double* K = pb->kappa;
  for (int64_t s = 0; s < ns; ++s) {
    double num = 0, den = 0;
    double kn[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a)
      for (int b = 0; b < dim; ++b) kn[a] += K[a * dim + b] * na[s * dim + b];
    for (int a = 0; a < dim; ++a) { num += na[s * dim + a] * kn[a]; den += na[s * dim + a] * pb->dists[s * dim + a]; }
    vo[s] = num / den;
    for (int a = 0; a < dim; ++a) vn[s * dim + a] = kn[a] - pb->dists[s * dim + a] * vo[s];
  }
  // L (symmetric, volume-weighted) as a map per row; B (fourier.py:51-107)
  std::vector<std::map<int64_t, double>> L(n);
  std::vector<double> B(n, 0.0);
  for (int64_t t = 0; t < pb->n_internal; ++t) {
    const int64_t s = pb->internal[t];
    if (!inr(s, ns)) { set_error("internal side out of range"); return OBTE_ERR_BAD_ARG; }
    const int64_t i = sem[2 * s], j = sem[2 * s + 1];
    if (!inr(i, n) || !inr(j, n)) { set_error("side_elem_map out of range"); return OBTE_ERR_BAD_ARG; }
    L[i][i] += vo[s]; L[i][j] -= vo[s];
    L[j][j] += vo[s]; L[j][i] -= vo[s];
  }
  for (int64_t k = 0; k < pb->n_mixed; ++k) {
    const int64_t s = pb->mixed_sides[k];
    if (!inr(s, ns)) { set_error("mixed side out of range"); return OBTE_ERR_BAD_ARG; }
    const int64_t i = sem[2 * s];
    const double h = pb->mixed_conductance[k];
    const double tmp = vo[s] * h / (h + vo[s] / pb->side_areas[s]);
    L[i][i] += tmp;
    B[i] = pb->mixed_value[k] * tmp / vol[i];
  }
  for (int64_t k = 0; k < pb->n_periodic; ++k) {
    const int64_t s = pb->periodic_sides[k];
    if (!inr(s, ns)) { set_error("periodic side out of range"); return OBTE_ERR_BAD_ARG; }
    const int64_t i = sem[2 * s], j = sem[2 * s + 1];
    B[i] += pb->periodic_jump[k] * vo[s] / vol[i];
    B[j] -= pb->periodic_jump[k] * vo[s] / vol[j];
  }
  if (pb->heat_source)
    for (int64_t i = 0; i < n; ++i) B[i] += pb->heat_source[i] * 1e-18;
  int pin = -1;
  if (pb->n_mixed == 0) {
    pin = pb->pin_elem;
    if (!inr(pin, n)) { set_error("pin element out of range"); return OBTE_ERR_BAD_ARG; }
    B[pin] = 0;
  }
  // masked CSR (row and column of the pinned element removed; its column kept aside)
  std::vector<int32_t> rp(n + 1, 0), ci;
  std::vector<double> val, dinv(n, 0.0), colpin(n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    if ((int)i != pin)
      for (auto& kv : L[i]) {
        if (kv.first == pin) { colpin[i] = kv.second; continue; }
        ci.push_back((int32_t)kv.first);
        val.push_back(kv.second);
        if (kv.first == i) dinv[i] = kv.second != 0 ? 1.0 / kv.second : 0.0;
      }
    rp[i + 1] = (int32_t)ci.size();
  }
  // gradient stencil (objects.py:330-403)
  std::vector<int32_t> gnb(n * nv, -1);
  std::vector<double> goff(n * nv, 0.0);
  std::vector<unsigned char> gmix(n * nv, 0);
  std::vector<int64_t> esm(pb->elem_side_map, pb->elem_side_map + n * nv);
  auto slot_of = [&](int64_t e, int64_t s) -> int {
    for (int k = 0; k < nv; ++k)
      if (esm[e * nv + k] == s) return k;
    return -1;
  };
  for (int64_t t = 0; t < pb->n_internal; ++t) {
    const int64_t s = pb->internal[t];
    const int64_t i = sem[2 * s], j = sem[2 * s + 1];
    const int a = slot_of(i, s), b = slot_of(j, s);
    if (a < 0 || b < 0) { set_error("elem_side_map does not list an internal side"); return OBTE_ERR_BAD_ARG; }
    gnb[i * nv + a] = (int32_t)j;
    gnb[j * nv + b] = (int32_t)i;
  }
  for (int64_t k = 0; k < pb->n_periodic; ++k) {
    const int64_t s = pb->periodic_sides[k];
    const int64_t i = sem[2 * s], j = sem[2 * s + 1];
    const int a = slot_of(i, s), b = slot_of(j, s);
    if (a < 0 || b < 0) { set_error("elem_side_map does not list a periodic side"); return OBTE_ERR_BAD_ARG; }
    goff[i * nv + a] += pb->periodic_jump[k];
    goff[j * nv + b] -= pb->periodic_jump[k];
  }
  for (int64_t k = 0; k < pb->n_mixed; ++k) {
    const int64_t s = pb->mixed_sides[k];
    const int64_t i = sem[2 * s];
    const int a = slot_of(i, s);
    if (a < 0) { set_error("elem_side_map does not list a mixed side"); return OBTE_ERR_BAD_ARG; }
    gmix[i * nv + a] = 1;
    goff[i * nv + a] = pb->mixed_value[k];
  }
  // correction: internal sides and per-element gather lists (+ side+1 / -(side+1))
  const int64_t ni = pb->n_internal;
  std::vector<int32_t> s_i(ni), s_j(ni);
  std::vector<double> s_w(ni), s_vn(ni * dim);
  std::vector<std::vector<int32_t>> gl(n);
  for (int64_t t = 0; t < ni; ++t) {
    const int64_t s = pb->internal[t];
    s_i[t] = (int32_t)sem[2 * s];
    s_j[t] = (int32_t)sem[2 * s + 1];
    s_w[t] = pb->interp_weights[s];
    for (int a = 0; a < dim; ++a) s_vn[t * dim + a] = vn[s * dim + a];
    gl[s_i[t]].push_back((int32_t)t);
    gl[s_j[t]].push_back((int32_t)(-t - 1));
  }
  std::vector<int32_t> cptr(n + 1, 0), cside;
  for (int64_t c = 0; c < n; ++c) {
    cside.insert(cside.end(), gl[c].begin(), gl[c].end());
    cptr[c + 1] = (int32_t)cside.size();
  }
  // contact (objects.py:139-172)
  std::vector<int32_t> ke1, ke2;
  std::vector<double> kco;
  double t2const = 0;
  if (pb->contact_kind == OBTE_CONTACT_PERIODIC || pb->contact_kind == OBTE_CONTACT_MIXED) {
    for (int64_t k = 0; k < pb->n_contact; ++k) {
      const int64_t s = pb->contact_sides[k];
      if (!inr(s, ns)) { set_error("contact side out of range"); return OBTE_ERR_BAD_ARG; }
      ke1.push_back((int32_t)sem[2 * s]);
      if (pb->contact_kind == OBTE_CONTACT_PERIODIC) {
        ke2.push_back((int32_t)sem[2 * s + 1]);
        kco.push_back(vo[s] * pb->normalization);
      } else {
        ke2.push_back(-1);
        const double h = pb->contact_conductance;
        kco.push_back(vo[s] * h / (h + vo[s] / pb->side_areas[s]) * pb->normalization);
      }
    }
    t2const = pb->contact_alpha;
  }
  auto* P = new obte_fourier_plan_s();
  P->ctx = ctx;
  P->n = n; P->dim = dim; P->nv = nv; P->pin = pin; P->ns_int = ni; P->nc = (int64_t)ke1.size();
  P->contact_t2 = t2const;
  P->kappa.assign(pb->kappa, pb->kappa + dim * dim);
  P->nb = (int)std::max<int64_t>(1, std::min<int64_t>((n + FT - 1) / FT, (int64_t)ctx->num_sms * 2));
  cudaStream_t st = ctx->stream;
  std::vector<double> volv(vol, vol + n);
  std::vector<double> gwv(pb->gradient_weights, pb->gradient_weights + n * dim * nv);
  std::vector<int32_t> gmix32(gmix.begin(), gmix.end());
  obte_status s0 = OBTE_OK;
  auto up = [&](obte_status s) { if (s0 == OBTE_OK) s0 = s; };
  up(upload(P->rp, rp, st)); up(upload(P->ci, ci, st)); up(upload(P->val, val, st)); up(upload(P->dinv, dinv, st));
  up(upload(P->vol, volv, st)); up(upload(P->B, B, st)); up(upload(P->colpin, colpin, st));
  up(upload(P->g_nb, gnb, st)); up(upload(P->g_off, goff, st));
  {
    std::vector<int32_t> tmpm(gmix.size());
    // stored as bytes on the device
    up(P->g_mixed.alloc(gmix.size()));
    if (s0 == OBTE_OK && !gmix.empty()) {
      cudaError_t e = cudaMemcpyAsync(P->g_mixed.p, gmix.data(), gmix.size(), cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) up(cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__));
    }
  }
  up(upload(P->gw, gwv, st));
  up(upload(P->s_i, s_i, st)); up(upload(P->s_j, s_j, st)); up(upload(P->s_w, s_w, st)); up(upload(P->s_vnon, s_vn, st));
  up(upload(P->c_ptr, cptr, st)); up(upload(P->c_side, cside, st));
  up(upload(P->k_e1, ke1, st)); up(upload(P->k_e2, ke2, st)); up(upload(P->k_coef, kco, st));
  up(upload(P->kap, P->kappa, st));
  const size_t vb = (size_t)n * sizeof(double);
  up(P->C.alloc(vb)); up(P->rhs.alloc(vb)); up(P->r.alloc(vb)); up(P->z.alloc(vb)); up(P->p.alloc(vb));
  up(P->Ap.alloc(vb)); up(P->part.alloc((size_t)P->nb * sizeof(double))); up(P->part2.alloc((size_t)P->nb * sizeof(double)));
  up(P->part3.alloc((size_t)P->nb * sizeof(double)));
  up(P->sc.alloc(8 * sizeof(double))); up(P->grad.alloc(vb * dim)); up(P->tmp.alloc((size_t)std::max<int64_t>(ni, 1) * 8));
  up(P->kout.alloc((size_t)std::max<int64_t>(P->nc, 1) * 8));
  up(P->pmx.alloc((size_t)P->nb * 8)); up(P->pmn.alloc((size_t)P->nb * 8));
  // OBTE_FOURIER_JACOBI=1 keeps the diagonal preconditioner (same solution, ~40x more CG iterations)
  const char* jac = std::getenv("OBTE_FOURIER_JACOBI");
  if (s0 == OBTE_OK && !(jac && std::atoi(jac) != 0))
    up(amg_build(n, rp, ci, val, pin, ctx->num_sms, st, P->amg));
  if (s0 == OBTE_OK) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s0 = cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
  }
  if (s0 != OBTE_OK) { delete P; return s0; }
  *out = P;
  return OBTE_OK;
}

extern "C" obte_status obte_fourier_plan_destroy(obte_fourier_plan plan) {
  if (plan && plan->ctx) cudaStreamSynchronize(plan->ctx->stream);
  delete plan;
  return OBTE_OK;
}

// Preconditioned CG (AMG V-cycle, or Jacobi) on the masked system, warm-started from T (device). Returns iterations.
static obte_status cg_solve(obte_fourier_plan P, double* T, double rtol, int max_iter, int& iters) {
  cudaStream_t st = P->ctx->stream;
  const int64_t n = P->n;
  const int nb = P->nb;
  double* sc = P->sc.as<double>();
  double *r = P->r.as<double>(), *z = P->z.as<double>(), *p = P->p.as<double>(), *Ap = P->Ap.as<double>();
  const int32_t *rp = P->rp.as<int32_t>(), *ci = P->ci.as<int32_t>();
  const double* val = P->val.as<double>();
  // r = rhs - L T, z = r dinv, p = z; rz -> sc[0], rr -> sc[3], ‖rhs‖^2 -> sc[5]
  const AmgHierarchy* amg = P->amg.get();
  spmv_kernel<<<nb, FT, 0, st>>>(n, rp, ci, val, T, Ap, P->part.as<double>());
  cg_init_kernel<<<nb, FT, 0, st>>>(n, P->rhs.as<double>(), Ap, P->dinv.as<double>(), r, z, p, P->part.as<double>(),
                                    P->part2.as<double>(), P->part3.as<double>());
  if (amg) {                         // z = M^-1 r, p = z, r.z
    count_launch(amg_apply(*amg, r, z, nullptr, 0, st));
    rz_kernel<<<nb, FT, 0, st>>>(n, r, z, p, P->part.as<double>());
    count_launch();
  }
  reduce_kernel<<<1, FT, 0, st>>>(P->part.as<double>(), nb, sc + 0);
  reduce_kernel<<<1, FT, 0, st>>>(P->part2.as<double>(), nb, sc + 3);
  reduce_kernel<<<1, FT, 0, st>>>(P->part3.as<double>(), nb, sc + 5);
  count_launch(5);
  OBTE_CUDA(cudaGetLastError());
  double hs[6];
  OBTE_CUDA(cudaMemcpyAsync(hs, sc, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
  OBTE_CUDA(cudaStreamSynchronize(st));
  {
    const double tol = rtol * std::max(std::sqrt(std::max(hs[5], 0.0)), 1e-300);
    iters = 0;
    if (std::sqrt(std::max(hs[3], 0.0)) <= tol) return OBTE_OK;
    // three launches per iteration; rz alternates between sc[0] and sc[1].  At a few microseconds of work
    // per launch the loop is launch-bound, so the `check` iterations between two convergence tests are
    // captured once as a CUDA graph (on a private stream: capture is not allowed on the legacy default
    // stream) and replayed on the plan's stream.  `check` is even, so every block starts with cur = 0.
    // With the AMG preconditioner a solve takes a few tens of iterations, so the check comes every 4.
    // The V-cycle writes z and the partials of r.z (cg_step_kernel then skips its Jacobi z).
    const int check = amg ? 4 : 8;
    double* pp = P->part.as<double>();
    double* prz = P->part2.as<double>();
    double* prr = P->part3.as<double>();
    const int per_iter = amg ? 3 + amg_launches(*amg, true) : 3;
    auto enqueue = [&](cudaStream_t s2) {
      for (int k = 0; k < check; ++k) {
        const int cur = k & 1;
        spmv_kernel<<<nb, FT, 0, s2>>>(n, rp, ci, val, p, Ap, pp);
        cg_step_kernel<<<nb, FT, 0, s2>>>(n, pp, nb, sc, cur, T, r, amg ? nullptr : z, p, Ap, P->dinv.as<double>(),
                                          prz, prr);
        if (amg) amg_apply(*amg, r, z, prz, nb, s2);
        cg_dir_kernel<<<nb, FT, 0, s2>>>(n, prz, prr, nb, sc, cur, p, z);
      }
    };
    if (P->cg_exec_T != T && !std::getenv("OBTE_NO_GRAPHS")) {
      if (P->cg_exec) { cudaGraphExecDestroy(P->cg_exec); P->cg_exec = nullptr; }
      if (!P->capture_stream) OBTE_CUDA(cudaStreamCreateWithFlags(&P->capture_stream, cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      OBTE_CUDA(cudaStreamBeginCapture(P->capture_stream, cudaStreamCaptureModeThreadLocal));
      enqueue(P->capture_stream);
      OBTE_CUDA(cudaStreamEndCapture(P->capture_stream, &g));
      const cudaError_t e = cudaGraphInstantiate(&P->cg_exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
      P->cg_exec_T = T;
    }
    while (iters < max_iter) {
      if (P->cg_exec && P->cg_exec_T == T) OBTE_CUDA(cudaGraphLaunch(P->cg_exec, st));
      else enqueue(st);
      count_launch(per_iter * check);
      iters += check;
      OBTE_CUDA(cudaGetLastError());
      OBTE_CUDA(cudaMemcpyAsync(hs, sc, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
      OBTE_CUDA(cudaStreamSynchronize(st));
      if (std::sqrt(std::max(hs[3], 0.0)) <= tol) break;
    }
  }
  return OBTE_OK;
}

extern "C" obte_status obte_fourier_solve(obte_fourier_plan P, const obte_fourier_opts* opts, double* T, double* J,
                                          obte_fourier_info* info) {
  if (!P || !opts || !T) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  cudaStream_t st = P->ctx->stream;
  const int64_t n = P->n;
  const int nb = P->nb;
  const int max_iter = opts->max_iter > 0 ? opts->max_iter : 40;
  const double rtol = opts->rtol > 0 ? opts->rtol : 1e-8;
  const double cg_rtol = opts->cg_rtol > 0 ? opts->cg_rtol : 1e-13;
  const int cg_max = opts->cg_max_iter > 0 ? opts->cg_max_iter : 20000;
  double* C = P->C.as<double>();
  OBTE_CUDA(cudaMemsetAsync(C, 0, n * sizeof(double), st));
  OBTE_CUDA(cudaMemsetAsync(T, 0, n * sizeof(double), st));
  double norm_old = 0, err = 1, kappa = 0;
  int it = 0, ncg = 0;
  while (err > rtol && it < max_iter) {                                          // fourier.py:149
    ++it;
    cg_rhs_kernel<<<nb, FT, 0, st>>>(n, P->vol.as<double>(), P->B.as<double>(), C, P->pin, P->colpin.as<double>(),
                                     P->rhs.as<double>());
    count_launch();
    int k = 0;
    if (P->pin >= 0) {
      // the previous T was re-centred; shift it back onto the pinned value so the warm start
      // differs from the new solution only by the change of C (a uniform shift is in L's null space)
      pin_delta_kernel<<<1, 1, 0, st>>>(T, P->B.as<double>(), C, P->pin, P->sc.as<double>() + 6);
      shift_by_kernel<<<nb, FT, 0, st>>>(n, T, P->sc.as<double>() + 6);
      count_launch(2);
    }
    OBTE_TRY(cg_solve(P, T, cg_rtol, cg_max, k));                                // fourier.py:152
    ncg += k;
    if (P->pin >= 0) {
      set_pin_kernel<<<1, 1, 0, st>>>(T, P->B.as<double>(), C, P->pin);
      count_launch();
      // T -= (max + min)/2                                                      // fourier.py:155-156
      minmax_kernel<<<nb, FT, 0, st>>>(n, T, P->pmx.as<double>(), P->pmn.as<double>());
      count_launch();
      std::vector<double> mx(nb), mn(nb);
      OBTE_CUDA(cudaMemcpyAsync(mx.data(), P->pmx.p, nb * 8, cudaMemcpyDeviceToHost, st));
      OBTE_CUDA(cudaMemcpyAsync(mn.data(), P->pmn.p, nb * 8, cudaMemcpyDeviceToHost, st));
      OBTE_CUDA(cudaStreamSynchronize(st));
      double a = mx[0], b = mn[0];
      for (int i = 1; i < nb; ++i) { a = std::max(a, mx[i]); b = std::min(b, mn[i]); }
      shift_kernel<<<nb, FT, 0, st>>>(n, T, (a + b) * 0.5);
      count_launch();
    }
    gradient_kernel<<<nb, FT, 0, st>>>(n, P->nv, P->dim, P->g_nb.as<int32_t>(), P->g_off.as<double>(),
                                       P->g_mixed.as<unsigned char>(), P->gw.as<double>(), T, P->grad.as<double>());
    side_flux_kernel<<<nb, FT, 0, st>>>(P->ns_int, P->dim, P->s_i.as<int32_t>(), P->s_j.as<int32_t>(),
                                        P->s_w.as<double>(), P->s_vnon.as<double>(), P->grad.as<double>(),
                                        P->tmp.as<double>());
    correction_kernel<<<nb, FT, 0, st>>>(n, P->c_ptr.as<int32_t>(), P->c_side.as<int32_t>(), P->tmp.as<double>(),
                                         P->vol.as<double>(), C, P->part.as<double>());
    reduce_kernel<<<1, FT, 0, st>>>(P->part.as<double>(), nb, P->sc.as<double>() + 4);
    count_launch(4);
    OBTE_CUDA(cudaGetLastError());
    double cc;
    OBTE_CUDA(cudaMemcpyAsync(&cc, P->sc.as<double>() + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
    OBTE_CUDA(cudaStreamSynchronize(st));
    const double norm_C = std::sqrt(std::max(cc, 0.0));
    err = norm_C == 0 ? 0 : std::fabs(norm_C - norm_old) / norm_C;                  // fourier.py:168-171
    norm_old = norm_C;
    if (P->nc > 0) {
      contact_kernel<<<nb, FT, 0, st>>>(P->nc, P->k_e1.as<int32_t>(), P->k_e2.as<int32_t>(), P->k_coef.as<double>(),
                                        P->contact_t2, T, P->kout.as<double>());
      count_launch();
      std::vector<double> kh(P->nc);
      OBTE_CUDA(cudaMemcpyAsync(kh.data(), P->kout.p, P->nc * 8, cudaMemcpyDeviceToHost, st));
      OBTE_CUDA(cudaStreamSynchronize(st));
      kappa = 0;
      for (double v : kh) kappa += v;
    }
  }
  if (J) {
    flux_kernel<<<nb, FT, 0, st>>>(n, P->dim, P->kap.as<double>(), P->grad.as<double>(), J);
    count_launch();
  }
  OBTE_CUDA(cudaGetLastError());
  OBTE_CUDA(cudaStreamSynchronize(st));
  if (info) {
    info->kappa = kappa;
    info->n_iter = it;
    info->n_cg = ncg;
  }
  return OBTE_OK;
}
