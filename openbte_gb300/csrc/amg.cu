// Smoothed-aggregation algebraic multigrid: the preconditioner of the Fourier CG.
//
// The Fourier first guess solves the volume-weighted diffusion operator L (symmetric, an M-matrix) ten or
// more times per call (one CG solve per deferred-correction pass, openbte/fourier.py:149-178).  With Jacobi
// preconditioning a 60k-element cell needs ~1,200 CG iterations per solve; one symmetric V-cycle of a
// smoothed-aggregation hierarchy brings that to a few tens.
//
// Setup (host, once per Fourier plan): per level, strong couplings |a_ij| >= theta sqrt(a_ii a_jj); greedy
// aggregation (seed aggregates whose strong neighbours are all free, then attach the rest to a neighbouring
// aggregate, then aggregate leftovers); piecewise-constant tentative prolongator smoothed by one weighted
// Jacobi step, P = (I - omega D^-1 A) P0 with omega = 4 / (3 lambda_max(D^-1 A)) (power iteration); Galerkin
// coarse operator A_c = P^T A P (row-wise sparse products, columns sorted: the hierarchy is deterministic).
// The coarsest operator (a few hundred unknowns) is inverted densely.
//
// The V-cycle smooths with one weighted-Jacobi step from zero before the coarse correction and the same
// step after it (so M is symmetric positive definite and CG keeps its guarantees):
//   x1 = w D^-1 b;  b_c = P^T (b - A x1);  x_c = M_c^-1 b_c;  x2 = x1 + P x_c;  x = x2 + w D^-1 (b - A x2).
// Both smoothing steps fold into the level's matrices: with Q = (I - w D^-1 A) P and
// G = w D^-1 (2 I - w A D^-1) (symmetric, A's pattern),
//   b_c = Q^T b    and    x = G b + Q x_c,
// so the device applies one sparse product per level on the way down and one on the way up, plus one dense
// product with the coarsest inverse: 2 (levels - 1) + 1 launches per V-cycle instead of 6 per level.  The
// launches are enqueued on a stream and are therefore capturable in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "internal.h"

namespace obte {

namespace {

constexpr int AT = 256;

struct HostCsr {
  int64_t n = 0, m = 0;
  std::vector<int64_t> rp;
  std::vector<int32_t> ci;
  std::vector<double> val;
};

HostCsr transpose(const HostCsr& A) {
  HostCsr T;
  T.n = A.m;
  T.m = A.n;
  T.rp.assign(T.n + 1, 0);
  for (int32_t c : A.ci) T.rp[c + 1]++;
  for (int64_t i = 0; i < T.n; ++i) T.rp[i + 1] += T.rp[i];
  T.ci.resize(A.ci.size());
  T.val.resize(A.val.size());
  std::vector<int64_t> pos(T.rp.begin(), T.rp.end() - 1);
  for (int64_t i = 0; i < A.n; ++i)          // rows in order: the columns of T come out sorted
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
      const int64_t d = pos[A.ci[k]]++;
      T.ci[d] = (int32_t)i;
      T.val[d] = A.val[k];
    }
  return T;
}

// C = A B, row by row with a dense accumulator; columns sorted, exact zeros dropped
HostCsr spgemm(const HostCsr& A, const HostCsr& B) {
  HostCsr C;
  C.n = A.n;
  C.m = B.m;
  C.rp.assign(A.n + 1, 0);
  std::vector<int64_t> mark(B.m, -1);
  std::vector<double> acc(B.m, 0.0);
  std::vector<int32_t> cols;
  for (int64_t i = 0; i < A.n; ++i) {
    cols.clear();
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
      const int32_t j = A.ci[k];
      const double a = A.val[k];
      for (int64_t l = B.rp[j]; l < B.rp[j + 1]; ++l) {
        const int32_t c = B.ci[l];
        if (mark[c] != i) {
          mark[c] = i;
          acc[c] = 0.0;
          cols.push_back(c);
        }
        acc[c] += a * B.val[l];
      }
    }
    std::sort(cols.begin(), cols.end());
    for (int32_t c : cols)
      if (acc[c] != 0.0) {
        C.ci.push_back(c);
        C.val.push_back(acc[c]);
      }
    C.rp[i + 1] = (int64_t)C.ci.size();
  }
  return C;
}

// C = X + diag(s) Y (row-wise merge; X and Y have sorted columns, so C does too)
HostCsr add_scaled(const HostCsr& X, const HostCsr& Y, const std::vector<double>& s) {
  HostCsr C;
  C.n = X.n;
  C.m = X.m;
  C.rp.assign(X.n + 1, 0);
  for (int64_t i = 0; i < X.n; ++i) {
    int64_t a = X.rp[i], b = Y.rp[i];
    const int64_t ae = X.rp[i + 1], be = Y.rp[i + 1];
    while (a < ae || b < be) {
      if (b >= be || (a < ae && X.ci[a] < Y.ci[b])) {
        C.ci.push_back(X.ci[a]);
        C.val.push_back(X.val[a]);
        ++a;
      } else if (a >= ae || Y.ci[b] < X.ci[a]) {
        C.ci.push_back(Y.ci[b]);
        C.val.push_back(s[i] * Y.val[b]);
        ++b;
      } else {
        C.ci.push_back(X.ci[a]);
        C.val.push_back(X.val[a] + s[i] * Y.val[b]);
        ++a;
        ++b;
      }
    }
    C.rp[i + 1] = (int64_t)C.ci.size();
  }
  return C;
}

std::vector<double> diagonal(const HostCsr& A) {
  std::vector<double> d(A.n, 0.0);
  for (int64_t i = 0; i < A.n; ++i)
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (A.ci[k] == i) d[i] = A.val[k];
  return d;
}

// largest eigenvalue of D^-1 A by power iteration (deterministic start), a few percent high for safety
double lambda_max(const HostCsr& A, const std::vector<double>& d) {
  std::vector<double> x(A.n), y(A.n);
  for (int64_t i = 0; i < A.n; ++i) x[i] = 1.0 + 0.5 * std::sin(0.7 * (double)i);
  double lam = 1.0;
  for (int it = 0; it < 20; ++it) {
    double nrm = 0;
    for (int64_t i = 0; i < A.n; ++i) {
      double s = 0;
      for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) s += A.val[k] * x[A.ci[k]];
      y[i] = d[i] != 0 ? s / d[i] : 0.0;
      nrm += y[i] * y[i];
    }
    nrm = std::sqrt(nrm);
    if (nrm == 0) return 1.0;
    double xn = 0;
    for (double v : x) xn += v * v;
    lam = nrm / std::sqrt(xn);
    for (int64_t i = 0; i < A.n; ++i) x[i] = y[i] / nrm;
  }
  return 1.05 * lam;
}

// one coarsening step; false when aggregation no longer reduces the size enough
bool coarsen(const HostCsr& A, double theta, HostCsr& Q, HostCsr& Ac, double& omega) {
  const int64_t n = A.n;
  const std::vector<double> d = diagonal(A);
  auto strong = [&](int64_t i, int64_t k) {
    const int32_t j = A.ci[k];
    return j != i && A.val[k] != 0 && std::fabs(A.val[k]) >= theta * std::sqrt(std::fabs(d[i] * d[j]));
  };
  std::vector<int32_t> agg(n, -1);
  int32_t na = 0;
  for (int64_t i = 0; i < n; ++i) {          // pass 1: seeds with all strong neighbours free
    if (agg[i] >= 0) continue;
    bool free_nb = true;
    for (int64_t k = A.rp[i]; k < A.rp[i + 1] && free_nb; ++k)
      if (strong(i, k) && agg[A.ci[k]] >= 0) free_nb = false;
    if (!free_nb) continue;
    agg[i] = na;
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (strong(i, k)) agg[A.ci[k]] = na;
    ++na;
  }
  std::vector<int32_t> agg1(agg);
  for (int64_t i = 0; i < n; ++i) {          // pass 2: join a neighbouring pass-1 aggregate
    if (agg[i] >= 0) continue;
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (strong(i, k) && agg1[A.ci[k]] >= 0) { agg[i] = agg1[A.ci[k]]; break; }
  }
  for (int64_t i = 0; i < n; ++i) {          // pass 3: leftovers (isolated nodes included)
    if (agg[i] >= 0) continue;
    agg[i] = na;
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (strong(i, k) && agg[A.ci[k]] < 0) agg[A.ci[k]] = na;
    ++na;
  }
  if (na == 0 || (double)na > 0.85 * (double)n) return false;
  HostCsr P0;
  P0.n = n;
  P0.m = na;
  P0.rp.resize(n + 1);
  P0.ci.resize(n);
  P0.val.assign(n, 1.0);
  for (int64_t i = 0; i <= n; ++i) P0.rp[i] = i;
  for (int64_t i = 0; i < n; ++i) P0.ci[i] = agg[i];
  omega = 4.0 / (3.0 * lambda_max(A, d));
  std::vector<double> s(n);
  for (int64_t i = 0; i < n; ++i) s[i] = d[i] != 0 ? -omega / d[i] : 0.0;
  const HostCsr P = add_scaled(P0, spgemm(A, P0), s);      // P = P0 - w D^-1 A P0
  const HostCsr AP = spgemm(A, P);
  Q = add_scaled(P, AP, s);                                 // Q = P - w D^-1 A P
  Ac = spgemm(transpose(P), AP);                            // A_c = P^T A P
  return true;
}

// dense inverse by Gauss-Jordan with partial pivoting (the coarsest operator, a few hundred unknowns)
bool dense_inverse(const HostCsr& A, std::vector<double>& inv) {
  const int64_t n = A.n;
  std::vector<double> M((size_t)n * n, 0.0);
  inv.assign((size_t)n * n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) M[(size_t)i * n + A.ci[k]] = A.val[k];
    inv[(size_t)i * n + i] = 1.0;
  }
  for (int64_t c = 0; c < n; ++c) {
    int64_t p = c;
    for (int64_t r = c + 1; r < n; ++r)
      if (std::fabs(M[(size_t)r * n + c]) > std::fabs(M[(size_t)p * n + c])) p = r;
    if (M[(size_t)p * n + c] == 0) return false;
    if (p != c)
      for (int64_t k = 0; k < n; ++k) {
        std::swap(M[(size_t)p * n + k], M[(size_t)c * n + k]);
        std::swap(inv[(size_t)p * n + k], inv[(size_t)c * n + k]);
      }
    const double piv = 1.0 / M[(size_t)c * n + c];
    for (int64_t k = 0; k < n; ++k) {
      M[(size_t)c * n + k] *= piv;
      inv[(size_t)c * n + k] *= piv;
    }
    for (int64_t r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = M[(size_t)r * n + c];
      if (f == 0) continue;
      for (int64_t k = 0; k < n; ++k) {
        M[(size_t)r * n + k] -= f * M[(size_t)c * n + k];
        inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
      }
    }
  }
  return true;
}

// ---- device V-cycle ----------------------------------------------------------------------------

// y = G gx + Q qx (G optional) with VEC lanes per row (lane-strided products, then an xor tree: a fixed
// summation order); with `part`, block partials of gx . y as well.  Every thread runs the same number of
// row passes, so the group shuffles always see full warps.
template <int VEC>
__global__ void __launch_bounds__(AT) amg_rows_kernel(
    int64_t n, const int32_t* __restrict__ grp, const int32_t* __restrict__ gci, const double* __restrict__ gv,
    const double* __restrict__ gx, const int32_t* __restrict__ qrp, const int32_t* __restrict__ qci,
    const double* __restrict__ qv, const double* __restrict__ qx, double* __restrict__ y, double* __restrict__ part) {
  constexpr int GPB = AT / VEC;
  const int lane = (int)(threadIdx.x % VEC);
  const int64_t stride = (int64_t)gridDim.x * GPB;
  const int64_t first = (int64_t)blockIdx.x * GPB + threadIdx.x / VEC;
  const int64_t trips = (n + stride - 1) / stride;
  double dot = 0;
  for (int64_t t = 0; t < trips; ++t) {
    const int64_t row = first + t * stride;
    double acc = 0;
    if (row < n) {
      if (gv)
        for (int k = grp[row] + lane; k < grp[row + 1]; k += VEC) acc += gv[k] * gx[gci[k]];
      for (int k = qrp[row] + lane; k < qrp[row + 1]; k += VEC) acc += qv[k] * qx[qci[k]];
    }
#pragma unroll
    for (int o = VEC / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (row < n && lane == 0) {
      y[row] = acc;
      if (part) dot += gx[row] * acc;
    }
  }
  if (part) {
    __shared__ double red[AT / 32];
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dot;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < AT / 32; ++w) t += red[w];
      part[blockIdx.x] = t;
    }
  }
}

// x = Ainv b (dense, one warp per row, fixed summation order)
__global__ void amg_coarse_kernel(int n, const double* __restrict__ inv, const double* __restrict__ b,
                                  double* __restrict__ x) {
  const int lane = threadIdx.x & 31;
  for (int row = (blockIdx.x * AT + threadIdx.x) >> 5; row < n; row += (gridDim.x * AT) >> 5) {
    double s = 0;
    for (int k = lane; k < n; k += 32) s += inv[(size_t)row * n + k] * b[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = s;
  }
}

// block partials of r . z (a one-level hierarchy has no up-sweep product to carry them)
__global__ void amg_dot_kernel(int64_t n, const double* __restrict__ r, const double* __restrict__ z,
                               double* __restrict__ part) {
  __shared__ double red[AT / 32];
  double dot = 0;
  for (int64_t i = (int64_t)blockIdx.x * AT + threadIdx.x; i < n; i += (int64_t)gridDim.x * AT) dot += r[i] * z[i];
  for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dot;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < AT / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

struct DevCsr {
  int64_t n = 0, nnz = 0;
  DevBuf rp, ci, val;
};

}  // namespace

struct AmgLevel {
  int64_t n = 0;
  DevCsr G;      // w D^-1 (2 I - w A D^-1)       (n_l x n_l)
  DevCsr Q;      // (I - w D^-1 A) P               (n_l x n_l+1)
  DevCsr Qt;     // Q^T                            (n_l+1 x n_l)
  DevBuf b, x;   // right-hand side and correction of this level (level 0 uses the caller's r and z)
};

struct AmgHierarchy {
  std::vector<std::unique_ptr<AmgLevel>> lv;
  DevBuf inv;                        // dense inverse of the coarsest operator
  int nc = 0;
  int num_sms = 1;
};

void AmgDeleter::operator()(AmgHierarchy* h) const { delete h; }

static obte_status upload_csr(const HostCsr& A, DevCsr& d, cudaStream_t st) {
  std::vector<int32_t> rp32(A.rp.begin(), A.rp.end());
  d.n = A.n;
  d.nnz = (int64_t)A.ci.size();
  OBTE_TRY(upload(d.rp, rp32, st));
  OBTE_TRY(upload(d.ci, A.ci, st));
  OBTE_TRY(upload(d.val, A.val, st));
  return OBTE_OK;
}

obte_status amg_build(int64_t n, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                      const std::vector<double>& val, int pin, int num_sms, cudaStream_t st, AmgPtr& out,
                      int coarse_max) {
  PhaseTimer timer("amg_build");
  if (n >= (int64_t)1 << 31 || rp.back() < 0) { set_error("AMG: matrix too large"); return OBTE_ERR_BAD_ARG; }
  HostCsr A;
  A.n = A.m = n;
  A.rp.assign(rp.begin(), rp.end());
  A.ci = ci;
  A.val = val;
  if (pin >= 0) {                    // the pinned element: an identity row, decoupled from the rest
    HostCsr B;
    B.n = B.m = n;
    B.rp.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
      if (i == pin) {
        B.ci.push_back((int32_t)i);
        B.val.push_back(1.0);
      } else {
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
          B.ci.push_back(A.ci[k]);
          B.val.push_back(A.val[k]);
        }
      }
      B.rp[i + 1] = (int64_t)B.ci.size();
    }
    A = std::move(B);
  }
  std::unique_ptr<AmgHierarchy> H(new AmgHierarchy());
  H->num_sms = std::max(1, num_sms);
  const double theta = 0.08;
  while (true) {
    H->lv.emplace_back(new AmgLevel());
    AmgLevel& L = *H->lv.back();
    L.n = A.n;
    if (H->lv.size() > 1) {
      OBTE_TRY(L.x.alloc((size_t)A.n * sizeof(double)));
      OBTE_TRY(L.b.alloc((size_t)A.n * sizeof(double)));
    }
    HostCsr Q, Ac;
    double omega = 0;
    const bool more = A.n > coarse_max && H->lv.size() < 12 && coarsen(A, theta, Q, Ac, omega);
    if (!more) {
      std::vector<double> inv;
      if (!dense_inverse(A, inv)) { set_error("AMG: singular coarsest operator"); return OBTE_ERR_BAD_ARG; }
      OBTE_TRY(upload(H->inv, inv, st));
      H->nc = (int)A.n;
      break;
    }
    // G = 2 w D^-1 - w^2 D^-1 A D^-1 on A's pattern
    const std::vector<double> d = diagonal(A);
    HostCsr G;
    G.n = G.m = A.n;
    G.rp = A.rp;
    G.ci = A.ci;
    G.val.resize(A.val.size());
    for (int64_t i = 0; i < A.n; ++i) {
      const double di = d[i] != 0 ? 1.0 / d[i] : 0.0;
      for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
        const int32_t j = A.ci[k];
        const double dj = d[j] != 0 ? 1.0 / d[j] : 0.0;
        G.val[k] = -omega * omega * di * A.val[k] * dj + (j == i ? 2.0 * omega * di : 0.0);
      }
    }
    OBTE_TRY(upload_csr(G, L.G, st));
    OBTE_TRY(upload_csr(Q, L.Q, st));
    OBTE_TRY(upload_csr(transpose(Q), L.Qt, st));
    A = std::move(Ac);
  }
  out.reset(H.release());
  return OBTE_OK;
}

int amg_levels(const AmgHierarchy& H) { return (int)H.lv.size(); }
int amg_launches(const AmgHierarchy& H, bool with_part) {
  const int nl = (int)H.lv.size();
  return 2 * (nl - 1) + 1 + (with_part && nl == 1 ? 1 : 0);
}

namespace {
// y = G gx + Q qx over n rows, lanes per row from the mean row length; `grid` > 0 fixes the grid (and is
// then the number of partials written to `part`)
void rows_launch(const DevCsr* G, const double* gx, const DevCsr& Q, const double* qx, double* y, double* part,
                 int grid, int num_sms, cudaStream_t st) {
  const int64_t n = Q.n;
  const double mean = (double)(Q.nnz + (G ? G->nnz : 0)) / (double)std::max<int64_t>(n, 1);
  const int vec = mean < 6 ? 1 : mean < 12 ? 2 : mean < 24 ? 4 : mean < 48 ? 8 : mean < 96 ? 16 : 32;
  const int blocks = grid > 0 ? grid
                              : (int)std::max<int64_t>(1, std::min<int64_t>((n * vec + AT - 1) / AT, (int64_t)num_sms * 8));
  const int32_t* grp = G ? G->rp.as<int32_t>() : nullptr;
  const int32_t* gci = G ? G->ci.as<int32_t>() : nullptr;
  const double* gv = G ? G->val.as<double>() : nullptr;
#define OBTE_AMG_ROWS(V)                                                                                       \
  amg_rows_kernel<V><<<blocks, AT, 0, st>>>(n, grp, gci, gv, gx, Q.rp.as<int32_t>(), Q.ci.as<int32_t>(),      \
                                            Q.val.as<double>(), qx, y, part)
  switch (vec) {
    case 1: OBTE_AMG_ROWS(1); break;
    case 2: OBTE_AMG_ROWS(2); break;
    case 4: OBTE_AMG_ROWS(4); break;
    case 8: OBTE_AMG_ROWS(8); break;
    case 16: OBTE_AMG_ROWS(16); break;
    default: OBTE_AMG_ROWS(32); break;
  }
#undef OBTE_AMG_ROWS
}
}  // namespace

// z = M^-1 r (level 0 reads r and writes z directly); with `part`, the nb_part block partials of r . z
int amg_apply(const AmgHierarchy& H, const double* r, double* z, double* part, int nb_part, cudaStream_t st) {
  const int nl = (int)H.lv.size();
  auto bvec = [&](int l) { return l == 0 ? r : H.lv[l]->b.as<double>(); };
  auto xvec = [&](int l) { return l == 0 ? z : H.lv[l]->x.as<double>(); };
  for (int l = 0; l < nl - 1; ++l)                        // b_l+1 = Q_l^T b_l
    rows_launch(nullptr, nullptr, H.lv[l]->Qt, bvec(l), H.lv[l + 1]->b.as<double>(), nullptr, 0, H.num_sms, st);
  {
    const int blocks = std::max(1, std::min(1024, (H.nc * 32 + AT - 1) / AT));
    amg_coarse_kernel<<<blocks, AT, 0, st>>>(H.nc, H.inv.as<double>(), bvec(nl - 1), xvec(nl - 1));
  }
  for (int l = nl - 2; l >= 0; --l) {                     // x_l = G_l b_l + Q_l x_l+1
    const AmgLevel& L = *H.lv[l];
    rows_launch(&L.G, bvec(l), L.Q, xvec(l + 1), xvec(l), l == 0 ? part : nullptr, l == 0 && part ? nb_part : 0,
                H.num_sms, st);
  }
  if (part && nl == 1) amg_dot_kernel<<<nb_part, AT, 0, st>>>(H.lv[0]->n, r, z, part);
  return amg_launches(H, part != nullptr);
}

}  // namespace obte
