// Diffusion-synthetic acceleration (DSA) of the GMRES on the sweep fixed point.
//
// The reference iterates the source step dT <- sum_mq t_coeff T_mq(dT) plainly (openbte/bte.py:193-249);
// where the transport is diffusive at the scale of the slow error — temperatures relaxing across a
// network of partially transmitting interfaces (openbte/inverse/bte.py:145-163), or through many mean
// free paths — each step removes only a small part of a smooth error and the iteration count grows
// with the size of the cell.  For a smooth temperature error e the transport operator acts as a
// diffusion operator: with T_mq = (1 + F_mq . grad)^-1 e ~ e - F . grad e + (F . grad)^2 e and
// sum_mq t_mq = 1, sum_mq t_mq F_mq = 0,
//     (I - K) e = div(sum_mq t_mq F_mq T_mq) ~ -div(D grad e),   D = sum_mq t_mq F_mq F_mq^T,
// F_mq = mfp_m v_q.  The right preconditioner M^-1 = I + E L^-1 R adds to a GMRES direction v the
// solution of the diffusion problem whose source is v's temperature part: R takes the temperature
// entries weighted by the element volumes, L is the finite-volume diffusion operator on the elements,
// E adds the cell correction to the temperatures, to the wall temperatures of each wall's element and to
// the periodic inflow of each source slot's element (a smooth correction shifts them alike).
//
// L (symmetric, volume-weighted): per internal side k between elements i, j, with area A and centre
// distance d, the conductance
//     A sum_m 1 / (d / D_m + (1 - t_k) / (G_m t_k))
// in series per MFP m: the bulk D_m = sum_q t_mq mfp_m^2 |v_q|^2 / dim and, on a side that transmits the
// fraction t < 1 of the phonons, the interface conductance G_m t / (1 - t), G_m = sum_q t_mq
// max(F_mq . n, 0) (the half-range flux; two-stream balance of the transmitted and reflected streams at
// the interface).  Periodic sides couple their elements like internal ones (the correction carries no
// jump); diffuse walls are insulating; isothermal walls hold the correction at zero through
// A sum_m 1 / (d / D_m + 1 / (2 G_m)).  No diagonal is below 5 % of the (upper) median (per volume): an element
// whose sides barely transmit keeps its slow mode to GMRES.  Without isothermal walls L has the constant
// null vector, as I - K has the uniform shift: the source is projected onto zero mean and the
// correction's volume-weighted mean removed, and a diagonal of 1e-6 of the largest keeps the hierarchy's
// coarsest operator invertible.
//
// The solve is `cycles` (OBTE_DSA_CYCLES, default 1) steps of d <- d + B (b - L d) from d = 0 with B one
// V-cycle of the smoothed-aggregation hierarchy of amg.cu: a fixed linear map, as the non-flexible GMRES
// requires of its preconditioner (on the 128^2-pixel design problem, 50 MFPs x 64 directions: 210 sweeps per
// gradient evaluation without it, 89 / 88 / 88 with 1 / 2 / 3 cycles).  The operator is built on the plan's
// first accelerated solve and rebuilt after new side transmissions.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "internal.h"

namespace obte {

namespace {

constexpr int DT = 256;

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) red[0] = v;
  __syncthreads();
  return red[0];
}

// part[block] = sum over the block's grid-stride range of V x (fixed order)
__global__ void dsa_partial_kernel(int64_t n, const double* __restrict__ vol, const double* __restrict__ x,
                                   double* __restrict__ part) {
  __shared__ double red[32];
  double s = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += vol[i] * x[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// sum of the np partials, the same value (same order) in every block
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int np, double* red) {
  double s = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  return block_sum(s, red);
}

// b = V in[0:n], minus V times the volume-weighted mean of in when `part` (the partials of V in) is given
__global__ void dsa_restrict_kernel(int64_t n, const double* __restrict__ vol, double inv_vol_sum,
                                    const double* __restrict__ part, int np, const double* __restrict__ in,
                                    double* __restrict__ b) {
  __shared__ double red[32];
  const double mu = part ? sum_partials(part, np, red) * inv_vol_sum : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = vol[i] * (in[i] - mu);
}

// r = b - L d (CSR, one thread per row)
__global__ void dsa_residual_kernel(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                    const double* __restrict__ val, const double* __restrict__ b,
                                    const double* __restrict__ d, double* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x; i < n; i += (int64_t)gridDim.x * DT) {
    double acc = b[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc -= val[k] * d[ci[k]];
    r[i] = acc;
  }
}

__global__ void dsa_axpy_kernel(int64_t n, const double* __restrict__ e, double* __restrict__ d) {
  for (int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x; i < n; i += (int64_t)gridDim.x * DT) d[i] += e[i];
}

// out[i] += d[cell(i)] - mean over the state: temperatures, wall temperatures (element of the wall),
// periodic inflow (element of the source slot, every MFP); the mean is the volume-weighted one of d from its
// partials (or 0 without them)
__global__ void dsa_extend_kernel(int64_t n, int64_t nd, int64_t nu, int n_mfp, const int32_t* __restrict__ wcell,
                                  const int32_t* __restrict__ xcell, const double* __restrict__ d,
                                  const double* __restrict__ part, int np, double inv_vol_sum,
                                  double* __restrict__ out) {
  __shared__ double red[32];
  const double mu = part ? sum_partials(part, np, red) * inv_vol_sum : 0.0;
  const int64_t xoff = n + nd;
  for (int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x; i < nu; i += (int64_t)gridDim.x * DT) {
    const int64_t c = i < n ? i : i < xoff ? (int64_t)wcell[i - n] : (int64_t)xcell[(i - xoff) / n_mfp];
    out[i] += d[c] - mu;
  }
}

int grid_for(int64_t n, int num_sms) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + DT - 1) / DT, (int64_t)num_sms * 8));
}

}  // namespace

bool dsa_default(const Schedule& s) {
  // on where a side transmits only part of the phonons (the transmission-interface model): the slow
  // modes there are interface-network diffusion modes
  for (double t : s.dsa.t)
    if (t < 1.0) return true;
  return false;
}

// L as CSR (columns sorted, duplicates merged); `project`: L has the constant null vector
void dsa_matrix(const Schedule& s, std::vector<int32_t>& rp, std::vector<int32_t>& ci, std::vector<double>& val,
                bool& project) {
  const Schedule::DsaData& D = s.dsa;
  const int64_t n = s.n;
  const int n_mfp = s.n_mfp;
  double Dsum = 0;
  for (double v : D.Dm) Dsum += v;
  // conductances of the sides
  const int64_t nfc = (int64_t)D.e1.size();
  std::vector<double> coef(nfc, 0.0);
  parallel_for(nfc, [&](int64_t k) {
    const double t = D.t[k];
    double c = 0;
    if (t >= 1.0) {
      c = Dsum / D.dist[k];
    } else {
      for (int m = 0; m < n_mfp; ++m) {
        const double r = D.dist[k] / D.Dm[m] + (1.0 - t) / (D.Gm[m] * t);
        if (r > 0 && std::isfinite(r)) c += 1.0 / r;
      }
    }
    coef[k] = D.area[k] * c;
  });
  std::vector<double> diag(n, 0.0);
  std::vector<int32_t> deg(n + 1, 0);
  for (int64_t k = 0; k < nfc; ++k) {
    if (D.e1[k] == D.e2[k]) continue;
    diag[D.e1[k]] += coef[k];
    diag[D.e2[k]] += coef[k];
    ++deg[D.e1[k] + 1];
    ++deg[D.e2[k] + 1];
  }
  for (size_t k = 0; k < D.iso_cell.size(); ++k) {
    double c = 0;
    for (int m = 0; m < n_mfp; ++m) c += 1.0 / (D.iso_dist[k] / D.Dm[m] + 0.5 / D.Gm[m]);
    diag[D.iso_cell[k]] += D.iso_area[k] * c;
  }
  project = D.iso_cell.empty();
  double dmax = 0;
  for (double v : diag) dmax = std::max(dmax, v);
  const double reg = 1e-6 * (dmax > 0 ? dmax : 1.0);
  // an element whose sides barely transmit (a pore pixel, t ~ 1e-12) has a temperature mode that I - K
  // relaxes at a rate ~t: the diffusion operator models that rate, but inverting it would multiply the
  // rounding noise of the FP32 sweeps in that element by ~1 / t.  Its diagonal is raised to 5 % of the
  // median, so the correction leaves such modes to GMRES as if there were no acceleration.
  {
    std::vector<double> dd;
    dd.reserve(n);
    for (int64_t i = 0; i < n; ++i) dd.push_back(diag[i] / D.vol[i]);
    std::nth_element(dd.begin(), dd.begin() + n / 2, dd.end());
    const double floor_per_vol = 0.05 * dd[n / 2];
    for (int64_t i = 0; i < n; ++i) diag[i] = std::max(diag[i], floor_per_vol * D.vol[i]);
  }
  // CSR: diagonal first, then the neighbours in side order; two sides joining the same pair (periodic
  // images) stay separate entries
  rp.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) rp[i + 1] = rp[i] + 1 + deg[i + 1];
  ci.assign(rp[n], 0);
  val.assign(rp[n], 0.0);
  std::vector<int32_t> pos(rp.begin(), rp.end() - 1);
  for (int64_t i = 0; i < n; ++i) {
    ci[pos[i]] = (int32_t)i;
    val[pos[i]++] = diag[i] + reg;
  }
  for (int64_t k = 0; k < nfc; ++k) {
    const int32_t i = D.e1[k], j = D.e2[k];
    if (i == j) continue;
    ci[pos[i]] = j; val[pos[i]++] = -coef[k];
    ci[pos[j]] = i; val[pos[j]++] = -coef[k];
  }
  // the hierarchy wants sorted columns with duplicates merged
  {
    std::vector<int32_t> rp2(n + 1, 0), ci2;
    std::vector<double> val2;
    ci2.reserve(ci.size());
    val2.reserve(val.size());
    std::vector<std::pair<int32_t, double>> row;
    for (int64_t i = 0; i < n; ++i) {
      row.clear();
      for (int32_t k = rp[i]; k < rp[i + 1]; ++k) row.emplace_back(ci[k], val[k]);
      std::sort(row.begin(), row.end(), [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& b) {
        return a.first < b.first;
      });
      for (size_t k = 0; k < row.size(); ++k) {
        if (!ci2.empty() && (int64_t)ci2.size() > rp2[i] && ci2.back() == row[k].first) {
          val2.back() += row[k].second;
        } else {
          ci2.push_back(row[k].first);
          val2.push_back(row[k].second);
        }
      }
      rp2[i + 1] = (int32_t)ci2.size();
    }
    rp.swap(rp2);
    ci.swap(ci2);
    val.swap(val2);
  }
}

obte_status ensure_dsa(obte_plan plan) {
  if (plan->dsa) return OBTE_OK;
  PhaseTimer timer("dsa setup");
  const auto t0 = std::chrono::steady_clock::now();
  const Schedule& s = plan->sched;
  const Schedule::DsaData& D = s.dsa;
  const int64_t n = s.n;
  const int64_t nfc = (int64_t)D.e1.size();
  std::vector<int32_t> rp, ci;
  std::vector<double> val;
  bool project = true;
  dsa_matrix(s, rp, ci, val, project);
  std::unique_ptr<DsaOp> op(new DsaOp());
  cudaStream_t st = plan->stream;
  // rebuilt for every density field of a design loop: coarsen down to 64 rows, whose dense inverse costs
  // little (on 128^2 pixels the hierarchy's set-up took 16.5 ms with the default 400-row coarsest
  // operator, 6.8 ms with 64 rows, for one more sweep per solve)
  OBTE_TRY(amg_build(n, rp, ci, val, -1, plan->ctx->num_sms, st, op->amg, 64));
  OBTE_TRY(upload(op->rp, rp, st));
  OBTE_TRY(upload(op->ci, ci, st));
  OBTE_TRY(upload(op->val, val, st));
  OBTE_TRY(upload(op->vol, D.vol, st));
  for (DevBuf* b : {&op->b, &op->d, &op->r, &op->e}) OBTE_TRY(b->alloc((size_t)n * sizeof(double)));
  OBTE_TRY(op->mean.alloc((size_t)grid_for(n, plan->ctx->num_sms) * sizeof(double)));   // partial sums
  double vs = 0;
  for (double v : D.vol) vs += v;
  op->inv_vol_sum = vs > 0 ? 1.0 / vs : 0.0;
  op->project = project;
  if (const char* e = std::getenv("OBTE_DSA_CYCLES")) op->cycles = std::max(1, std::min(16, std::atoi(e)));
  op->levels = amg_levels(*op->amg);
  op->bytes = (int64_t)(op->rp.bytes + op->ci.bytes + op->val.bytes + op->vol.bytes + 4 * n * sizeof(double));
  OBTE_CUDA(wait_stream(st));
  op->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (timer.on)
    std::fprintf(stderr, "[obte trace] dsa: %lld elements, %lld sides, %d levels, %d cycles per apply\n",
                 (long long)n, (long long)nfc, op->levels, op->cycles);
  plan->dsa = std::move(op);
  return OBTE_OK;
}

void dsa_start_async(obte_plan plan) {
  dsa_join(plan);
  if (!plan->ctx || !dsa_default(plan->sched)) return;
  plan->dsa.reset();
  plan->dsa_build_status = OBTE_OK;
  const int device = plan->ctx->device;
  plan->dsa_build = std::thread([plan, device] {
    if (cudaSetDevice(device) != cudaSuccess) {
      plan->dsa_build_status = OBTE_ERR_CUDA;
      return;
    }
    plan->dsa_build_status = ensure_dsa(plan);
  });
}

obte_status dsa_join(obte_plan plan) {
  if (plan->dsa_build.joinable()) plan->dsa_build.join();
  const obte_status st = plan->dsa_build_status;
  plan->dsa_build_status = OBTE_OK;
  if (st != OBTE_OK) plan->dsa.reset();      // a failed build is redone (with its message) by the solve
  return st;
}

void dsa_add(obte_plan plan, const double* in, double* out) {
  DsaOp& op = *plan->dsa;
  const Schedule& s = plan->sched;
  const int64_t n = s.n;
  cudaStream_t st = plan->stream;
  const int num_sms = plan->ctx->num_sms;
  const int gn = grid_for(n, num_sms);
  double* b = op.b.as<double>();
  double* d = op.d.as<double>();
  double* part = op.mean.as<double>();          // partial sums, one per block of the n-element grid
  if (op.project) {
    dsa_partial_kernel<<<gn, DT, 0, st>>>(n, op.vol.as<double>(), in, part);
    count_launch();
  }
  dsa_restrict_kernel<<<gn, DT, 0, st>>>(n, op.vol.as<double>(), op.inv_vol_sum, op.project ? part : nullptr, gn,
                                         in, b);
  count_launch();
  count_launch(amg_apply(*op.amg, b, d, nullptr, 0, st));
  for (int c = 1; c < op.cycles; ++c) {
    dsa_residual_kernel<<<gn, DT, 0, st>>>(n, op.rp.as<int32_t>(), op.ci.as<int32_t>(), op.val.as<double>(), b, d,
                                           op.r.as<double>());
    count_launch(amg_apply(*op.amg, op.r.as<double>(), op.e.as<double>(), nullptr, 0, st));
    dsa_axpy_kernel<<<gn, DT, 0, st>>>(n, op.e.as<double>(), d);
    count_launch(2);
  }
  if (op.project) {
    dsa_partial_kernel<<<gn, DT, 0, st>>>(n, op.vol.as<double>(), d, part);
    count_launch();
  }
  dsa_extend_kernel<<<grid_for(plan->nu, num_sms), DT, 0, st>>>(
      n, s.nd, plan->nu, s.n_mfp, plan->diffuse_cell.as<int32_t>(), plan->x_cell.as<int32_t>(), d,
      op.project ? part : nullptr, gn, op.inv_vol_sum, out);
  count_launch();
}

}  // namespace obte

using namespace obte;

extern "C" obte_status obte_bte_dsa_operator(obte_plan plan, int64_t* nnz, int32_t* row_ptr, int32_t* col,
                                             double* val, int32_t* project) {
  if (!plan || !nnz) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  std::vector<int32_t> rp, ci;
  std::vector<double> v;
  bool proj = true;
  dsa_matrix(plan->sched, rp, ci, v, proj);
  const int64_t cap = *nnz;
  *nnz = (int64_t)ci.size();
  if (project) *project = proj ? 1 : 0;
  if (!row_ptr && !col && !val) return OBTE_OK;          // size query
  if (cap < (int64_t)ci.size()) { set_error("dsa operator: arrays too small"); return OBTE_ERR_BAD_ARG; }
  if (row_ptr) std::copy(rp.begin(), rp.end(), row_ptr);
  if (col) std::copy(ci.begin(), ci.end(), col);
  if (val) std::copy(v.begin(), v.end(), val);
  return OBTE_OK;
}
