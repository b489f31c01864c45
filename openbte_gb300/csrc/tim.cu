// dkappa_eff / dt for transmission-interface problems (inverse design).
//
// The transmission-interface model (openbte/inverse/bte.py:97-168) lets each internal side s
// transmit a fraction t_s of the inflow from the neighbour; with partial reflection the rest is
// the element's own outgoing flux re-emitted diffusely.  kappa_eff depends on t_s through the
// transport rows and through the contact flux.  Its gradient is d_t kappa - lam . d_t r with the
// adjoint lam of the transport system.  Weighted by V tau, the system equals its transpose with
// every direction reversed (the adjoint sweep of direction q is the sweep of -q in reverse order),
// and the adjoint source dkappa/dX is the forward jump source reversed, so
//
//   lam_mq(c) = k V_c tau_mq X_m,qbar(c),   k = nrm a / jump,   sigma_mq = a tau_mq L_m s_q,
//
// the reference's G = -T[reflection] (openbte/inverse/bte.py:33) for an MFP-resolved material.
// One forward solve therefore gives both fields: the final sweep of the solve stores the
// per-ordinate temperatures X [q][element][m] (FP32), and one kernel evaluates per internal side
//
//   dkappa/dt_s = nrm sum_mq [max(sigma.n_s,0) X(e1) + min(sigma.n_s,0)(X(e2) + alpha)]   (contact sides)
//               - k sum_{f = e1->e2, e2->e1} sum_{q in(f)} (s_q . n_f) sum_m tau_mq L_m X_m,qbar(c_f)
//                                                   (X_mq(j_f) + J_f - R_f)
//
// with R_f the reflected temperature of directed face f (the final sweep's T_B output) and J_f the
// periodic jump seen from f.  The kernel is a per-side reduction over ordinates: one CTA per side,
// threads over (q, m) with m fastest so the reads of X are contiguous.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.h"

namespace obte {

static constexpr int kGradThreads = 128;

__global__ void __launch_bounds__(kGradThreads)
tim_gradient_kernel(const float* __restrict__ X, const float* __restrict__ Xq, const double* __restrict__ TB,
                    int64_t n, int n_dir, int n_mfp,
                    int dim, const double* __restrict__ dirs, const double* __restrict__ tl,
                    const double* __restrict__ sig, const int32_t* __restrict__ refl, int64_t ni,
                    const int32_t* __restrict__ side, const int32_t* __restrict__ e1, const int32_t* __restrict__ e2,
                    const int32_t* __restrict__ w1, const int32_t* __restrict__ w2, const double* __restrict__ na,
                    const double* __restrict__ jump, const int8_t* __restrict__ contact, double nrm, double alpha,
                    double kfac, double* __restrict__ grad) {
  __shared__ double red[2][kGradThreads / 32];
  const int total = n_dir * n_mfp;
  for (int64_t k = blockIdx.x; k < ni; k += gridDim.x) {
    const int64_t c1 = e1[k], c2 = e2[k];
    const double n0 = na[k * dim], n1 = na[k * dim + 1], n2 = dim > 2 ? na[k * dim + 2] : 0.0;
    const double J = jump[k];
    const double R1 = w1[k] >= 0 ? TB[w1[k]] : 0.0;
    const double R2 = w2[k] >= 0 ? TB[w2[k]] : 0.0;
    const bool con = contact[k] != 0;
    double e = 0, phi = 0;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int q = idx / n_mfp, m = idx - q * n_mfp;
      const double* sq = dirs + (int64_t)q * dim;
      const double sn = sq[0] * n0 + sq[1] * n1 + (dim > 2 ? sq[2] * n2 : 0.0);
      const int64_t qb = refl[q];
      const double w = tl[idx];
      if (sn < 0) {          // inflow of the e1 face (outward +n): owner e1, neighbour e2, jump +J
        const double xo = Xq[(qb * n + c1) * n_mfp + m], xn = X[((int64_t)q * n + c2) * n_mfp + m];
        e += sn * w * xo * (xn + J - R1);
      } else if (sn > 0) {   // inflow of the e2 face (outward -n): owner e2, neighbour e1, jump -J
        const double xo = Xq[(qb * n + c2) * n_mfp + m], xn = X[((int64_t)q * n + c1) * n_mfp + m];
        e += -sn * w * xo * (xn - J - R2);
      }
      if (con) {
        const double* sg = sig + (int64_t)idx * dim;
        const double gn = sg[0] * n0 + sg[1] * n1 + (dim > 2 ? sg[2] * n2 : 0.0);
        phi += gn > 0 ? gn * (double)X[((int64_t)q * n + c1) * n_mfp + m]
                      : gn * ((double)X[((int64_t)q * n + c2) * n_mfp + m] + alpha);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      e += __shfl_down_sync(0xffffffffu, e, o);
      phi += __shfl_down_sync(0xffffffffu, phi, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][warp] = e; red[1][warp] = phi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double se = 0, sp = 0;
      for (int i = 0; i < kGradThreads / 32; ++i) { se += red[0][i]; sp += red[1][i]; }
      grad[side[k]] = nrm * sp - kfac * se;
    }
    __syncthreads();
  }
}

// Host checks of the adjoint identity's assumptions, then the device tables.  `paired`: the reversed
// directions live in a separate adjoint plan (ordinate q of that plan is -s_q), so this plan's direction
// set need not be closed under reversal and refl is the identity into the adjoint plan's fields.
static obte_status ensure_tim(obte_plan plan, bool paired) {
  PhaseTimer timer("ensure_tim");
  if (plan->tim && plan->tim->ready && plan->tim->paired != paired) plan->tim.reset();
  if (!plan->tim) plan->tim.reset(new TimDevice());
  TimDevice& T = *plan->tim;
  if (T.ready) return OBTE_OK;
  T.paired = paired;
  const Schedule& s = plan->sched;
  const int dim = s.dim, nq = s.n_dir, nm = s.n_mfp;
  if (s.extra_sources) {
    set_error("gradient: isothermal walls, heat sources and nanowire terms are not supported");
    return OBTE_ERR_UNSUPPORTED;
  }
  // reversal of every direction
  std::vector<int32_t> refl(nq, -1);
  for (int q = 0; q < nq; ++q)
    for (int r = 0; r < nq && refl[q] < 0; ++r) {
      double d = 0;
      for (int k = 0; k < dim; ++k) d = std::max(d, std::fabs(s.dirs[(size_t)q * dim + k] + s.dirs[(size_t)r * dim + k]));
      if (d < 1e-9) refl[q] = r;
    }
  if (paired) {
    for (int q = 0; q < nq; ++q) refl[q] = q;
  } else {
    for (int q = 0; q < nq; ++q)
      if (refl[q] < 0) {
        set_error("gradient: the direction set is not closed under reversal (pass an adjoint plan with the "
                  "reversed directions to obte_bte_kappa_gradient_adjoint)");
        return OBTE_ERR_UNSUPPORTED;
      }
  }
  // tau L and the flux scale a (sigma = a tau L s)
  std::vector<double> tl((size_t)nq * nm), sg((size_t)nq * nm * dim);
  double a = 0;
  for (int q = 0; q < nq; ++q)
    for (int m = 0; m < nm; ++m) {
      const double tau = s.tco[(size_t)q * s.m_pad + m];
      if (!paired && std::fabs(tau - s.tco[(size_t)refl[q] * s.m_pad + m]) > 1e-12 * std::fabs(tau)) {
        set_error("gradient: ordinate weights differ between a direction and its reverse");
        return OBTE_ERR_UNSUPPORTED;
      }
      tl[(size_t)q * nm + m] = tau * s.mfp[m];
      double ss = 0, sn = 0;
      for (int k = 0; k < dim; ++k) {
        const double v = k < s.ds ? s.sig[((size_t)q * s.m_pad + m) * s.ds + k] : 0.0;
        sg[((size_t)q * nm + m) * dim + k] = v;
        ss += v * s.dirs[(size_t)q * dim + k];
        sn += v * v;
      }
      if (tl[(size_t)q * nm + m] > 0) {
        const double aq = ss / tl[(size_t)q * nm + m];
        if (a == 0) a = aq;
        double dev = 0;
        for (int k = 0; k < dim; ++k) {
          const double v = sg[((size_t)q * nm + m) * dim + k] - aq * tl[(size_t)q * nm + m] * s.dirs[(size_t)q * dim + k];
          dev += v * v;
        }
        if (std::fabs(aq - a) > 1e-9 * std::fabs(a) || dev > 1e-18 * std::max(sn, 1e-300)) {
          set_error("gradient: sigma is not proportional to t_coeff x mfp x direction (isotropic materials only)");
          return OBTE_ERR_UNSUPPORTED;
        }
      }
    }
  // the jump source and the contact flux must sit on the same sides
  const int64_t ni = (int64_t)s.tim_side.size();
  double J0 = 0;
  for (int64_t k = 0; k < ni; ++k) {
    if (s.tim_jump[k] != 0 && !s.tim_contact[k]) {
      set_error("gradient: a periodic side with a jump is not a contact side");
      return OBTE_ERR_UNSUPPORTED;
    }
    if (s.tim_contact[k]) {
      if (J0 == 0) J0 = s.tim_jump[k];
      if (s.tim_jump[k] == 0 || std::fabs(s.tim_jump[k] - J0) > 1e-12 * std::fabs(J0)) {
        set_error("gradient: contact sides need one common nonzero periodic jump");
        return OBTE_ERR_UNSUPPORTED;
      }
    }
  }
  if (J0 == 0 || a == 0) { set_error("gradient: no contact side with a periodic jump"); return OBTE_ERR_UNSUPPORTED; }
  T.kfac = s.normalization * a / J0;
  cudaStream_t st = plan->stream;
  std::vector<int8_t> con(s.tim_contact.begin(), s.tim_contact.end());
  OBTE_TRY(upload(T.side, s.tim_side, st));
  OBTE_TRY(upload(T.e1, s.tim_e1, st));
  OBTE_TRY(upload(T.e2, s.tim_e2, st));
  OBTE_TRY(upload(T.w1, s.tim_w1, st));
  OBTE_TRY(upload(T.w2, s.tim_w2, st));
  OBTE_TRY(upload(T.na, s.tim_na, st));
  OBTE_TRY(upload(T.jump, s.tim_jump, st));
  OBTE_TRY(upload(T.contact, con, st));
  OBTE_TRY(upload(T.dirs, s.dirs, st));
  OBTE_TRY(upload(T.tl, tl, st));
  OBTE_TRY(upload(T.sig, sg, st));
  OBTE_TRY(upload(T.refl, refl, st));
  OBTE_TRY(T.xs.alloc((size_t)nq * s.n * nm * sizeof(float)));
  OBTE_TRY(T.K.alloc((size_t)nq * nm * sizeof(double)));
  T.ready = true;
  return OBTE_OK;
}

}  // namespace obte

using namespace obte;

namespace {

// The adjoint plan must be the plan's problem with every direction reversed: same mesh, sides,
// transmissions and contact, ordinate q of `adj` = -s_q with the same weight and MFP and sigma negated.
obte_status check_adjoint_pair(const Schedule& s, const Schedule& a) {
  auto fail = [](const char* what) {
    set_error(std::string("gradient: the adjoint plan is not the plan's problem with reversed directions (") +
              what + ")");
    return OBTE_ERR_BAD_ARG;
  };
  if (!a.tim) return fail("no side transmissions");
  if (a.n != s.n || a.n_sides != s.n_sides || a.dim != s.dim || a.n_dir != s.n_dir || a.n_mfp != s.n_mfp ||
      a.nd != s.nd || a.m_pad != s.m_pad || a.ds != s.ds)
    return fail("sizes");
  if (a.tim_side != s.tim_side || a.tim_e1 != s.tim_e1 || a.tim_e2 != s.tim_e2 || a.tim_contact != s.tim_contact)
    return fail("sides");
  for (size_t k = 0; k < s.tim_jump.size(); ++k)
    if (a.tim_jump[k] != s.tim_jump[k]) return fail("periodic jump");
  for (size_t k = 0; k < s.dsa.t.size(); ++k)
    if (a.dsa.t[k] != s.dsa.t[k]) return fail("transmissions");
  for (size_t i = 0; i < s.dirs.size(); ++i)
    if (std::fabs(a.dirs[i] + s.dirs[i]) > 1e-9) return fail("directions");
  for (int m = 0; m < s.n_mfp; ++m)
    if (a.mfp[m] != s.mfp[m]) return fail("MFPs");
  double ssum[3] = {0, 0, 0}, sabs = 0;
  for (int q = 0; q < s.n_dir; ++q)
    for (int m = 0; m < s.n_mfp; ++m) {
      const double t0 = s.tco[(size_t)q * s.m_pad + m], t1 = a.tco[(size_t)q * a.m_pad + m];
      if (std::fabs(t0 - t1) > 1e-12 * std::fabs(t0)) return fail("ordinate weights");
      for (int d = 0; d < s.ds; ++d) {
        const double v0 = s.sig[((size_t)q * s.m_pad + m) * s.ds + d], v1 = a.sig[((size_t)q * a.m_pad + m) * a.ds + d];
        if (std::fabs(v0 + v1) > 1e-12 * std::fabs(v0) + 1e-300) return fail("sigma");
        if (d < 3) ssum[d] += v0;
        sabs += std::fabs(v0);
      }
    }
  // re-emitting sides normalise their weights by the incoming sigma flux; the reversed problem uses the
  // outgoing one, which is the same only when sum sigma = 0
  if (s.nd > 0)
    for (int d = 0; d < std::min(3, s.ds); ++d)
      if (std::fabs(ssum[d]) > 1e-9 * sabs) {
        set_error("gradient: sum of sigma over the ordinates is not zero (re-emitting sides would not conserve "
                  "energy in the reversed problem)");
        return OBTE_ERR_UNSUPPORTED;
      }
  return OBTE_OK;
}

obte_status gradient_impl(obte_plan plan, obte_plan adj, const obte_solve_opts* opts, const double* dT0,
                          double* grad_t, obte_solve_info* info, obte_solve_info* adj_info) {
  if (!plan || !opts || !dT0 || !grad_t) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (!plan->ctx) { set_error("host-only plan cannot solve"); return OBTE_ERR_BAD_ARG; }
  const Schedule& s = plan->sched;
  if (!s.tim) { set_error("gradient: the plan was created without side transmissions"); return OBTE_ERR_BAD_ARG; }
  if (adj) {
    if (!adj->ctx) { set_error("host-only adjoint plan cannot solve"); return OBTE_ERR_BAD_ARG; }
    if (adj == plan) { set_error("gradient: the adjoint plan is the plan itself"); return OBTE_ERR_BAD_ARG; }
    OBTE_TRY(check_adjoint_pair(s, adj->sched));
    OBTE_TRY(ensure_tim(adj, true));
  }
  OBTE_TRY(ensure_tim(plan, adj != nullptr));
  TimDevice& T = *plan->tim;
  obte_solve_info inf{};
  plan->xstore = T.xs.as<float>();
  const obte_status st = obte_bte_solve(plan, opts, dT0, nullptr, nullptr, T.K.as<double>(), nullptr, &inf);
  plan->xstore = nullptr;
  if (st != OBTE_OK && st != OBTE_ERR_NOT_CONVERGED) return st;
  const float* Xq = T.xs.as<float>();
  obte_status sta = OBTE_OK;
  if (adj) {
    // the adjoint fields: the forward solution of the reversed directions (the transposed sweep of every
    // direction, which visits its elements in reverse order), on the adjoint plan's own stream
    TimDevice& A = *adj->tim;
    obte_solve_info ainf{};
    OBTE_CUDA(wait_stream(plan->stream));
    adj->xstore = A.xs.as<float>();
    sta = obte_bte_solve(adj, opts, dT0, nullptr, nullptr, A.K.as<double>(), nullptr, &ainf);
    adj->xstore = nullptr;
    if (sta != OBTE_OK && sta != OBTE_ERR_NOT_CONVERGED) return sta;
    OBTE_CUDA(wait_stream(adj->stream));
    Xq = A.xs.as<float>();
    if (adj_info) *adj_info = ainf;
  }
  cudaStream_t stream = plan->stream;
  OBTE_CUDA(cudaMemsetAsync(grad_t, 0, (size_t)s.n_sides * sizeof(double), stream));
  const int64_t ni = (int64_t)s.tim_side.size();
  if (ni > 0) {
    const int blocks = (int)std::min<int64_t>(ni, (int64_t)plan->ctx->num_sms * 16);
    const double* TB = plan->work->Fu.as<double>() + s.n;   // reflected temperatures of the final sweep
    tim_gradient_kernel<<<blocks, kGradThreads, 0, stream>>>(
        T.xs.as<float>(), Xq, TB, s.n, s.n_dir, s.n_mfp, s.dim, T.dirs.as<double>(), T.tl.as<double>(),
        T.sig.as<double>(), T.refl.as<int32_t>(), ni, T.side.as<int32_t>(), T.e1.as<int32_t>(), T.e2.as<int32_t>(),
        T.w1.as<int32_t>(), T.w2.as<int32_t>(), T.na.as<double>(), T.jump.as<double>(), T.contact.as<int8_t>(),
        s.normalization, s.contact_alpha, T.kfac, grad_t);
    count_launch();
    OBTE_CUDA(cudaGetLastError());
  }
  OBTE_CUDA(cudaStreamSynchronize(stream));
  if (info) *info = inf;
  return st != OBTE_OK ? st : sta;
}

}  // namespace

extern "C" obte_status obte_bte_kappa_gradient(obte_plan plan, const obte_solve_opts* opts, const double* dT0,
                                               double* grad_t, obte_solve_info* info) {
  return gradient_impl(plan, nullptr, opts, dT0, grad_t, info, nullptr);
}

extern "C" obte_status obte_bte_kappa_gradient_adjoint(obte_plan plan, obte_plan adjoint_plan,
                                                       const obte_solve_opts* opts, const double* dT0,
                                                       double* grad_t, obte_solve_info* info,
                                                       obte_solve_info* adjoint_info) {
  return gradient_impl(plan, adjoint_plan, opts, dT0, grad_t, info, adjoint_info);
}
