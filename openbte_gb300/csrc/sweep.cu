// Batched upwind transport sweep for sm_103a.
//
// One CTA = one direction q x one chunk of MCP mean free paths.  The CTA walks
// the direction's elements level by level (longest-path layers of the upwind
// DAG with periodic inflow cut, split into units of at most 128 elements);
// within a unit every thread owns one element and loops over the chunk's MFPs:
//
//   T_mq[c] = (b[c] + L_m (p[c] - sum_in g_f T_up,m)) / (1 + L_m D_q[c])
//
// the row of A_mq T = B of openbte/bte.py:183-218 for an element whose upwind
// neighbours are known; b = DeltaT + heat source, p = perturbation minus the
// wall inflow g_w T_B (openbte/bte.py:200,211-214).
//
// T_up lives in a ring of shared-memory rows, one per live upstream element
// and one column per MFP (row-major by MFP).  Extra rows: a zero row for absent
// faces, a trash row for elements nobody reads, and two banks of rows for the
// inflow across cut periodic faces: while unit u runs, its threads load the
// periodic source values unit u+1 reads from the state vector and store them
// into bank (u+1) & 1, so inflow across a cut face is an ordinary row read and
// the ring does not grow with the number of periodic sources (3D meshes have
// thousands per direction).  The MFP loop is therefore branch-free; elements
// with per-MFP outputs (periodic source, wall re-emission, contact) read their
// T back from their row afterwards.
//
// Data movement per unit: the packed element records, the per-sweep values
// (b, p), the wall re-emission weights of the unit's wall entries and the
// periodic prefetch list of the next unit arrive in shared memory by TMA bulk
// copies (cp.async.bulk + mbarrier) issued two units ahead.  T never goes to
// HBM.  Reductions of
// openbte/bte.py:222-243 are register accumulations over the MFP loop followed
// by one FP64 atomic per element (DeltaT', T_B', J) or per MFP (K, S).
// Every mbarrier wait is bounded; on timeout the CTA raises the device error
// word, stops using the buffers, waits (bounded) for its copies in flight and
// leaves at the next block-wide barrier.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>

#include "internal.h"

namespace obte {

static constexpr int kUnit = 128;      // elements per level unit = threads per CTA

// ---- packed element records -------------------------------------------------------
// 32-bit words, ring rows in 16-bit halves:
//   w0 cell | w1 so, s0 | w2 s1, s2 | w3 s3, sp | the reals c0 .. c(NF-1), D | padding to 16 B
// so = output row, s* = inflow rows (s3 only for NF = 4), sp = 1 + index of the element's output entry
// among its unit's entries (0: no per-MFP outputs).  Triangles: 32 B (FP32) / 48 B (FP64);
// tetrahedra: 48 B / 64 B.  Output entries (int4: periodic source index xk, wall re-emission entries
// (begin << 3 | count, begin relative to the direction), contact entry, 0) are a separate per-unit table.
__host__ __device__ constexpr int rec_words(int real_bytes, int nf) {
  return ((4 + (nf + 1) * (real_bytes / 4)) + 3) & ~3;
}
template <typename Real, int NF> struct Rec {
  static constexpr int CSTEP = sizeof(Real) / 4, COEF = 4, D = COEF + NF * CSTEP;
  static constexpr int W = rec_words(sizeof(Real), NF);
};

// special-element table
//   si: xk wout contact nwall w0 w1 w2 pad     (8 ints)
//   sr: wc0 wc1 wc2 pad                          (4 reals)
static constexpr int SI = 8, SR = 4;

// Level units: each level of direction q split into runs of at most kUnit elements, and cut so that no
// unit holds more than kUnitPf cut periodic inflow faces or kUnitSx output entries.  The per-unit
// staging areas and the two periodic banks of the ring are sized by the largest unit; without the caps
// the few units on the periodic boundaries (up to ~110 cut faces and outputs each on the 60k-triangle
// cell) set them, and the extra ~5 KB cost a CTA per SM (4 instead of 5 at 8 MFPs per lane).  A cap only
// applies when at most 1 % of the uncapped units exceed it: where most units are over it (the pixel
// model, where every element has reflecting-wall outputs) it would split every unit and lengthen every
// chain instead.
constexpr int kUnitPf = 48;
constexpr int kUnitSx = 64;
struct Units {
  std::vector<int32_t> ptr;   // per direction: n[q] + 1 positions (relative to the direction)
  std::vector<int64_t> off;   // [n_dir] first entry of direction q in ptr (and in kpf, kwo)
  std::vector<int32_t> n;     // [n_dir] units of direction q
};

static void build_units_capped(const Schedule& s, int cap_pf, int cap_sx, Units& un, int64_t* over_pf,
                               int64_t* over_sx) {
  // directions in parallel into their own lists, concatenated in direction order
  std::vector<std::vector<int32_t>> per(s.n_dir);
  std::vector<int64_t> opf(s.n_dir, 0), osx(s.n_dir, 0);
  parallel_tasks(s.n_dir, [&](int64_t qq) {
    const int q = (int)qq;
    std::vector<int32_t>& ptr = per[q];
    const int32_t* lp = s.lev_ptr.data() + s.lev_off[q];
    ptr.push_back(0);
    for (int Lv = 0; Lv < s.nlev[q]; ++Lv) {
      int cnt = 0, npf = 0, nsx = 0;
      auto close = [&](int32_t end) {
        ptr.push_back(end);
        if (npf > kUnitPf) ++opf[q];
        if (nsx > kUnitSx) ++osx[q];
        cnt = npf = nsx = 0;
      };
      for (int32_t pos = lp[Lv]; pos < lp[Lv + 1]; ++pos) {
        const size_t it = (size_t)q * s.n + pos;
        int pf = 0;
        for (int f = 0; f < s.nf; ++f)
          if ((int)((uint32_t)s.in_idx[it * s.nf + f] >> ITEM_SHIFT) == ITEM_PERIODIC) ++pf;
        const int sx = (s.xk[it] >= 0 || s.wout[it] != 0 || s.contact[it] >= 0) ? 1 : 0;
        if (cnt > 0 && (cnt == kUnit || npf + pf > cap_pf || nsx + sx > cap_sx)) close(pos);
        ++cnt;
        npf += pf;
        nsx += sx;
      }
      if (cnt > 0) close(lp[Lv + 1]);
    }
  });
  un.ptr.clear();
  un.off.assign(s.n_dir, 0);
  un.n.assign(s.n_dir, 0);
  size_t total = 0;
  for (int q = 0; q < s.n_dir; ++q) total += per[q].size();
  un.ptr.reserve(total);
  for (int q = 0; q < s.n_dir; ++q) {
    un.off[q] = (int64_t)un.ptr.size();
    un.n[q] = (int32_t)per[q].size() - 1;
    un.ptr.insert(un.ptr.end(), per[q].begin(), per[q].end());
  }
  if (over_pf) *over_pf = std::accumulate(opf.begin(), opf.end(), (int64_t)0);
  if (over_sx) *over_sx = std::accumulate(osx.begin(), osx.end(), (int64_t)0);
}

static void build_units(const Schedule& s, Units& un) {
  constexpr int kNone = 1 << 30;
  int64_t over_pf = 0, over_sx = 0;
  build_units_capped(s, kNone, kNone, un, &over_pf, &over_sx);
  const int64_t units = (int64_t)un.ptr.size() - s.n_dir;
  const int cap_pf = over_pf * 100 <= units ? kUnitPf : kNone;
  const int cap_sx = over_sx * 100 <= units ? kUnitSx : kNone;
  if (cap_pf != kNone || cap_sx != kNone) build_units_capped(s, cap_pf, cap_sx, un, nullptr, nullptr);
}

struct Packed {
  RawVec<int32_t> rec, cellmap, spec;   // one entry per item, every one written by pass 2
  RawVec<double> P;
  std::vector<int32_t> si;
  std::vector<double> sr;
  // periodic inflow prefetch: the source indices read by unit u (one entry per cut inflow face, in
  // element then face order), each unit's list padded with -1 to a multiple of 4 ints; kpf[u] is the
  // absolute start of unit u's list (n[q] + 1 entries per direction, indexed like Units::ptr)
  std::vector<int32_t> pf, kpf;
  std::vector<int32_t> sx, ksx;  // output entries (4 ints each) in sweep order; first entry of unit u
  int unit_sx = 0;               // most output entries in one unit
  std::vector<int32_t> kwo;   // first wall re-emission entry of unit u, relative to the direction
  int emax = 0;               // most cut inflow faces in one unit
  int pf_pad = 0;             // longest padded list
  int unit_wo = 0;            // most wall re-emission entries in one unit
  int rows = 0;               // ring rows
};

static int ring_rows(const Schedule& s, int emax) { return s.max_slots + 2 + 2 * emax; }

// Ring rows: [0, S) slots, S zero row, S+1 trash row, then two banks of emax rows that alternate
// by unit parity: the cut inflow values of unit u live in bank u & 1, written during unit u - 1
// (at CTA start for unit 0) from the state vector.
template <typename Real>
static obte_status pack(const Schedule& s, const Units& un, Packed& pk) {
  const int W = rec_words(sizeof(Real), s.nf);
  constexpr int CSTEP = sizeof(Real) / 4, COEF = 4;
  const int S = s.max_slots;
  const int zero_row = S, trash_row = S + 1, prow0 = S + 2;
  // pass 1: per-unit counts of cut inflow faces, wall re-emission entries and output entries, in parallel
  // over directions; per-unit starts are running sums within the direction (kwo) or over the directions
  // in order (kpf, ksx), so the direction totals are summed in order between the two parallel steps
  pk.emax = pk.pf_pad = pk.unit_wo = pk.unit_sx = 0;
  pk.kwo.assign(un.ptr.size(), 0);
  pk.kpf.assign(un.ptr.size(), 0);
  pk.ksx.assign(un.ptr.size(), 0);
  std::vector<int64_t> pf_tot(s.n_dir + 1, 0), sx_tot(s.n_dir + 1, 0);
  std::vector<int> emax_q(s.n_dir, 0), pfpad_q(s.n_dir, 0), uwo_q(s.n_dir, 0), usx_q(s.n_dir, 0);
  std::vector<char> wo_bad(s.n_dir, 0);
  parallel_tasks(s.n_dir, [&](int64_t qq) {
    const int q = (int)qq;
    const int32_t* up = un.ptr.data() + un.off[q];
    int32_t wo_run = 0;
    int64_t pf_run = 0, sx_run = 0;
    for (int u = 0; u < un.n[q]; ++u) {
      int cnt = 0, wcnt = 0, scnt = 0;
      for (int32_t pos = up[u]; pos < up[u + 1]; ++pos) {
        const size_t it = (size_t)q * s.n + pos;
        for (int f = 0; f < s.nf; ++f)
          if ((int)((uint32_t)s.in_idx[it * s.nf + f] >> ITEM_SHIFT) == ITEM_PERIODIC) ++cnt;
        wcnt += s.wout[it] & 7;
        scnt += (s.xk[it] >= 0 || s.wout[it] != 0 || s.contact[it] >= 0) ? 1 : 0;
      }
      const int padded = (cnt + 3) & ~3;
      pk.kwo[un.off[q] + u] = wo_run;
      pk.kpf[un.off[q] + u] = (int32_t)pf_run;   // relative here, made absolute below
      pk.ksx[un.off[q] + u] = (int32_t)sx_run;
      sx_run += scnt;
      usx_q[q] = std::max(usx_q[q], scnt);
      wo_run += wcnt;
      pf_run += padded;
      emax_q[q] = std::max(emax_q[q], cnt);
      pfpad_q[q] = std::max(pfpad_q[q], padded);
      uwo_q[q] = std::max(uwo_q[q], wcnt);
    }
    pk.kwo[un.off[q] + un.n[q]] = wo_run;
    pk.kpf[un.off[q] + un.n[q]] = (int32_t)pf_run;
    pk.ksx[un.off[q] + un.n[q]] = (int32_t)sx_run;
    pf_tot[q + 1] = pf_run;
    sx_tot[q + 1] = sx_run;
    wo_bad[q] = wo_run != s.wo_off[q + 1] - s.wo_off[q];
  });
  for (int q = 0; q < s.n_dir; ++q) {
    if (wo_bad[q]) {
      set_error("wall re-emission entries are not in sweep order");
      return OBTE_ERR_BAD_ARG;
    }
    pf_tot[q + 1] += pf_tot[q];
    sx_tot[q + 1] += sx_tot[q];
    pk.emax = std::max(pk.emax, emax_q[q]);
    pk.pf_pad = std::max(pk.pf_pad, pfpad_q[q]);
    pk.unit_wo = std::max(pk.unit_wo, uwo_q[q]);
    pk.unit_sx = std::max(pk.unit_sx, usx_q[q]);
  }
  const int64_t n_pf = pf_tot[s.n_dir], n_sx = sx_tot[s.n_dir];
  if (n_pf >= (int64_t)1 << 31 || n_sx >= (int64_t)1 << 31) {
    set_error("too many periodic inflow faces or output entries"); return OBTE_ERR_UNSUPPORTED;
  }
  parallel_tasks(s.n_dir, [&](int64_t q) {
    for (int u = 0; u <= un.n[q]; ++u) {
      pk.kpf[un.off[q] + u] += (int32_t)pf_tot[q];
      pk.ksx[un.off[q] + u] += (int32_t)sx_tot[q];
    }
  });
  pk.sx.assign((size_t)std::max<int64_t>(n_sx, 1) * 4, 0);
  pk.rows = ring_rows(s, pk.emax);
  if (pk.rows >= 65535 || s.max_src >= (1 << 30)) {
    set_error("sweep ring rows do not fit 16-bit indices");
    return OBTE_ERR_UNSUPPORTED;
  }
  pk.pf.assign((size_t)n_pf, -1);
  const size_t total = (size_t)s.n_dir * s.n;
  pk.rec.resize(total * W);     // uninitialised: pass 2 writes every word of every record
  pk.cellmap.resize(total);
  pk.spec.resize(total);
  pk.P.resize(total);
  pk.si.clear();
  pk.sr.clear();
  // pass 2: records, in parallel over directions.  Elements with outputs or wall inflow get a "special"
  // entry (si/sr); a first sweep counts them per direction so every direction writes its own range.
  auto is_special = [&](size_t it) {
    if (s.xk[it] >= 0 || s.wout[it] != 0 || s.contact[it] >= 0) return true;
    for (int f = 0; f < s.nf; ++f)
      if ((int)((uint32_t)s.in_idx[it * s.nf + f] >> ITEM_SHIFT) == ITEM_WALL) return true;
    return false;
  };
  std::vector<int64_t> spec_base(s.n_dir + 1, 0);
  parallel_tasks(s.n_dir, [&](int64_t q) {
    int64_t c = 0;
    for (int64_t pos = 0; pos < s.n; ++pos) c += is_special((size_t)q * s.n + pos) ? 1 : 0;
    spec_base[q + 1] = c;
  });
  for (int q = 0; q < s.n_dir; ++q) spec_base[q + 1] += spec_base[q];
  pk.si.assign((size_t)spec_base[s.n_dir] * SI, 0);
  pk.sr.assign((size_t)spec_base[s.n_dir] * SR, 0.0);
  std::vector<int> dir_err(s.n_dir, 0);   // 1: outputs without a ring slot, 2: more than three wall inflows
  parallel_tasks(s.n_dir, [&](int64_t qq) {
    const int q = (int)qq;
    int64_t nsp = spec_base[q];
    const int32_t* up = un.ptr.data() + un.off[q];
    for (int u = 0; u < un.n[q]; ++u) {
      int ent = 0, sent = 0;
      const int bank = prow0 + (u & 1) * pk.emax;
      int32_t* plist = pk.pf.data() + pk.kpf[un.off[q] + u];
      int32_t* slist = pk.sx.data() + (size_t)pk.ksx[un.off[q] + u] * 4;
      for (int32_t pos = up[u]; pos < up[u + 1]; ++pos) {
        const size_t it = (size_t)q * s.n + pos;
        int32_t* r = pk.rec.data() + it * W;
        const int32_t so = s.slot[it] >= 0 ? s.slot[it] : trash_row;
        r[0] = s.cell[it];
        pk.cellmap[it] = s.cell[it];
        pk.P[it] = s.P[it];
        int32_t si[SI] = {s.xk[it], s.wout[it], s.contact[it], 0, 0, 0, 0, 0};
        double sr[SR] = {0, 0, 0, 0};
        const bool outputs = s.xk[it] >= 0 || s.wout[it] != 0 || s.contact[it] >= 0;
        if (outputs && s.slot[it] < 0) { dir_err[q] = 1; return; }
        bool special = outputs;
        double coef[4] = {0, 0, 0, 0};
        int32_t row_in[4] = {zero_row, zero_row, zero_row, zero_row};
        int k = 0;
        for (int f = 0; f < s.nf; ++f) {
          const int32_t code = s.in_idx[it * s.nf + f];
          const int kind = (int)((uint32_t)code >> ITEM_SHIFT);
          const int32_t idx = code & ITEM_MASK;
          const double g = s.in_coef[it * s.nf + f];
          if (kind == ITEM_CELL || kind == ITEM_PERIODIC) {
            if (kind == ITEM_CELL) {
              row_in[k] = idx;
            } else {
              plist[ent] = idx;
              row_in[k] = bank + ent;
              ++ent;
            }
            coef[k] = g;
            ++k;
          } else if (kind == ITEM_WALL) {
            if (si[3] >= 3) { dir_err[q] = 2; return; }
            si[4 + si[3]] = idx;
            sr[si[3]] = g;
            si[3]++;
            special = true;
          }
        }
        int sp = 0;
        if (outputs) {
          // wall re-emission entries: begin relative to the direction's first entry
          int32_t* e = slist + (size_t)sent * 4;
          e[0] = s.xk[it];
          e[1] = s.wout[it] ? (((s.wout[it] >> 3) - s.wo_off[q]) << 3) | (s.wout[it] & 7) : 0;
          e[2] = s.contact[it];
          e[3] = 0;
          sp = ++sent;
        }
        r[1] = (so & 0xFFFF) | (row_in[0] << 16);
        r[2] = (row_in[1] & 0xFFFF) | (row_in[2] << 16);
        r[3] = (row_in[3] & 0xFFFF) | (sp << 16);
        if (special) {
          pk.spec[it] = (int32_t)nsp;
          std::copy(si, si + SI, pk.si.begin() + (size_t)nsp * SI);
          std::copy(sr, sr + SR, pk.sr.begin() + (size_t)nsp * SR);
          ++nsp;
        } else {
          pk.spec[it] = -1;
        }
        for (int f = 0; f < s.nf; ++f) {
          const Real v = (Real)coef[f];
          std::memcpy(&r[COEF + f * CSTEP], &v, sizeof(Real));
        }
        const Real dv = (Real)s.D[it];
        std::memcpy(&r[COEF + s.nf * CSTEP], &dv, sizeof(Real));
        for (int wd = COEF + (s.nf + 1) * CSTEP; wd < W; ++wd) r[wd] = 0;   // padding to 16 bytes
      }
    }
  });
  for (int q = 0; q < s.n_dir; ++q) {
    if (dir_err[q] == 1) { set_error("element with per-MFP outputs has no ring slot"); return OBTE_ERR_BAD_ARG; }
    if (dir_err[q] == 2) {
      set_error("more than three wall inflow faces on one element");
      return OBTE_ERR_UNSUPPORTED;
    }
  }
  if (pk.si.empty()) {
    pk.si.assign(SI, 0);
    pk.sr.assign(SR, 0.0);
  }
  if (pk.pf.empty()) pk.pf.assign(4, -1);
  return OBTE_OK;
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
// Default cap on the polls of one mbarrier wait (each poll may suspend the thread for a while before it
// returns), far above any copy's latency; a wait that reaches it gives up and reports a timeout.
constexpr int kWaitPolls = 1 << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int limit = kWaitPolls) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---- per-sweep values: b = DeltaT + h, p = P - sum_walls g_w T_B ------------------
template <typename Real>
__global__ void sweep_values_kernel(const int32_t* __restrict__ cellmap, const double* __restrict__ Pq,
                                    const int32_t* __restrict__ spec, const int32_t* __restrict__ si,
                                    const Real* __restrict__ sr, const double* __restrict__ u_in, int64_t n,
                                    const double* __restrict__ hs, int with_src, int64_t total, Real* __restrict__ vals) {
  const double* TB = u_in + n;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < total; it += (int64_t)gridDim.x * blockDim.x) {
    const int c = cellmap[it];
    double b = u_in[c];
    double pp = 0;
    if (with_src) {
      if (hs) b += hs[c];
      pp = Pq[it];
    }
    const int sp = spec[it];
    if (sp >= 0) {
      const int32_t* s = si + (int64_t)sp * SI;
      const Real* r = sr + (int64_t)sp * SR;
      for (int k = 0; k < s[3]; ++k) pp -= (double)r[k] * TB[s[4 + k]];
    }
    vals[2 * it] = (Real)b;
    vals[2 * it + 1] = (Real)pp;
  }
}

template <typename Real>
struct SweepParams {
  int64_t n;
  int64_t nd;
  int n_mfp, n_dir, ds, m_pad;
  int n_chunks;            // chunks of MCP MFPs per direction
  int rows;                // ring rows
  int S;                   // slot rows before the zero/trash/periodic rows
  int emax;                // rows per periodic bank
  int unit_wo, pf_pad;     // staging sizes: wall entries and prefetch-list ints per unit
  int nbuf;                // TMA pipeline depth (units staged at once)
  const int32_t* __restrict__ rec;
  const Real* __restrict__ vals;
  const int32_t* __restrict__ lev_ptr;   // unit boundaries (n[q] + 1 per direction)
  const int64_t* __restrict__ lev_off;
  const int32_t* __restrict__ nlev;      // units per direction
  const int32_t* __restrict__ kwo;       // first wall entry of each unit (relative to the direction)
  const int32_t* __restrict__ kpf;       // start of each unit's prefetch list in pf
  const int32_t* __restrict__ pf;        // periodic source index per cut inflow face (-1 = padding)
  const int32_t* __restrict__ ksx;       // first output entry of each unit (absolute)
  const int32_t* __restrict__ sx;        // output entries: xk, wall entries, contact, 0
  int unit_sx;                           // most output entries in one unit
  const int64_t* __restrict__ x_base;
  const int32_t* __restrict__ wo_off;   // [n_dir+1] first wall-output entry of each direction
  const int32_t* __restrict__ wo_wall;
  const Real* __restrict__ mfp;    // [m_pad]
  const Real* __restrict__ tco;    // [n_dir * m_pad]
  const Real* __restrict__ sig;    // [n_dir * m_pad * ds]
  const Real* __restrict__ wo_geo; // [wall entry][4]: wall area vector / volume (x, y, z), 1 / (-sum_mq min(sigma.w, 0))
  const Real* __restrict__ kcoef;  // [n_ce * m_pad]
  const Real* __restrict__ scoef;  // [n_ce]
  const double* __restrict__ u_in;
  double* __restrict__ u_out;
  double* __restrict__ Jraw;
  double* __restrict__ K;
  double* __restrict__ S_out;
  int* __restrict__ err;
  const double* __restrict__ rinv;   // FP64: 1 / (1 + mfp D) [n_dir][n_chunks][n][MC], or null: divide
  float* __restrict__ Xs;   // final pass only: per-ordinate temperatures [n_dir][n][n_mfp], or null
  int xs_add;               // 1: add this pass's temperatures to Xs (the pass at a correction d)
  double* __restrict__ Xd;  // the same in FP64 (FP64 sweeps of obte_bte_sweep_fields), or null
  const int32_t* __restrict__ cta_map;   // CTA -> direction * n_chunks + chunk (a subset), or null: all
  // batched subset sweeps (batch_stride > 0): CTA b runs entry b % n_cta_batch of cta_map on the state
  // vectors u_in / u_out + (b / n_cta_batch) batch_stride.  The batch shares one set of staged values
  // (computed from the first state), so its states must agree on DeltaT and T_B.
  int n_cta_batch;
  int64_t batch_stride;
  // bounded-wait test (obte_bte_plan_test_wait_timeout): level unit whose bulk copy is not issued (-1: none)
  // and the poll cap of the wait for a unit's copy (kWaitPolls normally)
  int skip_unit;
  int wait_limit;
  // deterministic reductions (det != 0, full sweeps only): each (direction, chunk) CTA stores its partial sums
  // instead of adding them atomically; fixed-order reduction kernels sum them afterwards
  int det;
  Real* __restrict__ dpart;   // [n_dir n_chunks][n] lattice-temperature partial of each sweep position
  Real* __restrict__ jpart;   // [n_dir n_chunks][n][ds] flux partials (final pass)
  Real* __restrict__ wpart;   // [n_chunks][n_wo] wall-output partials (wall-output entries of all directions)
  Real* __restrict__ kpart;   // [n_ce][m_pad] kcoef T of each contact entry (final pass)
  Real* __restrict__ spart;   // [n_ce][m_pad] scoef T
  int64_t n_wo;
};

template <typename Real>
__device__ __forceinline__ Real word_real(const int32_t* r, int word);
template <>
__device__ __forceinline__ float word_real<float>(const int32_t* r, int word) {
  return __int_as_float(r[word]);
}
template <>
__device__ __forceinline__ double word_real<double>(const int32_t* r, int word) {
  return __hiloint2double(r[word + 1], r[word]);
}

// num / den.  FP32: hardware reciprocal.  FP64: an FP32 reciprocal seed r (relative error e <= 2^-21)
// and one residual correction of the quotient (Markstein's method), t = num r, q = t + (num - den t) r,
// with relative error e^2 <= 2^-42 (~2e-13): three FP64 operations instead of the five of a fully
// refined reciprocal, on GB300's narrow FP64 pipe, which bounds the FP64 sweep.
__device__ __forceinline__ float quot(float num, float den) { return num * __fdividef(1.0f, den); }
__device__ __forceinline__ double quot(double num, double den) {
  const double r = (double)__fdividef(1.0f, (float)den);
  const double t = num * r;
  return fma(fma(-den, t, num), r, t);
}

// ---- double-float arithmetic (the output pass of the FP32+refine solve) ----------------------------
// A value is an unevaluated pair hi + lo of FP32 numbers (~44 significant bits), computed on the FP32 pipe
// with error-free transformations: Knuth's two-sum, the FMA two-product (Dekker 1971; Ogita, Rump and
// Oishi 2005), here on two MFPs at once with Blackwell's packed FP32x2 instructions.  The intrinsics round
// every operation and are never contracted, which these transformations rely on.  In the ring and the
// per-thread registers a pair lives in the 8 bytes of a double: low word hi, high word lo.
struct df2 {
  float2 h, l;   // hi and lo parts of two MFPs' values
};
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __fadd2_rn(a, f2neg(b)); }
__device__ __forceinline__ df2 two_sum2(float2 a, float2 b) {
  const float2 s = __fadd2_rn(a, b);
  const float2 bb = f2sub(s, a);
  return {s, __fadd2_rn(f2sub(a, f2sub(s, bb)), f2sub(b, bb))};
}
__device__ __forceinline__ df2 fast_two_sum2(float2 a, float2 b) {   // |a| >= |b| (or a exact)
  const float2 s = __fadd2_rn(a, b);
  return {s, f2sub(b, f2sub(s, a))};
}
__device__ __forceinline__ df2 dadd2(df2 a, df2 b) {
  const df2 s = two_sum2(a.h, b.h);
  return fast_two_sum2(s.h, __fadd2_rn(s.l, __fadd2_rn(a.l, b.l)));
}
__device__ __forceinline__ df2 dneg2(df2 a) { return {f2neg(a.h), f2neg(a.l)}; }
__device__ __forceinline__ df2 dmul2(df2 a, df2 b) {
  const float2 p = __fmul2_rn(a.h, b.h);
  float2 e = __ffma2_rn(a.h, b.h, f2neg(p));
  e = __ffma2_rn(a.h, b.l, e);
  e = __ffma2_rn(a.l, b.h, e);
  return fast_two_sum2(p, e);
}
// a / b: an FP32 reciprocal seed y, the quotient q = a y and one correction by the residual a - q b
__device__ __forceinline__ df2 ddiv2(df2 a, df2 b) {
  const float2 y = make_float2(__fdividef(1.0f, b.h.x), __fdividef(1.0f, b.h.y));
  const float2 q = __fmul2_rn(a.h, y);
  float2 r = __ffma2_rn(f2neg(q), b.h, a.h);
  r = __fadd2_rn(r, a.l);
  r = __ffma2_rn(f2neg(q), b.l, r);
  return fast_two_sum2(q, __fmul2_rn(r, y));
}
// split a double into hi + lo (FP64 pipe: two conversions and a subtraction)
__device__ __forceinline__ float2 dsplit(double d) {
  const float h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}
__device__ __forceinline__ df2 dbcast(double d) {   // the same value in both lanes
  const float2 s = dsplit(d);
  return {make_float2(s.x, s.x), make_float2(s.y, s.y)};
}
__device__ __forceinline__ double dpack(float h, float l) { return __hiloint2double(__float_as_int(l), __float_as_int(h)); }
__device__ __forceinline__ double dpack_split(double d) { const float2 s = dsplit(d); return dpack(s.x, s.y); }
__device__ __forceinline__ float dpack_hi(double x) { return __int_as_float(__double2loint(x)); }
__device__ __forceinline__ float dpack_lo(double x) { return __int_as_float(__double2hiint(x)); }
__device__ __forceinline__ double dpack_value(double x) { return (double)dpack_hi(x) + (double)dpack_lo(x); }
__device__ __forceinline__ df2 dunpack2(double a, double b) {   // two packed pairs -> lanes x, y
  return {make_float2(dpack_hi(a), dpack_hi(b)), make_float2(dpack_lo(a), dpack_lo(b))};
}

// Shared memory layout (bytes):
//   [0,64) mbarriers  [64,128) unused
//   [128, ...) nbuf x records | nbuf x values | nbuf x wall weights | nbuf x prefetch lists | sig | K S | ring
// nbuf = TMA pipeline depth: unit u + nbuf - 1 is issued while unit u runs (at most kMaxBuf mbarriers)
static constexpr int kMaxBuf = 8;
// 2 units staged: measured 2.19 ms per FP32 sweep on the 60k-triangle benchmark against 2.46 ms with 3
// (the smaller staging area lets 6 instead of 5 CTAs share an SM); deeper pipelines were no faster.
static constexpr int kDefaultBuf = 2;

template <typename Real>
struct SmemLayout {
  size_t rec, val, gg, pfl, sxo, rec_stride, val_stride, gg_stride, pf_stride, sx_stride, sig, kacc, sacc, ring,
      total;
  __host__ __device__ SmemLayout(int nf, int mcp, int rows, int unit_wo, int pf_pad, int unit_sx, int nbuf) {
    const int W = rec_words(sizeof(Real), nf);
    size_t o = 128;
    rec_stride = (size_t)kUnit * W * 4;
    val_stride = (size_t)(kUnit + 2) * 2 * sizeof(Real);
    val_stride = (val_stride + 15) & ~(size_t)15;
    gg_stride = (size_t)unit_wo * 4 * sizeof(Real);        // 4 Reals per wall entry (16-B multiple)
    pf_stride = (size_t)pf_pad * 4;                        // pf_pad is a multiple of 4
    sx_stride = (size_t)unit_sx * 16;                      // output entries, int4 each
    rec = o; o += nbuf * rec_stride;
    val = o; o += nbuf * val_stride;
    gg = o; o += nbuf * gg_stride;
    pfl = o; o += nbuf * pf_stride;
    sxo = o; o += nbuf * sx_stride;
    sig = o; o += (size_t)mcp * 3 * sizeof(Real);
    kacc = o; o += (size_t)mcp * sizeof(Real);
    sacc = o; o += (size_t)mcp * sizeof(Real);
    o = (o + 15) & ~(size_t)15;
    ring = o; o += (size_t)mcp * rows * sizeof(Real);
    total = o;
  }
};

// 16-byte vectors of the ring: 4 floats or 2 doubles per lane.
template <typename Real> struct V16;
template <> struct V16<float> { static constexpr int K = 4; };
template <> struct V16<double> { static constexpr int K = 2; };

template <int K>
__device__ __forceinline__ void vload(const float* p, float (&x)[K]) {
  if constexpr (K % 4 == 0) {
#pragma unroll
    for (int i = 0; i < K; i += 4) {
      const float4 v = *reinterpret_cast<const float4*>(p + i);
      x[i] = v.x; x[i + 1] = v.y; x[i + 2] = v.z; x[i + 3] = v.w;
    }
  } else {                 // 2 FP32 MFPs per lane: 8-byte rows
    static_assert(K % 2 == 0, "an even number of FP32 MFPs per lane");
#pragma unroll
    for (int i = 0; i < K; i += 2) {
      const float2 v = *reinterpret_cast<const float2*>(p + i);
      x[i] = v.x; x[i + 1] = v.y;
    }
  }
}
template <int K>
__device__ __forceinline__ void vload(const double* p, double (&x)[K]) {
#pragma unroll
  for (int i = 0; i < K; i += 2) {
    const double2 v = *reinterpret_cast<const double2*>(p + i);
    x[i] = v.x; x[i + 1] = v.y;
  }
}
template <int K>
__device__ __forceinline__ void vstore(float* p, const float (&x)[K]) {
  if constexpr (K % 4 == 0) {
#pragma unroll
    for (int i = 0; i < K; i += 4) *reinterpret_cast<float4*>(p + i) = make_float4(x[i], x[i + 1], x[i + 2], x[i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < K; i += 2) *reinterpret_cast<float2*>(p + i) = make_float2(x[i], x[i + 1]);
  }
}
template <int K>
__device__ __forceinline__ void vstore(double* p, const double (&x)[K]) {
#pragma unroll
  for (int i = 0; i < K; i += 2) *reinterpret_cast<double2*>(p + i) = make_double2(x[i], x[i + 1]);
}

// Sum over the G lanes of an element group (aligned groups of G lanes inside a warp).
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v, unsigned mask) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// One CTA = direction q x a chunk of MC = G * KV mean free paths, 128 G threads (KV a multiple of the
// 16-byte vector: 4 or 8 FP32, 2 or 4 FP64).  Every element of
// a unit is owned by a group of G consecutive threads; lane l of the group computes the KV MFPs
// [l KV, (l+1) KV) of the chunk.  The ring is [row][MC] (MFP fastest), so an upstream read is one
// 16-byte shared load per lane and a group of 8 reads one full 128-byte row.
// Resident CTAs per SM the register allocation is bounded for: 8 FP32 MFPs per lane would otherwise take
// ~125 registers and hold an SM to 4 CTAs (a third wave of 32 CTAs on the 60k-triangle cell, 1,248 CTAs
// over 608 slots); at 5 the 1,248 CTAs fit in two waves.  (Capping 4 FP32 MFPs per lane at 64 registers
// made the 110k-tetrahedron sweep, held to 3 CTAs per SM by shared memory, 5 % slower.)
template <typename Real, int G, int KV>
struct SweepMinBlocks { static constexpr int v = (sizeof(Real) == 4 && G == 1 && KV == 8) ? 5 : 1; };

// The thread that issues the bulk copies: lane 0 of the last warp.  Its elements are the last of a unit,
// which most units do not have (median 88 of 128 elements on the 60k-triangle cell), so the issue work stays
// off the warps that every unit keeps busy.
template <int G>
struct Issuer { static constexpr int tid = kUnit * G - 32; };

// DF (Real = double, FINAL only): the FP64 tables swept in double-float arithmetic (see df2).
template <typename Real, int NF, int G, int KV, bool FINAL, bool DF = false>
__global__ void __launch_bounds__(kUnit * G, SweepMinBlocks<Real, G, KV>::v) bte_sweep_kernel(const SweepParams<Real> p) {
  static_assert(!DF || (sizeof(Real) == 8 && FINAL && KV % 2 == 0), "double-float sweeps: FP64 tables, output pass");
  constexpr int RW = Rec<Real, NF>::W;           // record words
  constexpr int MC = G * KV;                     // MFPs per CTA
  constexpr int VB = 2 * sizeof(Real);           // bytes of one (b, p) pair
  extern __shared__ __align__(128) unsigned char smem[];
  const int rows = p.rows;
  const int nbuf = p.nbuf;
  const SmemLayout<Real> L(NF, MC, rows, p.unit_wo, p.pf_pad, p.unit_sx, nbuf);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  Real* s_k = reinterpret_cast<Real*>(smem + L.kacc);
  Real* s_s = reinterpret_cast<Real*>(smem + L.sacc);
  Real* ring = reinterpret_cast<Real*>(smem + L.ring);    // [rows][MC]

  int bid = (int)blockIdx.x;
  int64_t boff = 0;
  if (p.batch_stride > 0) {
    const int bt = bid / p.n_cta_batch;
    bid -= bt * p.n_cta_batch;
    boff = (int64_t)bt * p.batch_stride;
  }
  const int cta = p.cta_map ? p.cta_map[bid] : bid;
  const int q = cta / p.n_chunks;
  const int chunk = cta - q * p.n_chunks;
  const int m0 = chunk * MC;
  const int mc = min(MC, p.n_mfp - m0);
  const int tid = threadIdx.x;
  const int el = tid / G;                        // element of the unit owned by this group
  const int lane = tid - el * G;
  const int mo = lane * KV;                      // first MFP of this lane (within the chunk)
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((tid & 31) & ~(G - 1)));
  const int32_t* __restrict__ lev = p.lev_ptr + p.lev_off[q];
  const int32_t* __restrict__ kwo = p.kwo + p.lev_off[q];
  const int32_t* __restrict__ kpf = p.kpf + p.lev_off[q];
  const int32_t* __restrict__ ksx = p.ksx + p.lev_off[q];
  const int nlev = p.nlev[q];
  const int32_t* __restrict__ rec_q = p.rec + (int64_t)q * p.n * RW;
  // values: absolute byte offsets from the (256-B aligned) array base keep every TMA window 16-B aligned
  const unsigned char* __restrict__ val_base = reinterpret_cast<const unsigned char*>(p.vals);
  const int64_t val_q0 = (int64_t)q * p.n * VB;
  const int64_t xq = p.x_base[q];
  const int wo0 = p.wo_off[q];
  const int nwo = p.wo_off[q + 1] - wo0;
  // wall weights of this (direction, chunk): [entry][MC], entries in sweep order
  const Real* __restrict__ gg_q = p.wo_geo + (int64_t)wo0 * 4;
  const int prow0 = p.S + 2;
  const double* __restrict__ X = p.u_in + boff + p.n + p.nd;
  double* __restrict__ dT_out = p.u_out + boff;
  double* __restrict__ TB_out = p.u_out + boff + p.n;
  double* __restrict__ X_out = p.u_out + boff + p.n + p.nd;

  // this lane's ordinate data in registers; padded MFPs get L = t = sigma = 0 (harmless T = b).
  // sigma (wall re-emission and the final pass only) is read from shared memory: [MC][3]
  Real lam[KV], tt[KV];
#pragma unroll
  for (int j = 0; j < KV; ++j) {
    const bool ok = mo + j < mc;
    const int64_t m = m0 + mo + j;
    lam[j] = ok ? p.mfp[m] : Real(0);
    tt[j] = ok ? p.tco[(int64_t)q * p.m_pad + m] : Real(0);
  }
  Real* s_sig = reinterpret_cast<Real*>(smem + L.sig);
  for (int i = tid; i < MC * 3; i += blockDim.x) {
    const int jj = i / 3, d = i - 3 * jj;
    const Real sv = (jj < mc && d < p.ds) ? p.sig[((int64_t)q * p.m_pad + m0 + jj) * p.ds + d] : Real(0);
    if constexpr (DF) s_sig[i] = dpack_split(sv);   // packed hi / lo pairs
    else s_sig[i] = sv;
  }
  // real value of a shared sigma entry (DF keeps them as packed pairs)
  auto sigv = [&](Real x) -> Real {
    if constexpr (DF) return dpack_value(x);
    else return x;
  };
  // DF: this lane's MFPs and weights as pairs (lanes x, y = MFPs j, j + 1)
  df2 lam2[DF ? KV / 2 : 1], tt2[DF ? KV / 2 : 1];
  if constexpr (DF) {
#pragma unroll
    for (int j = 0; j < KV; j += 2) {
      const float2 l0 = dsplit(lam[j]), l1 = dsplit(lam[j + 1]), t0 = dsplit(tt[j]), t1 = dsplit(tt[j + 1]);
      lam2[j / 2] = {make_float2(l0.x, l1.x), make_float2(l0.y, l1.y)};
      tt2[j / 2] = {make_float2(t0.x, t1.x), make_float2(t0.y, t1.y)};
    }
  }
  if (FINAL)
    for (int j = tid; j < MC; j += blockDim.x) { s_k[j] = 0; s_s[j] = 0; }
  // ring: zero everything, then bank 0 holds the cut inflow values of unit 0
  const int npf0 = nlev > 0 ? kpf[1] - kpf[0] : 0;
  for (int i = tid; i < MC * rows; i += blockDim.x) {
    const int row = i / MC, col = i - row * MC;
    Real v = 0;
    const int j = row - prow0;
    if (j >= 0 && j < npf0 && col < mc) {
      const int k = p.pf[kpf[0] + j];
      if (k >= 0) v = (Real)X[(xq + k) * p.n_mfp + m0 + col];
    }
    if constexpr (DF) ring[i] = dpack_split(v);
    else ring[i] = v;
  }
  if (tid == 0) {
    for (int i = 0; i < nbuf; ++i) mbar_init(&bars[i], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // TMA of unit u into buffer bi: records [a, e), values [a, e) (16-B aligned window), the
  // wall weights of the unit's wall entries and the prefetch list of unit u + 1
  auto issue = [&](int u, int bi) {
    if (u == p.skip_unit) return;   // test of the bounded wait: this unit's copy never arrives
    const int a = lev[u], e = lev[u + 1];
    const unsigned rbytes = (unsigned)(e - a) * RW * 4u;
    const int64_t vb0 = (val_q0 + (int64_t)a * VB) & ~(int64_t)15;
    const int64_t vb1 = (val_q0 + (int64_t)e * VB + 15) & ~(int64_t)15;
    const unsigned vbytes = (unsigned)(vb1 - vb0);
    const int w0 = kwo[u], w1 = kwo[u + 1];
    const unsigned gbytes = (unsigned)(w1 - w0) * 4u * (unsigned)sizeof(Real);
    const int f0 = u + 1 < nlev ? kpf[u + 1] : 0, f1 = u + 1 < nlev ? kpf[u + 2] : 0;
    const unsigned pbytes = (unsigned)(f1 - f0) * 4u;
    const int x0 = ksx[u], x1 = ksx[u + 1];
    const unsigned sbytes = (unsigned)(x1 - x0) * 16u;
    uint64_t* bar = &bars[bi];
    fence_proxy_async();
    mbar_expect_tx(bar, rbytes + vbytes + gbytes + pbytes + sbytes);
    tma_load_1d(smem + L.rec + bi * L.rec_stride, rec_q + (int64_t)a * RW, rbytes, bar);
    tma_load_1d(smem + L.val + bi * L.val_stride, val_base + vb0, vbytes, bar);
    if (gbytes) tma_load_1d(smem + L.gg + bi * L.gg_stride, gg_q + (int64_t)w0 * 4, gbytes, bar);
    if (pbytes) tma_load_1d(smem + L.pfl + bi * L.pf_stride, p.pf + f0, pbytes, bar);
    if (sbytes) tma_load_1d(smem + L.sxo + bi * L.sx_stride, p.sx + (int64_t)x0 * 4, sbytes, bar);
  };
  constexpr int kIssuer = Issuer<G>::tid;
  if (tid == kIssuer)
    for (int u = 0; u < nbuf - 1 && u < nlev; ++u) issue(u, u);

  // per-unit metadata, loaded one unit ahead so that its latency stays off the unit's critical path
  int a = nlev > 0 ? lev[0] : 0, e = nlev > 0 ? lev[1] : 0;
  int wu = kwo[0];
  int kpf1 = nlev > 1 ? kpf[1] : 0, kpf2 = nlev > 1 ? kpf[2] : 0;
  // the value window of a unit starts (q n + a) pairs into the array; FP32 pairs are 8 bytes, so the
  // 16-byte aligned window starts one pair early when q n + a is odd (FP64 pairs are 16 bytes: never)
  const int qn_odd = (int)(((int64_t)q * p.n) & 1);
  // FP64 with the reciprocal table: this element's 1 / (1 + mfp D) for the current unit, and for the next
  // unit loaded one unit ahead (a coalesced 16-byte global load per lane, off the unit's critical path)
  constexpr bool kRinv = sizeof(Real) == 8 && !DF;
  double rcur[KV], rnxt[KV];
  const double* __restrict__ rinv_qc =
      (kRinv && p.rinv) ? p.rinv + ((int64_t)q * p.n_chunks + chunk) * p.n * MC : nullptr;
  if (rinv_qc && nlev > 0 && el < e - a) vload(rinv_qc + (int64_t)(a + el) * MC + mo, rcur);
  int bi = 0;            // buffer of unit u (u mod nbuf)
  unsigned phase = 0;    // parity of its mbarrier phase ((u / nbuf) & 1)
  for (int u = 0; u < nlev; ++u) {
    const int e_next = u + 2 <= nlev ? lev[u + 2] : 0;
    const int wu_next = kwo[u + 1];
    const int kpf3 = u + 3 <= nlev ? kpf[u + 3] : 0;
    const int npf = u + 1 < nlev ? kpf2 - kpf1 : 0;   // padded length of unit u+1's list
    const int prow_next = prow0 + ((u + 1) & 1) * p.emax;
    if (rinv_qc && u + 1 < nlev && el < e_next - e) vload(rinv_qc + (int64_t)(e + el) * MC + mo, rnxt);
    // buffer (u + nbuf - 1) mod nbuf was last read during unit u - 1, finished at the barrier below
    if (tid == kIssuer && u + nbuf - 1 < nlev) issue(u + nbuf - 1, bi == 0 ? nbuf - 1 : bi - 1);
    const bool ready = mbar_wait_bounded(&bars[bi], phase, p.wait_limit);
    // the periodic prefetch runs on the high thread indices (list entry i on element kUnit - 1 - i), which
    // most units leave without an element
    const int pf_i = kUnit - 1 - el;
    if (!ready) {
      atomicOr(p.err, 1);
    } else {
      // cut inflow values of unit u+1: loads issued now, stored into bank (u+1)&1 after the MFP loop
      const int32_t* s_pf = reinterpret_cast<const int32_t*>(smem + L.pfl + bi * L.pf_stride);
      const int pk = pf_i < npf ? s_pf[pf_i] : -1;
      double xv[KV];
      if (pk >= 0) {
        const double* xs = X + (xq + pk) * p.n_mfp + m0 + mo;
#pragma unroll
        for (int j = 0; j < KV; ++j) xv[j] = mo + j < mc ? __ldg(xs + j) : 0.0;
      }
      if (el < e - a) {
        // record: RW/4 vector loads (the G lanes of the group read the same record)
        int32_t r[RW];
        const int4* r4 = reinterpret_cast<const int4*>(smem + L.rec + bi * L.rec_stride) + el * (RW / 4);
#pragma unroll
        for (int i = 0; i < RW / 4; ++i) {
          const int4 x = r4[i];
          r[4 * i] = x.x; r[4 * i + 1] = x.y; r[4 * i + 2] = x.z; r[4 * i + 3] = x.w;
        }
        const int voff = sizeof(Real) == 4 ? ((qn_odd + a) & 1) : 0;
        const Real* v = reinterpret_cast<const Real*>(smem + L.val + bi * L.val_stride) + 2 * (voff + el);
        const Real b = v[0], pw = v[1];
        const int c = r[0];
        const int so = r[1] & 0xFFFF, s0 = (int)((unsigned)r[1] >> 16);
        const int s1 = r[2] & 0xFFFF, s2 = (int)((unsigned)r[2] >> 16);
        const int s3 = r[3] & 0xFFFF, sp = (int)((unsigned)r[3] >> 16);
        int xk = -1, wo = 0, ce = -1;
        if (sp) {
          const int4 ent = reinterpret_cast<const int4*>(smem + L.sxo + bi * L.sx_stride)[sp - 1];
          xk = ent.x; wo = ent.y; ce = ent.z;
        }
        using RR = Rec<Real, NF>;
        const Real c0 = word_real<Real>(r, RR::COEF);
        const Real c1 = word_real<Real>(r, RR::COEF + RR::CSTEP);
        const Real c2 = word_real<Real>(r, RR::COEF + 2 * RR::CSTEP);
        const Real c3 = NF > 3 ? word_real<Real>(r, RR::COEF + 3 * RR::CSTEP) : Real(0);
        const Real D = word_real<Real>(r, RR::D);
        Real v0[KV], v1[KV], v2[KV], v3[KV];
        vload(ring + s0 * MC + mo, v0);
        vload(ring + s1 * MC + mo, v1);
        vload(ring + s2 * MC + mo, v2);
        if (NF > 3) vload(ring + s3 * MC + mo, v3);
        Real T[KV];
        Real dacc = 0, j0 = 0, j1 = 0, j2 = 0;
        if constexpr (DF) {
          // output pass in double-float: the ring holds packed pairs, every product and sum is a pair
          const df2 C0 = dbcast(c0), C1 = dbcast(c1), C2 = dbcast(c2), C3 = dbcast(c3), DD = dbcast(D);
          const df2 BB = dbcast(b), PW = dbcast(pw);
          const df2 ONE = {make_float2(1.0f, 1.0f), make_float2(0.0f, 0.0f)};
          df2 da = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)}, ja = da, jb = da, jc = da;
          Real Tp[KV];
#pragma unroll
          for (int j = 0; j < KV; j += 2) {
            df2 sm = dmul2(C0, dunpack2(v0[j], v0[j + 1]));
            sm = dadd2(sm, dmul2(C1, dunpack2(v1[j], v1[j + 1])));
            sm = dadd2(sm, dmul2(C2, dunpack2(v2[j], v2[j + 1])));
            if (NF > 3) sm = dadd2(sm, dmul2(C3, dunpack2(v3[j], v3[j + 1])));
            const df2 LM = lam2[j / 2];
            const df2 num = dadd2(BB, dmul2(LM, dadd2(PW, dneg2(sm))));   // b + L (pw - sm)
            const df2 den = dadd2(ONE, dmul2(LM, DD));                    // 1 + L D
            const df2 t2 = ddiv2(num, den);
            Tp[j] = dpack(t2.h.x, t2.l.x);
            Tp[j + 1] = dpack(t2.h.y, t2.l.y);
            da = dadd2(da, dmul2(tt2[j / 2], t2));
            const Real* sj = s_sig + (mo + j) * 3;   // packed sigma of MFPs j (sj[0..2]) and j + 1 (sj[3..5])
            ja = dadd2(ja, dmul2(dunpack2(sj[0], sj[3]), t2));
            jb = dadd2(jb, dmul2(dunpack2(sj[1], sj[4]), t2));
            if (p.ds > 2) jc = dadd2(jc, dmul2(dunpack2(sj[2], sj[5]), t2));
          }
          dacc = ((double)da.h.x + (double)da.h.y) + ((double)da.l.x + (double)da.l.y);
          j0 = ((double)ja.h.x + (double)ja.h.y) + ((double)ja.l.x + (double)ja.l.y);
          j1 = ((double)jb.h.x + (double)jb.h.y) + ((double)jb.l.x + (double)jb.l.y);
          j2 = ((double)jc.h.x + (double)jc.h.y) + ((double)jc.l.x + (double)jc.l.y);
          vstore(ring + so * MC + mo, Tp);
          // real values for the per-MFP outputs below (periodic outflow, walls, contact, stored fields)
          const bool need = sp != 0 || p.Xs != nullptr || p.Xd != nullptr;
#pragma unroll
          for (int j = 0; j < KV; ++j) T[j] = need ? dpack_value(Tp[j]) : Real(0);
        } else if constexpr (sizeof(Real) == 4 && KV % 2 == 0) {
          // FP32: the MFPs in pairs with Blackwell's packed FP32x2 arithmetic (one instruction per two MFPs;
          // each lane of a packed operation rounds like the scalar one)
          const float2 C0 = make_float2(c0, c0), C1 = make_float2(c1, c1), C2 = make_float2(c2, c2);
          const float2 C3 = make_float2(c3, c3), DD = make_float2(D, D), BB = make_float2(b, b);
          const float2 PW = make_float2(pw, pw), ONE = make_float2(1.0f, 1.0f), NEG = make_float2(-1.0f, -1.0f);
          float2 da = make_float2(0.0f, 0.0f), ja = da, jb = da, jc = da;
#pragma unroll
          for (int j = 0; j < KV; j += 2) {
            float2 sm = __fmul2_rn(C0, make_float2(v0[j], v0[j + 1]));
            sm = __ffma2_rn(C1, make_float2(v1[j], v1[j + 1]), sm);
            sm = __ffma2_rn(C2, make_float2(v2[j], v2[j + 1]), sm);
            if (NF > 3) sm = __ffma2_rn(C3, make_float2(v3[j], v3[j + 1]), sm);
            const float2 lm = make_float2(lam[j], lam[j + 1]);
            const float2 num = __ffma2_rn(lm, __ffma2_rn(NEG, sm, PW), BB);    // b + L (pw - sm)
            const float2 den = __ffma2_rn(lm, DD, ONE);                        // 1 + L D
            const float2 t2 = __fmul2_rn(num, make_float2(__fdividef(1.0f, den.x), __fdividef(1.0f, den.y)));
            T[j] = t2.x;
            T[j + 1] = t2.y;
            da = __ffma2_rn(make_float2(tt[j], tt[j + 1]), t2, da);
            if (FINAL) {
              const Real* sj = s_sig + (mo + j) * 3;
              ja = __ffma2_rn(make_float2(sj[0], sj[3]), t2, ja);
              jb = __ffma2_rn(make_float2(sj[1], sj[4]), t2, jb);
              if (p.ds > 2) jc = __ffma2_rn(make_float2(sj[2], sj[5]), t2, jc);
            }
          }
          dacc = da.x + da.y;
          j0 = ja.x + ja.y;
          j1 = jb.x + jb.y;
          j2 = jc.x + jc.y;
        } else {
#pragma unroll
          for (int j = 0; j < KV; ++j) {
            Real sm = c0 * v0[j] + c1 * v1[j] + c2 * v2[j];
            if (NF > 3) sm += c3 * v3[j];
            if (kRinv && rinv_qc) T[j] = (Real)((b + lam[j] * (pw - sm)) * rcur[j]);
            else T[j] = quot(b + lam[j] * (pw - sm), Real(1) + lam[j] * D);
            dacc += tt[j] * T[j];
            if (FINAL) {
              const Real* sj = s_sig + (mo + j) * 3;
              j0 += sj[0] * T[j];
              j1 += sj[1] * T[j];
              if (p.ds > 2) j2 += sj[2] * T[j];
            }
          }
        }
        if constexpr (!DF) vstore(ring + so * MC + mo, T);
        if (FINAL && p.Xs != nullptr) {
#pragma unroll
          for (int j = 0; j < KV; ++j)
            if (mo + j < mc) {
              float* xs = p.Xs + ((int64_t)q * p.n + c) * p.n_mfp + m0 + mo + j;
              *xs = p.xs_add ? *xs + (float)T[j] : (float)T[j];
            }
        }
        if (FINAL && p.Xd != nullptr) {
#pragma unroll
          for (int j = 0; j < KV; ++j)
            if (mo + j < mc) p.Xd[((int64_t)q * p.n + c) * p.n_mfp + m0 + mo + j] = (double)T[j];
        }
        dacc = group_sum<G>(dacc, gmask);
        if (lane == 0) {
          if (p.det) p.dpart[(int64_t)cta * p.n + a + el] = dacc;
          else atomicAdd(&dT_out[c], (double)dacc);
        }
        if (FINAL) {
          j0 = group_sum<G>(j0, gmask);
          j1 = group_sum<G>(j1, gmask);
          j2 = group_sum<G>(j2, gmask);
          if (lane == 0) {
            if (p.det) {
              Real* jp = p.jpart + ((int64_t)cta * p.n + a + el) * p.ds;
              jp[0] = j0;
              if (p.ds > 1) jp[1] = j1;
              if (p.ds > 2) jp[2] = j2;
            } else {
              atomicAdd(&p.Jraw[(int64_t)c * p.ds], (double)j0);
              if (p.ds > 1) atomicAdd(&p.Jraw[(int64_t)c * p.ds + 1], (double)j1);
              if (p.ds > 2) atomicAdd(&p.Jraw[(int64_t)c * p.ds + 2], (double)j2);
            }
          }
        }
        // per-MFP outputs of special elements (the group is uniform in these conditions)
        if (xk >= 0) {
#pragma unroll
          for (int j = 0; j < KV; ++j)
            if (mo + j < mc) X_out[(xq + xk) * p.n_mfp + m0 + mo + j] = (double)T[j];
        }
        if (wo != 0) {
          const int wb = wo >> 3, wn = wo & 7;
          // re-emission weight max(sigma . w, 0) / (-sum min(sigma . w, 0)) from the staged wall geometry
          // (bte.py:73-78); absent entries read the first entry (unused)
          const Real* gw = reinterpret_cast<const Real*>(smem + L.gg + bi * L.gg_stride) + (size_t)(wb - wu) * 4;
          const Real* gw1 = gw + (wn > 1 ? 4 : 0);
          const Real* gw2 = gw + (wn > 2 ? 8 : 0);
          Real w0 = 0, w1 = 0, w2 = 0;
#pragma unroll
          for (int j = 0; j < KV; ++j) {
            const Real* sj = s_sig + (mo + j) * 3;
            const Real s0r = sigv(sj[0]), s1r = sigv(sj[1]), s2r = sigv(sj[2]);
            const Real a0 = s0r * gw[0] + s1r * gw[1] + s2r * gw[2];
            const Real a1 = s0r * gw1[0] + s1r * gw1[1] + s2r * gw1[2];
            const Real a2 = s0r * gw2[0] + s1r * gw2[1] + s2r * gw2[2];
            w0 += (a0 > Real(0) ? a0 * gw[3] : Real(0)) * T[j];
            w1 += (a1 > Real(0) ? a1 * gw1[3] : Real(0)) * T[j];
            w2 += (a2 > Real(0) ? a2 * gw2[3] : Real(0)) * T[j];
          }
          w0 = group_sum<G>(w0, gmask);
          if (wn > 1) w1 = group_sum<G>(w1, gmask);
          if (wn > 2) w2 = group_sum<G>(w2, gmask);
          if (lane == 0) {
            if (p.det) {
              Real* wp = p.wpart + (int64_t)chunk * p.n_wo + wo0 + wb;
              wp[0] = w0;
              if (wn > 1) wp[1] = w1;
              if (wn > 2) wp[2] = w2;
            } else {
              atomicAdd(&TB_out[p.wo_wall[wo0 + wb]], (double)w0);
              if (wn > 1) atomicAdd(&TB_out[p.wo_wall[wo0 + wb + 1]], (double)w1);
              if (wn > 2) atomicAdd(&TB_out[p.wo_wall[wo0 + wb + 2]], (double)w2);
            }
          }
        }
        if (FINAL && ce >= 0) {
#pragma unroll
          for (int j = 0; j < KV; ++j) {
            if (mo + j < mc) {
              const Real kv = p.kcoef[(int64_t)ce * p.m_pad + m0 + mo + j] * T[j], sv = p.scoef[ce] * T[j];
              if (p.det) {
                p.kpart[(int64_t)ce * p.m_pad + m0 + mo + j] = kv;
                p.spart[(int64_t)ce * p.m_pad + m0 + mo + j] = sv;
              } else {
                atomicAdd(&s_k[mo + j], kv);
                atomicAdd(&s_s[mo + j], sv);
              }
            }
          }
        }
      }
      // bank (u+1)&1 was last read during unit u-1
      if (pk >= 0) {
        Real xr[KV];
#pragma unroll
        for (int j = 0; j < KV; ++j) {
          if constexpr (DF) xr[j] = dpack_split(xv[j]);
          else xr[j] = (Real)xv[j];
        }
        vstore(ring + (prow_next + pf_i) * MC + mo, xr);
      }
      for (int i = pf_i + kUnit; i < npf; i += kUnit) {   // units with more than kUnit cut inflow faces
        const int k = s_pf[i];
        if (k < 0) continue;
        const double* xs = X + (xq + k) * p.n_mfp + m0 + mo;
        for (int j = 0; j < KV; ++j) {
          const Real xval = mo + j < mc ? (Real)xs[j] : Real(0);
          if constexpr (DF) ring[(size_t)(prow_next + i) * MC + mo + j] = dpack_split(xval);
          else ring[(size_t)(prow_next + i) * MC + mo + j] = xval;
        }
      }
    }
    // block barrier that also tells every thread whether any wait of this unit gave up
    if (__syncthreads_or(ready ? 0 : 1)) {
      // let the copies this CTA still has in flight land before leaving (bounded)
      if (tid == kIssuer)
        for (int w = u + 1; w < nlev && w < u + nbuf; ++w) mbar_wait_bounded(&bars[w % nbuf], (unsigned)(w / nbuf) & 1u);
      __syncthreads();
      return;
    }
    if (++bi == nbuf) { bi = 0; phase ^= 1u; }
    a = e;
    e = e_next;
    wu = wu_next;
    kpf1 = kpf2;
    kpf2 = kpf3;
    if (rinv_qc) {
#pragma unroll
      for (int j = 0; j < KV; ++j) rcur[j] = rnxt[j];
    }
  }
  if (FINAL && !p.det) {
    for (int j = tid; j < mc; j += blockDim.x) {
      p.K[(int64_t)(m0 + j) * p.n_dir + q] = (double)s_k[j];
      p.S_out[(int64_t)(m0 + j) * p.n_dir + q] = (double)s_s[j];
    }
  }
}

// ---- deterministic reductions -------------------------------------------------------
// Every sum below runs in a fixed order (chunks, then directions; a wall's entries in entry order; a
// direction's contact entries in order), so the result does not depend on which CTA ran first.

// S[q][pos] = sum over chunks of the lattice-temperature partials (and the flux partials)
template <typename Real>
__global__ void det_pos_sum_kernel(const Real* __restrict__ dpart, const Real* __restrict__ jpart, int n_chunks,
                                   int64_t n, int64_t total, int ds, double* __restrict__ S, double* __restrict__ SJ) {
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < total; it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = it / n, pos = it - q * n;
    const int64_t b0 = q * n_chunks * n + pos;
    double acc = 0;
    for (int ch = 0; ch < n_chunks; ++ch) acc += (double)dpart[b0 + (int64_t)ch * n];
    S[it] = acc;
    if (jpart)
      for (int d = 0; d < ds; ++d) {
        double aj = 0;
        for (int ch = 0; ch < n_chunks; ++ch) aj += (double)jpart[(b0 + (int64_t)ch * n) * ds + d];
        SJ[it * ds + d] = aj;
      }
  }
}

// element sums over the directions, through the position of the element in each direction's order
__global__ void det_elem_sum_kernel(const double* __restrict__ S, const double* __restrict__ SJ,
                                    const int32_t* __restrict__ inv, int n_dir, int64_t n, int ds,
                                    double* __restrict__ dT_out, double* __restrict__ Jraw) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0, a0 = 0, a1 = 0, a2 = 0;
    for (int q = 0; q < n_dir; ++q) {
      const int64_t it = (int64_t)q * n + inv[(int64_t)q * n + c];
      acc += S[it];
      if (SJ) {
        a0 += SJ[it * ds];
        if (ds > 1) a1 += SJ[it * ds + 1];
        if (ds > 2) a2 += SJ[it * ds + 2];
      }
    }
    dT_out[c] = acc;
    if (SJ) {
      Jraw[c * ds] = a0;
      if (ds > 1) Jraw[c * ds + 1] = a1;
      if (ds > 2) Jraw[c * ds + 2] = a2;
    }
  }
}

template <typename Real>
__global__ void det_wall_sum_kernel(const Real* __restrict__ wpart, int n_chunks, int64_t n_wo,
                                    const int32_t* __restrict__ wptr, const int32_t* __restrict__ went, int64_t nd,
                                    double* __restrict__ TB_out) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nd; w += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int k = wptr[w]; k < wptr[w + 1]; ++k)
      for (int ch = 0; ch < n_chunks; ++ch) acc += (double)wpart[(int64_t)ch * n_wo + went[k]];
    TB_out[w] = acc;
  }
}

template <typename Real>
__global__ void det_contact_sum_kernel(const Real* __restrict__ kpart, const Real* __restrict__ spart,
                                       const int32_t* __restrict__ ce_off, int n_dir, int n_mfp, int m_pad,
                                       double* __restrict__ K, double* __restrict__ S) {
  const int64_t total = (int64_t)n_mfp * n_dir;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < total; it += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(it / n_dir), q = (int)(it - (int64_t)m * n_dir);
    double ak = 0, as = 0;
    for (int ce = ce_off[q]; ce < ce_off[q + 1]; ++ce) {
      ak += (double)kpart[(int64_t)ce * m_pad + m];
      as += (double)spart[(int64_t)ce * m_pad + m];
    }
    K[it] = ak;
    S[it] = as;
  }
}

// ---- table upload ---------------------------------------------------------------

size_t DevSchedule::bytes() const {
  const DevBuf* all[] = {&rec, &klev_ptr, &klev_off, &knlev, &kwo, &kpf, &pf, &sx, &ksx, &mfp, &tco, &sig, &wo_wall, &wo_geo,
                         &kcoef, &scoef, &hs, &vals, &cellmap, &Pq, &si, &sr, &wo_off, &spec, &lpt, &rinv};
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


// Compiled thread shapes (lanes per element G, MFPs per lane KV) for each precision.
struct Shape { int G, KV; };
template <typename Real> struct Shapes;
template <> struct Shapes<float> { static constexpr Shape v[] = {{1, 4}, {1, 8}, {2, 4}, {1, 2}}; };
template <> struct Shapes<double> { static constexpr Shape v[] = {{1, 2}, {1, 4}, {2, 2}}; };
constexpr Shape Shapes<float>::v[];
constexpr Shape Shapes<double>::v[];

// Choose the thread shape.  Measured on the 60k-triangle (100 MFP x 96 directions) and 110k-tetrahedron
// (30 x 512) benchmark meshes: one thread per element (G = 1) is fastest (2.32 / 10.5 ms per FP32 sweep
// against 2.40 / 16.7 ms at G = 2 and 2.90 ms at G = 8), because each CTA is a chain of level barriers
// and more, smaller CTAs per SM keep more chains in flight.
// OBTE_SWEEP_G / OBTE_SWEEP_KV force a shape (tuning); a shape whose shared memory does not fit is
// skipped.
template <typename Real>
static Shape choose_shape(const Schedule& s, int rows, int unit_wo, int pf_pad, int unit_sx, int nbuf,
                          size_t optin) {
  const char* eg = std::getenv("OBTE_SWEEP_G");
  const char* ek = std::getenv("OBTE_SWEEP_KV");
  const int want_g = eg ? std::atoi(eg) : 1;
  const int want_k = ek ? std::atoi(ek) : V16<Real>::K;
  auto fits = [&](Shape sh) {
    return SmemLayout<Real>(s.nf, sh.G * sh.KV, rows, unit_wo, pf_pad, unit_sx, nbuf).total <= optin;
  };
  if (eg || ek) {
    for (Shape sh : Shapes<Real>::v)
      if (sh.G == want_g && sh.KV == want_k && fits(sh)) return sh;
  } else {
    // two vectors per lane halve the per-element overhead per MFP; worth it while at least 4 CTAs still
    // share an SM (60k triangles: 2.14 against 2.23 ms; 110k tetrahedra, 2 CTAs per SM: 20.8 against 11.6 ms)
    const Shape wide{1, 2 * V16<Real>::K};
    const size_t sm = SmemLayout<Real>(s.nf, wide.KV, rows, unit_wo, pf_pad, unit_sx, nbuf).total;
    if (sizeof(Real) == 4 && sm + 1024 <= (228 * 1024) / 4 && fits(wide)) return wide;
  }
  const Shape base{1, V16<Real>::K};
  return fits(base) ? base : Shape{0, 0};
}

template <typename Real>
static obte_status upload_tables(obte_plan plan, DevSchedule& d) {
  PhaseTimer timer(sizeof(Real) == 4 ? "upload_tables fp32" : "upload_tables fp64");
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  // split levels into units of at most kUnit elements (slots were assigned per level, so this stays valid)
  Units un;
  build_units(s, un);
  Packed pk;
  {
    PhaseTimer tp("pack");
    OBTE_TRY(pack<Real>(s, un, pk));
  }
  const int rows = pk.rows;
  const char* nb_env = std::getenv("OBTE_SWEEP_NBUF");
  const int nbuf = nb_env ? std::max(2, std::min(kMaxBuf, std::atoi(nb_env))) : kDefaultBuf;
  const Shape sh = choose_shape<Real>(s, rows, pk.unit_wo, pk.pf_pad, pk.unit_sx, nbuf, plan->ctx->smem_optin);
  const int G = sh.G;
  if (!G) {
    set_error("sweep front needs more shared memory than one CTA can have (" + std::to_string(rows) + " rows)");
    return OBTE_ERR_UNSUPPORTED;
  }
  const int mcp = G * sh.KV;
  d.G = G;
  d.KV = sh.KV;
  d.mc = mcp;
  d.mcp = mcp;
  d.n_chunks = (s.n_mfp + mcp - 1) / mcp;
  d.zero_slot = s.max_slots;
  d.rows = rows;
  d.emax = pk.emax;
  d.unit_wo = pk.unit_wo;
  d.pf_pad = pk.pf_pad;
  d.nbuf = nbuf;
  d.unit_sx = pk.unit_sx;
  d.smem = SmemLayout<Real>(s.nf, mcp, rows, pk.unit_wo, pk.pf_pad, pk.unit_sx, nbuf).total;
  if (timer.on)
    std::fprintf(stderr, "[obte trace] sweep shape %s: G %d KV %d, %d chunks x %d directions = %d CTAs, %zu B shared "
                 "memory (%d rows = %d slots + 2 + 2 x %d bank rows; staging per unit: %d wall entries, %d prefetch ints, %d "
                 "output entries), <= %zu CTAs per SM by shared memory\n", sizeof(Real) == 4 ? "fp32" : "fp64", G,
                 sh.KV, d.n_chunks, s.n_dir, d.n_chunks * s.n_dir, d.smem, rows, s.max_slots, pk.emax, pk.unit_wo,
                 pk.pf_pad, pk.unit_sx, (size_t)(233472 / (d.smem + 1024)));
  OBTE_TRY(upload(d.rec, pk.rec, st));
  OBTE_TRY(upload(d.cellmap, pk.cellmap, st));
  OBTE_TRY(upload(d.Pq, pk.P, st));
  OBTE_TRY(upload(d.si, pk.si, st));
  OBTE_TRY(upload(d.spec, pk.spec, st));
  OBTE_TRY(upload_real<Real>(d.sr, pk.sr, st));
  {
    // Each CTA is a serial chain of its direction's units (602-846 per direction on the 60k-triangle
    // cell), and the grid runs in about two waves: launching the longest chains first keeps a slot from
    // drawing two long ones (longest-processing-time-first order; the hardware dispatches blocks in index
    // order).
    // (FP32 only: 1.920 -> 1.855 ms per sweep there, while the FP64 sweep, bound by the FP64 pipe and not
    // by chain latency, was 5 % slower in this order.)
    std::vector<int32_t> dirs(s.n_dir);
    for (int q = 0; q < s.n_dir; ++q) dirs[q] = q;
    if (sizeof(Real) == 4)
      std::stable_sort(dirs.begin(), dirs.end(), [&](int a, int b) { return un.n[a] > un.n[b]; });
    std::vector<int32_t> lpt;
    lpt.reserve((size_t)s.n_dir * d.n_chunks);
    for (int q : dirs)
      for (int c = 0; c < d.n_chunks; ++c) lpt.push_back(q * d.n_chunks + c);
    OBTE_TRY(upload(d.lpt, lpt, st));
  }
  OBTE_TRY(upload(d.klev_ptr, un.ptr, st));
  OBTE_TRY(upload(d.klev_off, un.off, st));
  OBTE_TRY(upload(d.knlev, un.n, st));
  OBTE_TRY(upload(d.kwo, pk.kwo, st));
  OBTE_TRY(upload(d.kpf, pk.kpf, st));
  OBTE_TRY(upload(d.pf, pk.pf, st));
  OBTE_TRY(upload(d.sx, pk.sx, st));
  OBTE_TRY(upload(d.ksx, pk.ksx, st));
  std::vector<int32_t> wo = s.wo_wall;
  if (wo.empty()) wo.push_back(0);
  OBTE_TRY(upload(d.wo_wall, wo, st));
  OBTE_TRY(upload(d.wo_off, s.wo_off, st));
  OBTE_TRY(upload_real<Real>(d.mfp, s.mfp, st));
  OBTE_TRY(upload_real<Real>(d.tco, s.tco, st));
  OBTE_TRY(upload_real<Real>(d.sig, s.sig, st));
  {
    // wall weights regrouped [direction][chunk][entry][mcp] so one unit's entries are one contiguous copy
    // per wall entry: area vector / volume of the wall's element and 1 / (-sum_mq min(sigma . w, 0))
    const int64_t n_wo = (int64_t)s.wo_wall.size();
    std::vector<Real> geo(std::max<size_t>((size_t)n_wo * 4, 4), Real(0));
    parallel_for(n_wo, [&](int64_t e) {
      const int32_t w = s.wo_wall[e];
      for (int k = 0; k < s.dim; ++k) geo[(size_t)e * 4 + k] = (Real)s.w_db[(size_t)w * s.dim + k];
      geo[(size_t)e * 4 + 3] = s.gbm_sum[w] != 0 ? (Real)(1.0 / (-s.gbm_sum[w])) : Real(0);
    });
    OBTE_TRY(upload(d.wo_geo, geo, st));
  }
  OBTE_TRY(upload_real<Real>(d.kcoef, s.kcoef, st));
  OBTE_TRY(upload_real<Real>(d.scoef, s.scoef, st));
  if (!s.hs.empty()) OBTE_TRY(upload(d.hs, s.hs, st));
  // per-sweep values (b, p), padded by 32 B for the aligned TMA window
  OBTE_TRY(d.vals.alloc((size_t)s.n_dir * s.n * 2 * sizeof(Real) + 32));
  OBTE_CUDA(cudaMemsetAsync(d.vals.p, 0, d.vals.bytes, st));
  if (s.tf.ok) {   // transmission plans: keep what refresh_tables rewrites
    d.refreshable = true;
    d.h_spec = std::move(pk.spec);
    d.n_spec = (int64_t)(pk.sr.size() / SR);
  }
  d.ready = true;
  return OBTE_OK;
}

// New transmissions: rewrite the coefficient words of the records and the wall inflow coefficients of
// the special entries (the same walk over the inflow entries as pack), then P and the contact
// coefficients; indices, units and launch order stay.
// Coefficient word w of item `it`'s record from inflow slot f: g0 x (t_s, 1 - t_s or 1 by the slot's mode),
// the same arithmetic as set_transmission on the host, rounded to the record's precision.
template <typename Real, int NF>
__global__ void refresh_rec_kernel(int64_t items, const double* __restrict__ g0, const int32_t* __restrict__ mode,
                                   const int8_t* __restrict__ word, const double* __restrict__ t,
                                   int32_t* __restrict__ rec) {
  using RR = Rec<Real, NF>;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items; it += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const int64_t e = it * NF + f;
      const int w = word[e];
      if (w < 0) continue;
      const int32_t md = mode[e];
      const double g = md >= 0 ? g0[e] * t[md] : md == -1 ? g0[e] * 1.0 : g0[e] * (1.0 - t[-md - 2]);
      int32_t* r = rec + it * RR::W + RR::COEF + w * RR::CSTEP;
      if constexpr (sizeof(Real) == 4) {
        r[0] = __float_as_int((float)g);
      } else {
        r[0] = __double2loint(g);
        r[1] = __double2hiint(g);
      }
    }
  }
}

// The transmission-free factors of a transmission plan on the device (once), and the new t
static obte_status upload_transmission(obte_plan plan, const double* t) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  if (!plan->tf_g0.p) {
    const int64_t items = (int64_t)s.n_dir * s.n;
    std::vector<int8_t> word((size_t)items * s.nf, -1);
    parallel_for(items, [&](int64_t it) {
      int k = 0;
      for (int f = 0; f < s.nf; ++f) {
        const int kind = (int)((uint32_t)s.in_idx[it * s.nf + f] >> ITEM_SHIFT);
        if (kind == ITEM_CELL || kind == ITEM_PERIODIC) word[(size_t)it * s.nf + f] = (int8_t)k++;
      }
    });
    OBTE_TRY(upload(plan->tf_g0, s.tf.g0, st));
    OBTE_TRY(upload(plan->tf_mode, s.tf.mode, st));
    OBTE_TRY(upload(plan->tf_word, word, st));
  }
  std::vector<double> tv(t, t + s.n_sides);
  return upload(plan->tf_t, tv, st);
}

__global__ void narrow_kernel(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// `done`: the FP64 tables, refreshed just before (the FP32 refresh then copies P and narrows the contact
// coefficients on the device instead of uploading them again)
template <typename Real>
static obte_status refresh_impl(obte_plan plan, DevSchedule& d, int64_t* bytes, const DevSchedule* done = nullptr) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  if (!d.refreshable) { d.ready = false; return OBTE_OK; }   // rebuilt on next use
  const int64_t items = (int64_t)s.n_dir * s.n;
  // the records' coefficient words, on the device from the transmission-free factors and t
  const int blocks = (int)std::min<int64_t>((items + 255) / 256, (int64_t)plan->ctx->num_sms * 8);
  auto kern = s.nf == 3 ? refresh_rec_kernel<Real, 3> : refresh_rec_kernel<Real, 4>;
  if (s.nf != 3 && s.nf != 4) { d.ready = false; return OBTE_OK; }
  kern<<<blocks, 256, 0, st>>>(items, plan->tf_g0.as<double>(), plan->tf_mode.as<int32_t>(),
                               plan->tf_word.as<int8_t>(), plan->tf_t.as<double>(), d.rec.as<int32_t>());
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  // wall coefficients of the special entries (host, small)
  PhaseTimer th(sizeof(Real) == 4 ? "refresh fp32: walls and uploads" : "refresh fp64: walls and uploads");
  std::vector<double> sr((size_t)d.n_spec * SR, 0.0);
  parallel_for(items, [&](int64_t it) {
    const int32_t sp = d.h_spec[it];
    if (sp < 0) return;
    int j = 0;
    for (int f = 0; f < s.nf; ++f) {
      const int32_t code = s.in_idx[it * s.nf + f];
      if ((int)((uint32_t)code >> ITEM_SHIFT) == ITEM_WALL) sr[(size_t)sp * SR + j++] = s.in_coef[it * s.nf + f];
    }
  });
  const size_t kc_n = std::max<size_t>(s.kcoef.size(), 1);
  const bool reuse = sizeof(Real) == 4 && done && done->Pq.p && d.Pq.bytes == done->Pq.bytes && done->kcoef.p &&
                     d.kcoef.p && d.kcoef.bytes >= kc_n * sizeof(Real) && done->kcoef.bytes >= kc_n * sizeof(double);
  if (reuse) {
    OBTE_CUDA(cudaMemcpyAsync(d.Pq.p, done->Pq.p, s.P.size() * sizeof(double), cudaMemcpyDeviceToDevice, st));
    narrow_kernel<<<(int)std::min<size_t>((kc_n + 255) / 256, 1024), 256, 0, st>>>(
        (int64_t)kc_n, done->kcoef.as<double>(), d.kcoef.as<float>());
    count_launch();
    OBTE_CUDA(cudaGetLastError());
  } else {
    OBTE_CUDA(cudaMemcpyAsync(d.Pq.p, s.P.data(), s.P.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  OBTE_CUDA(wait_stream(st));
  OBTE_TRY(upload_real<Real>(d.sr, sr, st));
  if (!reuse) OBTE_TRY(upload_real<Real>(d.kcoef, s.kcoef, st));
  if (bytes) *bytes += (int64_t)(sr.size() * sizeof(Real) + (reuse ? 0 : s.kcoef.size() * sizeof(Real) + s.P.size() * 8));
  return OBTE_OK;
}

// FNV-1a over the packed tables of one precision, built on the host (no device involved).
namespace {
struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  }
  template <typename V>
  void vec(const V& v) {
    const uint64_t n = v.size();
    bytes(&n, sizeof n);
    if (n) bytes(v.data(), n * sizeof(v[0]));
  }
  void i(int64_t x) { bytes(&x, sizeof x); }
};
}  // namespace

template <typename Real>
static obte_status tables_digest_impl(const Schedule& s, uint64_t* digest) {
  Units un;
  {
    PhaseTimer tu("units");
    build_units(s, un);
  }
  Packed pk;
  {
    PhaseTimer tp("pack");
    OBTE_TRY(pack<Real>(s, un, pk));
  }
  Fnv f;
  f.vec(un.ptr); f.vec(un.off); f.vec(un.n);
  f.vec(pk.rec); f.vec(pk.cellmap); f.vec(pk.si); f.vec(pk.spec); f.vec(pk.P); f.vec(pk.sr);
  f.vec(pk.pf); f.vec(pk.kpf); f.vec(pk.sx); f.vec(pk.ksx); f.vec(pk.kwo);
  f.i(pk.unit_sx); f.i(pk.emax); f.i(pk.pf_pad); f.i(pk.unit_wo); f.i(pk.rows);
  // the schedule's own uploads: contact coefficients, K shifts, wall outputs, periodic sources
  f.vec(s.kcoef); f.vec(s.scoef); f.vec(s.kconst); f.vec(s.kshift); f.vec(s.sshift);
  f.vec(s.wo_wall); f.vec(s.wo_off); f.vec(s.x_cell); f.vec(s.x_base); f.vec(s.ell_B);
  *digest = f.h;
  return OBTE_OK;
}

obte_status tables_digest(obte_plan plan, bool fp32, uint64_t* digest) {
  PhaseTimer timer("tables_digest");
  return fp32 ? tables_digest_impl<float>(plan->sched, digest) : tables_digest_impl<double>(plan->sched, digest);
}

obte_status refresh_tables(obte_plan plan, const double* side_transmission, int64_t* bytes) {
  PhaseTimer timer("refresh_tables");
  if (!plan->d32.ready && !plan->d64.ready) return OBTE_OK;
  {
    PhaseTimer tt("refresh: transmissions to the device");
    OBTE_TRY(upload_transmission(plan, side_transmission));
  }
  if (bytes) *bytes += (int64_t)plan->sched.n_sides * 8;
  if (plan->d64.ready) OBTE_TRY(refresh_impl<double>(plan, plan->d64, bytes));
  if (plan->d32.ready) OBTE_TRY(refresh_impl<float>(plan, plan->d32, bytes, plan->d64.ready ? &plan->d64 : nullptr));
  return OBTE_OK;
}

// 1 / (1 + mfp_m D) for every (direction, chunk, position, MFP of the chunk) of the FP64 tables, D read
// from the packed records (padded MFPs: 1, as their mfp is 0)
template <int NF>
__global__ void rinv_build_kernel(const int32_t* __restrict__ rec, int64_t n, int n_dir, int n_chunks, int mcp,
                                  int n_mfp, const double* __restrict__ mfp, double* __restrict__ out) {
  using RR = Rec<double, NF>;
  const int64_t total = (int64_t)n_dir * n_chunks * n * mcp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % mcp);
    int64_t t = i / mcp;
    const int64_t pos = t % n;
    t /= n;
    const int chunk = (int)(t % n_chunks);
    const int64_t q = t / n_chunks;
    const int m = chunk * mcp + j;
    const int32_t* r = rec + (q * n + pos) * RR::W;
    const double D = __hiloint2double(r[RR::D + 1], r[RR::D]);
    const double L = m < n_mfp ? mfp[m] : 0.0;
    out[i] = 1.0 / (1.0 + L * D);
  }
}

// The FP64 reciprocal table, unless OBTE_SWEEP64_RINV=0 or it would exceed OBTE_SWEEP64_RINV_GB (default 32)
// or device memory (the sweep then divides)
static obte_status build_rinv(obte_plan plan, DevSchedule& d) {
  const Schedule& s = plan->sched;
  if (const char* e = std::getenv("OBTE_SWEEP64_RINV"))
    if (std::atoi(e) == 0) return OBTE_OK;
  double cap_gb = 32.0;
  if (const char* e = std::getenv("OBTE_SWEEP64_RINV_GB")) cap_gb = std::atof(e);
  const int64_t total = (int64_t)s.n_dir * d.n_chunks * s.n * d.mcp;
  if ((double)total * 8.0 > cap_gb * 1e9 || (s.nf != 3 && s.nf != 4)) return OBTE_OK;
  if (d.rinv.alloc((size_t)total * sizeof(double)) != OBTE_OK) {
    cudaGetLastError();
    d.rinv.release();
    return OBTE_OK;            // no room: the sweep divides
  }
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)plan->ctx->num_sms * 16);
  if (s.nf == 3)
    rinv_build_kernel<3><<<blocks, 256, 0, plan->stream>>>(d.rec.as<int32_t>(), s.n, s.n_dir, d.n_chunks, d.mcp,
                                                            s.n_mfp, d.mfp.as<double>(), d.rinv.as<double>());
  else
    rinv_build_kernel<4><<<blocks, 256, 0, plan->stream>>>(d.rec.as<int32_t>(), s.n, s.n_dir, d.n_chunks, d.mcp,
                                                            s.n_mfp, d.mfp.as<double>(), d.rinv.as<double>());
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  return OBTE_OK;
}

obte_status ensure_tables(obte_plan plan, bool fp32) {
  if (!plan->err.p) {
    OBTE_TRY(plan->err.alloc(sizeof(int)));
    OBTE_CUDA(cudaMemsetAsync(plan->err.p, 0, sizeof(int), plan->stream));
  }
  if (fp32) {
    if (!plan->d32.ready) return upload_tables<float>(plan, plan->d32);
  } else {
    if (!plan->d64.ready) {
      OBTE_TRY(upload_tables<double>(plan, plan->d64));
      OBTE_TRY(build_rinv(plan, plan->d64));
    }
  }
  return OBTE_OK;
}

// ---- launch -----------------------------------------------------------------------

// Deterministic reductions requested (OBTE_DETERMINISTIC=1, read per call).
static bool deterministic() {
  const char* e = std::getenv("OBTE_DETERMINISTIC");
  return e && std::atoi(e) != 0;
}

// Tables and partial buffers of the deterministic reductions (plan-level tables once, buffers per precision).
template <typename Real>
static obte_status ensure_det(obte_plan plan, DevSchedule& d) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  const int64_t n = s.n, n_wo = (int64_t)s.wo_wall.size();
  if (plan->det_nce < 0) {
    std::vector<int32_t> inv((size_t)s.n_dir * n);
    parallel_for(s.n_dir, [&](int64_t q) {
      for (int64_t pos = 0; pos < n; ++pos) inv[(size_t)q * n + s.cell[(size_t)q * n + pos]] = (int32_t)pos;
    });
    std::vector<int32_t> wptr(s.nd + 1, 0), went(std::max<int64_t>(n_wo, 1), 0);
    for (int64_t e = 0; e < n_wo; ++e) wptr[s.wo_wall[e] + 1]++;
    for (int64_t w = 0; w < s.nd; ++w) wptr[w + 1] += wptr[w];
    {
      std::vector<int32_t> fill(wptr.begin(), wptr.end() - 1);
      for (int64_t e = 0; e < n_wo; ++e) went[fill[s.wo_wall[e]]++] = (int32_t)e;   // entry order within a wall
    }
    std::vector<int32_t> ceoff(s.n_dir + 1, 0);
    for (int q = 0; q < s.n_dir; ++q) {
      int32_t cnt = 0;
      for (int64_t pos = 0; pos < n; ++pos) cnt += s.contact[(size_t)q * n + pos] >= 0 ? 1 : 0;
      ceoff[q + 1] = ceoff[q] + cnt;
    }
    OBTE_TRY(upload(plan->det_inv, inv, st));
    OBTE_TRY(upload(plan->det_wptr, wptr, st));
    OBTE_TRY(upload(plan->det_went, went, st));
    OBTE_TRY(upload(plan->det_ceoff, ceoff, st));
    plan->det_nce = ceoff[s.n_dir];
  }
  if (!d.det_d.p) {
    const size_t parts = (size_t)s.n_dir * d.n_chunks * n;
    OBTE_TRY(d.det_d.alloc(parts * sizeof(Real)));
    OBTE_TRY(d.det_j.alloc(parts * s.ds * sizeof(Real)));
    OBTE_TRY(d.det_w.alloc((size_t)std::max<int64_t>(n_wo, 1) * d.n_chunks * sizeof(Real)));
    OBTE_TRY(d.det_k.alloc((size_t)std::max<int64_t>(plan->det_nce, 1) * s.m_pad * sizeof(Real)));
    OBTE_TRY(d.det_s.alloc((size_t)std::max<int64_t>(plan->det_nce, 1) * s.m_pad * sizeof(Real)));
    OBTE_TRY(d.det_S.alloc((size_t)s.n_dir * n * sizeof(double)));
    OBTE_TRY(d.det_SJ.alloc((size_t)s.n_dir * n * s.ds * sizeof(double)));
    // wall partials of entries a chunk does not reach (MFPs beyond n_mfp) stay zero
    OBTE_CUDA(cudaMemsetAsync(d.det_w.p, 0, d.det_w.bytes, st));
  }
  return OBTE_OK;
}

template <typename Real, int NF, int G, int KV, bool FINAL, bool DF = false>
static obte_status launch_impl(obte_plan plan, const DevSchedule& d, const double* u_in, double* u_out,
                               bool with_src, double* Jraw, double* K, double* S) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  // the double-float pass chunks the MFPs by its own thread shape (G KV per CTA), not by the tables'
  int n_chunks = d.n_chunks;
  size_t smem = d.smem;
  if (DF) {
    n_chunks = (s.n_mfp + G * KV - 1) / (G * KV);
    smem = SmemLayout<Real>(s.nf, G * KV, d.rows, d.unit_wo, d.pf_pad, d.unit_sx, d.nbuf).total;
    if (smem > plan->ctx->smem_optin) {
      set_error("the double-float sweep front needs more shared memory than one CTA can have");
      return OBTE_ERR_UNSUPPORTED;
    }
  }
  const int64_t total = (int64_t)s.n_dir * s.n;
  const int vblocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)plan->ctx->num_sms * 8);
  sweep_values_kernel<Real><<<vblocks, 256, 0, st>>>(
      d.cellmap.as<int32_t>(), d.Pq.as<double>(), d.spec.as<int32_t>(), d.si.as<int32_t>(),
      d.sr.as<Real>(), u_in, s.n, s.hs.empty() ? nullptr : d.hs.as<double>(), with_src ? 1 : 0, total,
      d.vals.as<Real>());
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  auto kern = bte_sweep_kernel<Real, NF, G, KV, FINAL, DF>;
  // the limit is per kernel, shared by every plan and thread: always the device maximum, so concurrent
  // plans with different footprints cannot lower it under each other's launches
  OBTE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan->ctx->smem_optin));
  SweepParams<Real> p;
  p.n = s.n; p.nd = s.nd; p.n_mfp = s.n_mfp; p.n_dir = s.n_dir; p.ds = s.ds; p.m_pad = s.m_pad;
  p.n_chunks = n_chunks; p.rows = d.rows; p.S = s.max_slots;
  p.emax = d.emax; p.unit_wo = d.unit_wo; p.pf_pad = d.pf_pad; p.nbuf = d.nbuf;
  p.rec = d.rec.as<int32_t>(); p.vals = d.vals.as<Real>();
  p.lev_ptr = d.klev_ptr.as<int32_t>(); p.lev_off = d.klev_off.as<int64_t>(); p.nlev = d.knlev.as<int32_t>();
  p.kwo = d.kwo.as<int32_t>(); p.kpf = d.kpf.as<int32_t>(); p.pf = d.pf.as<int32_t>();
  p.ksx = d.ksx.as<int32_t>(); p.sx = d.sx.as<int32_t>(); p.unit_sx = d.unit_sx;
  p.x_base = plan->x_base_dev.as<int64_t>();
  p.wo_off = d.wo_off.as<int32_t>();
  p.wo_wall = d.wo_wall.as<int32_t>();
  p.mfp = d.mfp.as<Real>(); p.tco = d.tco.as<Real>(); p.sig = d.sig.as<Real>(); p.wo_geo = d.wo_geo.as<Real>();
  p.kcoef = d.kcoef.as<Real>(); p.scoef = d.scoef.as<Real>();
  p.u_in = u_in; p.u_out = u_out; p.Jraw = Jraw; p.K = K; p.S_out = S;
  p.err = plan->err.as<int>();
  p.rinv = (sizeof(Real) == 8 && !DF) ? d.rinv.as<double>() : nullptr;
  p.Xs = FINAL ? plan->xstore : nullptr;
  p.xs_add = plan->xstore_add ? 1 : 0;
  p.Xd = FINAL ? plan->xstore64 : nullptr;
  p.skip_unit = plan->test_skip_unit;
  p.wait_limit = plan->test_wait_limit > 0 ? plan->test_wait_limit : kWaitPolls;
  const bool subset = !FINAL && plan->sweep_cta_map != nullptr;
  // deterministic reductions: full sweeps of the FP32 and FP64 kernels (not the probes' subset sweeps, not the
  // double-float pass)
  const bool det = deterministic() && !subset && !DF;
  p.det = det ? 1 : 0;
  p.dpart = p.jpart = p.wpart = p.kpart = p.spart = nullptr;
  p.n_wo = (int64_t)s.wo_wall.size();
  if (det) {
    OBTE_TRY(ensure_det<Real>(plan, const_cast<DevSchedule&>(d)));
    p.dpart = d.det_d.as<Real>();
    p.jpart = d.det_j.as<Real>();
    p.wpart = d.det_w.as<Real>();
    p.kpart = d.det_k.as<Real>();
    p.spart = d.det_s.as<Real>();
  }
  static const bool index_order = std::getenv("OBTE_SWEEP_NO_LPT") != nullptr;   // plain index order
  // (the double-float pass runs in index order: the launch order table belongs to the tables' chunking)
  p.cta_map = subset ? plan->sweep_cta_map : (index_order || DF ? nullptr : d.lpt.as<int32_t>());
  const int batch = subset && plan->sweep_batch > 1 ? plan->sweep_batch : 1;
  p.n_cta_batch = subset ? plan->sweep_n_cta : 0;
  p.batch_stride = batch > 1 ? plan->sweep_batch_stride : 0;
  const int grid = subset ? plan->sweep_n_cta * batch : s.n_dir * n_chunks;
  kern<<<grid, kUnit * G, smem, st>>>(p);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  if (det) {
    const int nb = plan->ctx->num_sms * 8;
    const int64_t total = (int64_t)s.n_dir * s.n;
    det_pos_sum_kernel<Real><<<(int)std::min<int64_t>((total + 255) / 256, nb), 256, 0, st>>>(
        d.det_d.as<Real>(), FINAL ? d.det_j.as<Real>() : nullptr, n_chunks, s.n, total, s.ds, d.det_S.as<double>(),
        d.det_SJ.as<double>());
    det_elem_sum_kernel<<<(int)std::min<int64_t>((s.n + 255) / 256, nb), 256, 0, st>>>(
        d.det_S.as<double>(), FINAL ? d.det_SJ.as<double>() : nullptr, plan->det_inv.as<int32_t>(), s.n_dir, s.n, s.ds,
        u_out, Jraw);
    count_launch(2);
    if (s.nd > 0) {
      det_wall_sum_kernel<Real><<<(int)std::min<int64_t>((s.nd + 255) / 256, nb), 256, 0, st>>>(
          d.det_w.as<Real>(), n_chunks, p.n_wo, plan->det_wptr.as<int32_t>(), plan->det_went.as<int32_t>(), s.nd,
          u_out + s.n);
      count_launch();
    }
    if (FINAL) {
      const int64_t nk = (int64_t)s.n_mfp * s.n_dir;
      det_contact_sum_kernel<Real><<<(int)std::min<int64_t>((nk + 255) / 256, nb), 256, 0, st>>>(
          d.det_k.as<Real>(), d.det_s.as<Real>(), plan->det_ceoff.as<int32_t>(), s.n_dir, s.n_mfp, s.m_pad, K, S);
      count_launch();
    }
    OBTE_CUDA(cudaGetLastError());
  }
  return OBTE_OK;
}

template <typename Real, int G, int KV>
static obte_status launch_w(obte_plan plan, const DevSchedule& d, const double* u_in, double* u_out, bool with_src,
                            bool final_pass, double* Jraw, double* K, double* S) {
  if (plan->sched.nf == 3) {
    if (final_pass) return launch_impl<Real, 3, G, KV, true>(plan, d, u_in, u_out, with_src, Jraw, K, S);
    return launch_impl<Real, 3, G, KV, false>(plan, d, u_in, u_out, with_src, Jraw, K, S);
  }
  if (final_pass) return launch_impl<Real, 4, G, KV, true>(plan, d, u_in, u_out, with_src, Jraw, K, S);
  return launch_impl<Real, 4, G, KV, false>(plan, d, u_in, u_out, with_src, Jraw, K, S);
}

obte_status launch_sweep(obte_plan plan, bool fp32, const double* u_in, double* u_out, bool with_src,
                         bool final_pass, double* Jraw, double* K, double* S) {
  OBTE_TRY(ensure_tables(plan, fp32));
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  if (s.ds > 3) { set_error("sigma with more than 3 components"); return OBTE_ERR_UNSUPPORTED; }
  if (s.nf > 4) { set_error("elements with more than 4 sides are not supported"); return OBTE_ERR_UNSUPPORTED; }
  OBTE_CUDA(cudaMemsetAsync(u_out, 0, (size_t)(s.n + s.nd) * sizeof(double), st));
  if (final_pass) OBTE_CUDA(cudaMemsetAsync(Jraw, 0, (size_t)s.n * s.ds * sizeof(double), st));
  const DevSchedule& d = fp32 ? plan->d32 : plan->d64;
#define OBTE_W(R, GG, KK) \
  if (d.G == GG && d.KV == KK) return launch_w<R, GG, KK>(plan, d, u_in, u_out, with_src, final_pass, Jraw, K, S)
  if (fp32) {
    OBTE_W(float, 1, 4); OBTE_W(float, 1, 8); OBTE_W(float, 2, 4); OBTE_W(float, 1, 2);
  } else {
    OBTE_W(double, 1, 2); OBTE_W(double, 1, 4); OBTE_W(double, 2, 2);
  }
#undef OBTE_W
  set_error("no compiled sweep kernel for this thread shape");
  return OBTE_ERR_UNSUPPORTED;
}

// The output pass in double-float arithmetic on the FP64 tables (J, K and S accumulated like a final pass).
obte_status launch_sweep_df(obte_plan plan, const double* u_in, double* u_out, bool with_src, double* Jraw, double* K,
                            double* S) {
  OBTE_TRY(ensure_tables(plan, false));
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  if (s.ds > 3) { set_error("sigma with more than 3 components"); return OBTE_ERR_UNSUPPORTED; }
  if (s.nf > 4) { set_error("elements with more than 4 sides are not supported"); return OBTE_ERR_UNSUPPORTED; }
  OBTE_CUDA(cudaMemsetAsync(u_out, 0, (size_t)(s.n + s.nd) * sizeof(double), st));
  OBTE_CUDA(cudaMemsetAsync(Jraw, 0, (size_t)s.n * s.ds * sizeof(double), st));
  const DevSchedule& d = plan->d64;
  if (s.nf == 3) return launch_impl<double, 3, 1, 4, true, true>(plan, d, u_in, u_out, with_src, Jraw, K, S);
  return launch_impl<double, 4, 1, 4, true, true>(plan, d, u_in, u_out, with_src, Jraw, K, S);
}

// Device error word: nonzero after a bounded wait gave up (cleared on read).
obte_status check_device_error(obte_plan plan) {
  if (!plan->err.p) return OBTE_OK;
  int h = 0;
  OBTE_CUDA(cudaMemcpyAsync(&h, plan->err.p, sizeof(int), cudaMemcpyDeviceToHost, plan->stream));
  OBTE_CUDA(wait_stream(plan->stream));
  if (h) {
    OBTE_CUDA(cudaMemsetAsync(plan->err.p, 0, sizeof(int), plan->stream));
    set_error("a device-side wait timed out in the sweep kernel");
    return OBTE_ERR_DEVICE_TIMEOUT;
  }
  return OBTE_OK;
}

}  // namespace obte

// ---- sweep on library-owned static scratch ---------------------------------------------
//
// obte_bte_sweep keeps its per-sweep scratch (the (b, p) values the sweep kernel streams by
// TMA, and the device error word) in buffers the plan allocates on first use.  Some callers
// cannot allocate device memory when they sweep: a host framework that has reserved nearly
// all of the GPU's memory for its own pool (cudaMalloc then fails or forces that pool to give
// memory back), or a latency-bound loop in which cudaMalloc / cudaFree would synchronise the
// device and stall work on other streams.  obte_bte_sweep_static runs the same two kernels
// with that scratch in the fixed array below instead, and allocates nothing.
//
// The array is a file-scope __device__ variable: every GPU that loads this library holds
// kStaticScratchBytes of it until the process exits.  Its name in host code is only a
// host-side stand-in, so host code passes the kernels the device address that
// cudaGetSymbolAddress returns, looked up once per device (with that device current) on
// the first call on that device.  Layout: [0, 256) device error word, [256, ...) the values.
// All calls share the array, and it keeps the previous call's contents; each call clears
// the error word before its kernels run, and the values are written in full by
// sweep_values_kernel before the sweep kernel reads them.
namespace obte {

static constexpr size_t kStaticScratchBytes = (size_t)8 << 20;
static constexpr size_t kStaticValsOffset = 256;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_addr[kMaxDevices] = {};
}  // namespace

// Device address of g_static_scratch on `device`, which must be the current device.
static obte_status static_scratch_address(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) { set_error("device ordinal out of range"); return OBTE_ERR_BAD_ARG; }
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[device]) {
    void* p = nullptr;
    OBTE_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
    g_static_addr[device] = p;
  }
  *out = g_static_addr[device];
  return OBTE_OK;
}

template <typename Real, int NF, int G, int KV>
static obte_status launch_static_impl(obte_plan plan, const DevSchedule& d, const double* u_in, double* u_out,
                                      bool with_src, Real* vals, int* err) {
  const Schedule& s = plan->sched;
  cudaStream_t st = plan->stream;
  const int64_t total = (int64_t)s.n_dir * s.n;
  const int vblocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)plan->ctx->num_sms * 8);
  sweep_values_kernel<Real><<<vblocks, 256, 0, st>>>(
      d.cellmap.as<int32_t>(), d.Pq.as<double>(), d.spec.as<int32_t>(), d.si.as<int32_t>(), d.sr.as<Real>(), u_in,
      s.n, s.hs.empty() ? nullptr : d.hs.as<double>(), with_src ? 1 : 0, total, vals);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  auto kern = bte_sweep_kernel<Real, NF, G, KV, false>;
  OBTE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan->ctx->smem_optin));
  SweepParams<Real> p;
  p.n = s.n; p.nd = s.nd; p.n_mfp = s.n_mfp; p.n_dir = s.n_dir; p.ds = s.ds; p.m_pad = s.m_pad;
  p.n_chunks = d.n_chunks; p.rows = d.rows; p.S = s.max_slots;
  p.emax = d.emax; p.unit_wo = d.unit_wo; p.pf_pad = d.pf_pad; p.nbuf = d.nbuf;
  p.rec = d.rec.as<int32_t>(); p.vals = vals;
  p.lev_ptr = d.klev_ptr.as<int32_t>(); p.lev_off = d.klev_off.as<int64_t>(); p.nlev = d.knlev.as<int32_t>();
  p.kwo = d.kwo.as<int32_t>(); p.kpf = d.kpf.as<int32_t>(); p.pf = d.pf.as<int32_t>();
  p.ksx = d.ksx.as<int32_t>(); p.sx = d.sx.as<int32_t>(); p.unit_sx = d.unit_sx;
  p.x_base = plan->x_base_dev.as<int64_t>();
  p.wo_off = d.wo_off.as<int32_t>();
  p.wo_wall = d.wo_wall.as<int32_t>();
  p.mfp = d.mfp.as<Real>(); p.tco = d.tco.as<Real>(); p.sig = d.sig.as<Real>(); p.wo_geo = d.wo_geo.as<Real>();
  p.kcoef = d.kcoef.as<Real>(); p.scoef = d.scoef.as<Real>();
  p.u_in = u_in; p.u_out = u_out; p.Jraw = nullptr; p.K = nullptr; p.S_out = nullptr;
  p.err = err;
  p.Xs = nullptr;
  p.xs_add = 0;
  p.rinv = nullptr;
  p.Xd = nullptr;
  // the launch order of obte_bte_sweep: longest chains first (FP32 tables), unless OBTE_SWEEP_NO_LPT is set
  static const bool index_order = std::getenv("OBTE_SWEEP_NO_LPT") != nullptr;
  p.cta_map = index_order ? nullptr : d.lpt.as<int32_t>();
  p.n_cta_batch = 0;
  p.batch_stride = 0;
  p.skip_unit = -1;
  p.wait_limit = kWaitPolls;
  p.det = 0;
  p.dpart = p.jpart = p.wpart = p.kpart = p.spart = nullptr;
  p.n_wo = 0;
  kern<<<s.n_dir * d.n_chunks, kUnit * G, d.smem, st>>>(p);
  count_launch();
  OBTE_CUDA(cudaGetLastError());
  return OBTE_OK;
}

template <typename Real, int G, int KV>
static obte_status launch_static_w(obte_plan plan, const DevSchedule& d, const double* u_in, double* u_out,
                                   bool with_src, Real* vals, int* err) {
  if (plan->sched.nf == 3) return launch_static_impl<Real, 3, G, KV>(plan, d, u_in, u_out, with_src, vals, err);
  return launch_static_impl<Real, 4, G, KV>(plan, d, u_in, u_out, with_src, vals, err);
}

// Runs with the plan's device current; the caller restores its own.
static obte_status sweep_static_on_device(obte_plan plan, bool fp32, const double* u_in, double* u_out,
                                          bool with_src) {
  const Schedule& s = plan->sched;
  const DevSchedule& d = fp32 ? plan->d32 : plan->d64;
  cudaStream_t st = plan->stream;
  void* base = nullptr;
  OBTE_TRY(static_scratch_address(plan->ctx->device, &base));
  int* err = static_cast<int*>(base);
  void* vals = static_cast<unsigned char*>(base) + kStaticValsOffset;
  OBTE_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  OBTE_CUDA(cudaMemsetAsync(u_out, 0, (size_t)(s.n + s.nd) * sizeof(double), st));
  obte_status rc = OBTE_ERR_UNSUPPORTED;
#define OBTE_SW(R, GG, KK) \
  if (d.G == GG && d.KV == KK) rc = launch_static_w<R, GG, KK>(plan, d, u_in, u_out, with_src, static_cast<R*>(vals), err)
  if (fp32) {
    OBTE_SW(float, 1, 4); else OBTE_SW(float, 1, 8); else OBTE_SW(float, 2, 4); else OBTE_SW(float, 1, 2);
  } else {
    OBTE_SW(double, 1, 2); else OBTE_SW(double, 1, 4); else OBTE_SW(double, 2, 2);
  }
#undef OBTE_SW
  if (rc == OBTE_ERR_UNSUPPORTED) set_error("no compiled sweep kernel for this thread shape");
  if (rc != OBTE_OK) return rc;
  int h = 0;
  OBTE_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  OBTE_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("a device-side wait timed out in the sweep kernel");
    return OBTE_ERR_DEVICE_TIMEOUT;
  }
  return OBTE_OK;
}

}  // namespace obte

using namespace obte;

extern "C" obte_status obte_bte_sweep_static(obte_plan plan, int32_t precision, const double* u_in, double* u_out,
                                             int32_t with_source) {
  if (!plan || !u_in || !u_out) { set_error("null argument"); return OBTE_ERR_BAD_ARG; }
  if (!plan->ctx) { set_error("host-only plan cannot sweep"); return OBTE_ERR_BAD_ARG; }
  if (precision != OBTE_FP64 && precision != OBTE_FP32 && precision != OBTE_FP32_REFINE) {
    set_error("bad precision"); return OBTE_ERR_BAD_ARG;
  }
  const Schedule& s = plan->sched;
  const bool fp32 = precision != OBTE_FP64;
  const size_t need = kStaticValsOffset + (size_t)s.n_dir * (size_t)s.n * 2 * (fp32 ? sizeof(float) : sizeof(double)) + 32;
  if (need > kStaticScratchBytes) {
    set_error("obte_bte_sweep_static: this problem needs " + std::to_string(need) + " bytes of scratch (n_dir x n_elems x " +
              std::to_string(fp32 ? 8 : 16) + " + 288), more than the " + std::to_string(kStaticScratchBytes) +
              " bytes of static scratch the library holds; use obte_bte_sweep");
    return OBTE_ERR_UNSUPPORTED;
  }
  if (s.ds > 3) { set_error("sigma with more than 3 components"); return OBTE_ERR_UNSUPPORTED; }
  if (s.nf > 4) { set_error("elements with more than 4 sides are not supported"); return OBTE_ERR_UNSUPPORTED; }
  if (!(fp32 ? plan->d32.ready : plan->d64.ready)) {
    set_error("obte_bte_sweep_static: the plan's device tables for this precision are not built yet; building them "
              "allocates, so run obte_bte_sweep or obte_bte_solve once in this precision at set-up");
    return OBTE_ERR_BAD_ARG;
  }
  int prev = -1;
  OBTE_CUDA(cudaGetDevice(&prev));
  if (prev != plan->ctx->device) OBTE_CUDA(cudaSetDevice(plan->ctx->device));
  const obte_status rc = sweep_static_on_device(plan, fp32, u_in, u_out, with_source != 0);
  if (prev != plan->ctx->device) {
    const cudaError_t e = cudaSetDevice(prev);
    if (rc == OBTE_OK && e != cudaSuccess) return cuda_fail(e, "cudaSetDevice", __FILE__, __LINE__);
  }
  return rc;
}
