// Host construction of the per-direction sweep schedule.
//
// For every direction q this restates the operator preparation of the
// reference (openbte/bte.py:47-158) on directed faces, then orders the
// elements for an upwind sweep:
//   * directed internal faces carry k = ±(n A)/V (bte.py:48-54); the
//     coefficient g = s_q·k splits into outflow (D, bte.py:59-62) and inflow;
//   * inflow across a kept periodic side is *cut*: its upstream value becomes
//     an interface unknown (periodic source cell) instead of a graph edge;
//   * the remaining inflow edges form a DAG (checked); elements are layered by
//     longest path from the sources and ordered by (level, element id);
//   * each element that feeds a later element gets a slot in a ring of
//     shared-memory rows that is recycled once its last consumer's level is done.
// Directions are independent: they are built by a pool of host threads into
// per-direction buffers and merged in direction order, so the result does not
// depend on the thread count.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <cstdlib>
#include <thread>
#include <unordered_map>

#include "internal.h"

namespace obte {

namespace {

bool in_range(int64_t v, int64_t n) { return v >= 0 && v < n; }

}  // namespace

obte_status build_schedule(const obte_problem* pb, const obte_material* mt, Schedule& s) {
  PhaseTimer timer("build_schedule");
  if (!pb || !mt) { set_error("null problem/material"); return OBTE_ERR_BAD_ARG; }
  const int dim = pb->dim;
  if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3"); return OBTE_ERR_BAD_ARG; }
  const int64_t n = pb->n_elems;
  const int64_t ns = pb->n_sides;
  if (n <= 0 || ns <= 0 || n >= (1LL << 30)) { set_error("bad element/side count"); return OBTE_ERR_BAD_ARG; }
  if (pb->elem_nv < dim + 1 || pb->elem_nv > 7) { set_error("bad elem_nv"); return OBTE_ERR_BAD_ARG; }
  if (!pb->side_elem_map || !pb->normal_areas || !pb->elem_volumes || !pb->internal) {
    set_error("missing mesh arrays"); return OBTE_ERR_BAD_ARG;
  }
  const int n_mfp = mt->n_mfp, n_dir = mt->n_dir;
  if (n_mfp <= 0 || n_dir <= 0 || mt->dim_dir < dim || mt->dim_sigma < dim || !mt->mfps || !mt->vmfp ||
      !mt->sigma || !mt->t_coeff) {
    set_error("bad material"); return OBTE_ERR_BAD_ARG;
  }
  if (pb->is_nanowire && mt->dim_dir < 3) { set_error("nanowire needs 3 direction components"); return OBTE_ERR_BAD_ARG; }
  const int nf = pb->elem_nv;
  const int64_t* sem = pb->side_elem_map;
  const double* na = pb->normal_areas;
  const double* vol = pb->elem_volumes;
  for (int64_t k = 0; k < 2 * ns; ++k)
    if (!in_range(sem[k], n)) { set_error("side_elem_map out of range"); return OBTE_ERR_BAD_ARG; }
  for (int64_t e = 0; e < n; ++e)
    if (!(vol[e] > 0)) { set_error("non-positive element volume"); return OBTE_ERR_BAD_ARG; }

  s.dim = dim; s.nf = nf; s.n = n; s.n_dir = n_dir; s.n_mfp = n_mfp;
  s.n_chunks = (n_mfp + 31) / 32; s.m_pad = s.n_chunks * 32; s.ds = mt->dim_sigma;
  const int m_pad = s.m_pad, ds = s.ds, dd = mt->dim_dir;

  // ---- directed internal faces (bte.py:48-54) ----
  const int64_t ni = pb->n_internal;
  std::vector<char> is_per(ns, 0);
  for (int64_t k = 0; k < pb->n_periodic; ++k) {
    if (!in_range(pb->periodic_sides[k], ns)) { set_error("periodic side out of range"); return OBTE_ERR_BAD_ARG; }
    is_per[pb->periodic_sides[k]] = 1;
  }
  const int64_t nfd = 2 * ni;
  // side transmission (transmission-interface model); 1 = plain internal side
  std::vector<double> t_side(ns, 1.0);
  if (pb->side_transmission) {
    for (int64_t k = 0; k < ns; ++k) {
      const double t = pb->side_transmission[k];
      if (!(t > 0 && t <= 1)) { set_error("side transmission outside (0, 1]"); return OBTE_ERR_BAD_ARG; }
      t_side[k] = t;
    }
  }
  const bool reflect = pb->reflect_internal != 0;
  // transmission plans keep the transmission-free factors of their coefficients (set_transmission)
  const bool keep_tf = pb->side_transmission != nullptr && pb->n_mixed == 0 && !pb->is_nanowire;
  Schedule::TransmissionFactors& tf = s.tf;
  tf = Schedule::TransmissionFactors();
  tf.ok = keep_tf;
  tf.contact_kind = pb->contact_kind;
  std::vector<int32_t> f_row(nfd), f_nb(nfd);
  std::vector<char> f_cut(nfd);
  std::vector<double> f_k(nfd * dim), f_t(nfd);
  for (int64_t t = 0; t < ni; ++t) {
    const int64_t sd = pb->internal[t];
    if (!in_range(sd, ns)) { set_error("internal side out of range"); return OBTE_ERR_BAD_ARG; }
    const int64_t i = sem[2 * sd], j = sem[2 * sd + 1];
    if (i == j) { set_error("internal side with a single element"); return OBTE_ERR_BAD_ARG; }
    f_row[t] = (int32_t)i; f_nb[t] = (int32_t)j; f_cut[t] = is_per[sd];
    f_row[ni + t] = (int32_t)j; f_nb[ni + t] = (int32_t)i; f_cut[ni + t] = is_per[sd];
    f_t[t] = f_t[ni + t] = t_side[sd];
    for (int d = 0; d < dim; ++d) {
      f_k[t * dim + d] = na[sd * dim + d] / vol[i];
      f_k[(ni + t) * dim + d] = -na[sd * dim + d] / vol[j];
    }
  }
  // ---- walls: diffuse walls, then (reflect) one reflecting wall per directed internal face ----
  //   w_db = area vector / volume of the wall's element; w_na = area vector; w_scale scales the
  //   inflow (1 for diffuse walls, 1 - t for reflection); only diffuse walls take outflow into D
  const int64_t nd0 = pb->n_diffuse;
  const int64_t nd = nd0 + (reflect ? nfd : 0);
  s.nd = nd;
  std::vector<int32_t> w_cell(nd);
  std::vector<double> w_db(nd * dim), w_na(nd * dim), w_scale(nd, 1.0);
  for (int64_t w = 0; w < nd0; ++w) {
    const int64_t sd = pb->diffuse_sides[w];
    if (!in_range(sd, ns)) { set_error("diffuse side out of range"); return OBTE_ERR_BAD_ARG; }
    const int64_t i = sem[2 * sd];
    w_cell[w] = (int32_t)i;
    for (int d = 0; d < dim; ++d) {
      w_db[w * dim + d] = na[sd * dim + d] / vol[i];
      w_na[w * dim + d] = na[sd * dim + d];
    }
  }
  if (reflect)
    for (int64_t f = 0; f < nfd; ++f) {
      const int64_t w = nd0 + f;
      const int64_t sd = pb->internal[f % ni];
      const double sg = f < ni ? 1.0 : -1.0;
      w_cell[w] = f_row[f];
      w_scale[w] = 1.0 - f_t[f];
      for (int d = 0; d < dim; ++d) {
        w_db[w * dim + d] = f_k[f * dim + d];
        w_na[w * dim + d] = sg * na[sd * dim + d];
      }
    }
  s.diffuse_cell = w_cell;
  // re-emission weights GG (bte.py:73-78): -GG[m,q,w] = Gbp / (-sum_mq Gbm)
  std::vector<double> gbm_sum(nd, 0.0);
  auto gb_of = [&](int m, int q, int64_t w) {
    double v = 0;
    for (int d = 0; d < dim; ++d) v += mt->sigma[((int64_t)m * n_dir + q) * ds + d] * w_db[w * dim + d];
    return v;
  };
  // Walls with the same w_db vector (bit for bit) have the same sigma . w_db products: on structured
  // grids a handful of vectors cover every wall of the transmission-interface model (4 on a pixel
  // grid against 2 x 32,768 walls), so the sums over (m, q) are taken once per distinct vector.
  // key_out[k * n_dir + q]: some MFP of direction q leaves through walls of vector k (re-emission).
  std::vector<int32_t> w_key(nd);
  std::vector<int64_t> key_wall;
  {
    struct KeyHash {
      size_t operator()(const std::array<uint64_t, 3>& a) const {
        uint64_t h = 0x9e3779b97f4a7c15ull;
        for (uint64_t v : a) h = (h ^ v) * 0x100000001b3ull + (h >> 29);
        return (size_t)h;
      }
    };
    std::unordered_map<std::array<uint64_t, 3>, int32_t, KeyHash> idx;
    for (int64_t w = 0; w < nd; ++w) {
      std::array<uint64_t, 3> k{0, 0, 0};
      std::memcpy(k.data(), &w_db[w * dim], dim * sizeof(double));
      auto it = idx.emplace(k, (int32_t)key_wall.size());
      if (it.second) key_wall.push_back(w);
      w_key[w] = it.first->second;
    }
  }
  const int64_t n_key = (int64_t)key_wall.size();
  std::vector<double> key_gbm(n_key);
  std::vector<char> key_out((size_t)n_key * n_dir);
  parallel_for(n_key, [&](int64_t k) {
    const int64_t w = key_wall[k];
    double acc = 0;
    for (int m = 0; m < n_mfp; ++m)
      for (int q = 0; q < n_dir; ++q) acc += std::min(gb_of(m, q, w), 0.0);
    key_gbm[k] = acc;
    for (int q = 0; q < n_dir; ++q) {
      bool any = false;
      for (int m = 0; m < n_mfp && !any; ++m) any = gb_of(m, q, w) > 0;
      key_out[(size_t)k * n_dir + q] = any;
    }
  });
  for (int64_t w = 0; w < nd; ++w) gbm_sum[w] = key_gbm[w_key[w]];
  s.w_db = w_db;
  s.gbm_sum = gbm_sum;
  // ---- contact (bte.py:132-158) ----
  std::vector<int32_t> c_e1, c_e2;
  std::vector<double> c_na;  // [nc * dim]
  std::vector<double> c_area, c_t;   // c_t: transmission of the contact side (heat flux across it scales by t)
  const int ck = pb->contact_kind;
  const double nrm = pb->normalization;
  if (ck == OBTE_CONTACT_PERIODIC || ck == OBTE_CONTACT_MIXED) {
    for (int64_t k = 0; k < pb->n_contact; ++k) {
      const int64_t sd = pb->contact_sides[k];
      if (!in_range(sd, ns)) { set_error("contact side out of range"); return OBTE_ERR_BAD_ARG; }
      c_e1.push_back((int32_t)sem[2 * sd]);
      c_e2.push_back(ck == OBTE_CONTACT_PERIODIC ? (int32_t)sem[2 * sd + 1] : -1);
      c_t.push_back(t_side[sd]);
      double a2 = 0;
      for (int d = 0; d < dim; ++d) { c_na.push_back(na[sd * dim + d]); a2 += na[sd * dim + d] * na[sd * dim + d]; }
      c_area.push_back(std::sqrt(a2));
    }
  } else if (ck != OBTE_CONTACT_NONE && ck != OBTE_CONTACT_NANOWIRE) {
    set_error("bad contact kind"); return OBTE_ERR_BAD_ARG;
  }
  if (ck == OBTE_CONTACT_NANOWIRE && ds < 3) { set_error("nanowire contact needs sigma_z"); return OBTE_ERR_BAD_ARG; }
  const int64_t nc = (int64_t)c_e1.size();
  // contact element e -> its (contact side k, role) pairs, role 1 = e1, 2 = e2, in contact-side order:
  // co_k / co_role [co_ptr[e], co_ptr[e + 1])
  std::vector<int32_t> co_ptr(n + 1, 0), co_k, co_role;
  for (int64_t k = 0; k < nc; ++k) {
    co_ptr[c_e1[k] + 1]++;
    if (c_e2[k] >= 0) co_ptr[c_e2[k] + 1]++;
  }
  for (int64_t e = 0; e < n; ++e) co_ptr[e + 1] += co_ptr[e];
  co_k.assign(co_ptr[n], 0);
  co_role.assign(co_ptr[n], 0);
  {
    std::vector<int32_t> fill(co_ptr.begin(), co_ptr.end() - 1);
    for (int64_t k = 0; k < nc; ++k) {
      co_k[fill[c_e1[k]]] = (int32_t)k;
      co_role[fill[c_e1[k]]++] = 1;
      if (c_e2[k] >= 0) {
        co_k[fill[c_e2[k]]] = (int32_t)k;
        co_role[fill[c_e2[k]]++] = 2;
      }
    }
  }
  if (keep_tf) {
    for (int64_t k = 0; k < nc; ++k) tf.c_side.push_back((int32_t)pb->contact_sides[k]);
    tf.c_na = c_na;
    tf.co_ptr = co_ptr;
    tf.co_k = co_k;
    tf.co_role = co_role;
  }
  auto sigma_n = [&](int m, int q, int64_t k) {
    double v = 0;
    for (int d = 0; d < dim; ++d) v += mt->sigma[((int64_t)m * n_dir + q) * ds + d] * c_na[k * dim + d];
    return v;
  };

  // ---- per-ordinate tables ----
  s.mfp.assign(m_pad, 0.0);
  for (int m = 0; m < n_mfp; ++m) s.mfp[m] = mt->mfps[m];
  s.tco.assign((size_t)n_dir * m_pad, 0.0);
  s.sig.assign((size_t)n_dir * m_pad * ds, 0.0);
  s.sig_sum.assign(ds, 0.0);
  for (int q = 0; q < n_dir; ++q)
    for (int m = 0; m < n_mfp; ++m) {
      s.tco[(size_t)q * m_pad + m] = mt->t_coeff[(int64_t)m * n_dir + q];
      for (int d = 0; d < ds; ++d) {
        const double v = mt->sigma[((int64_t)m * n_dir + q) * ds + d];
        s.sig[((size_t)q * m_pad + m) * ds + d] = v;
        s.sig_sum[d] += v;
      }
    }
  s.hs.clear();
  if (pb->heat_source) {
    s.hs.resize(n);
    for (int64_t e = 0; e < n; ++e) s.hs[e] = pb->heat_source[e] * mt->heat_source_coeff;
  }
  s.kconst.assign((size_t)n_mfp * n_dir, 0.0);
  s.kshift.assign((size_t)n_mfp * n_dir, 0.0);
  s.sshift.assign((size_t)n_mfp * n_dir, 0.0);
  // offset weights
  s.ell_T.assign(vol, vol + n);
  //   ell_B[w] = w_scale[w] sum_q max(-s_q . A_w, 0) sum_m t_coeff[m, q] mfp_m
  s.ell_B.assign(nd, 0.0);
  {
    std::vector<double> tl_q(n_dir, 0.0);
    for (int q = 0; q < n_dir; ++q)
      for (int m = 0; m < n_mfp; ++m) tl_q[q] += mt->t_coeff[(int64_t)m * n_dir + q] * mt->mfps[m];
    if (keep_tf) {
      tf.ell0.assign(nd, 0.0);
      tf.w_side.assign(nd, -1);
      for (int64_t w = nd0; w < nd; ++w) tf.w_side[w] = (int32_t)pb->internal[(w - nd0) % ni];
    }
    parallel_for(nd, [&](int64_t w) {
      double acc = 0;
      for (int q = 0; q < n_dir; ++q) {
        double sn = 0;
        for (int d = 0; d < dim; ++d) sn += mt->vmfp[(int64_t)q * dd + d] * w_na[w * dim + d];
        if (sn < 0) acc += tl_q[q] * (-sn);
      }
      if (keep_tf) tf.ell0[w] = acc;
      s.ell_B[w] = acc * w_scale[w];
    });
  }


  // transmission-interface tables for the gradient dkappa/dt
  s.n_sides = ns;
  s.dirs.assign((size_t)n_dir * dim, 0.0);
  for (int q = 0; q < n_dir; ++q)
    for (int d = 0; d < dim; ++d) s.dirs[(size_t)q * dim + d] = mt->vmfp[(int64_t)q * dd + d];
  s.tim = pb->side_transmission != nullptr;
  s.contact_alpha = pb->contact_alpha;
  s.extra_sources = pb->n_mixed > 0 || pb->is_nanowire || pb->heat_source != nullptr;
  s.isothermal = pb->n_mixed > 0;

  // diffusion-synthetic acceleration: the cell diffusion operator's faces and coefficients.  Distance
  // from an element's centre to a side: dim V / (sides x area), exact for simplices (the centroid sits
  // at 1 / (dim + 1) of the height over the side) and for squares and cubes.
  {
    Schedule::DsaData& D = s.dsa;
    D = Schedule::DsaData();
    D.vol.assign(vol, vol + n);
    auto side_area = [&](int64_t sd) {
      double a2 = 0;
      for (int d = 0; d < dim; ++d) a2 += na[sd * dim + d] * na[sd * dim + d];
      return std::sqrt(a2);
    };
    auto half = [&](int64_t e, double a) { return (double)dim * vol[e] / ((double)nf * a); };
    D.e1.resize(ni); D.e2.resize(ni); D.side.resize(ni); D.area.resize(ni); D.dist.resize(ni); D.t.resize(ni);
    for (int64_t k = 0; k < ni; ++k) {
      const int64_t sd = pb->internal[k];
      const double a = side_area(sd);
      D.e1[k] = f_row[k];
      D.e2[k] = f_nb[k];
      D.side[k] = (int32_t)sd;
      D.area[k] = a;
      D.dist[k] = a > 0 ? half(f_row[k], a) + half(f_nb[k], a) : 1.0;
      D.t[k] = t_side[sd];
    }
    for (int64_t k = 0; k < pb->n_mixed; ++k) {
      const int64_t sd = pb->mixed_sides[k];
      const double a = side_area(sd);
      if (!(a > 0)) continue;
      D.iso_cell.push_back((int32_t)sem[2 * sd]);
      D.iso_area.push_back(a);
      D.iso_dist.push_back(half(sem[2 * sd], a));
    }
    // isotropic parts: n . (sum_q c_q F_q F_q^T) . n -> sum_q c_q |F_q|^2 / dim and sum_q c_q max(F_q . n, 0)
    // -> sum_q c_q |F_q| <max(cos, 0)> (1 / pi in 2D, 1 / 4 in 3D), F_q = mfp v_q
    const double cmean = dim == 2 ? 1.0 / 3.14159265358979323846 : 0.25;
    D.Dm.assign(n_mfp, 0.0);
    D.Gm.assign(n_mfp, 0.0);
    for (int m = 0; m < n_mfp; ++m)
      for (int q = 0; q < n_dir; ++q) {
        double v2 = 0;
        for (int d = 0; d < dim; ++d) v2 += mt->vmfp[(int64_t)q * dd + d] * mt->vmfp[(int64_t)q * dd + d];
        const double c = mt->t_coeff[(int64_t)m * n_dir + q], L = mt->mfps[m];
        D.Dm[m] += c * L * L * v2 / dim;
        D.Gm[m] += c * L * std::sqrt(v2) * cmean;
      }
  }
  s.normalization = nrm;
  if (s.tim) {
    std::vector<double> jump_of(ns, 0.0);
    for (int64_t k = 0; k < pb->n_periodic; ++k) jump_of[pb->periodic_sides[k]] = pb->periodic_jump[k];
    std::vector<char> is_contact(ns, 0);
    if (ck == OBTE_CONTACT_PERIODIC)
      for (int64_t k = 0; k < pb->n_contact; ++k) is_contact[pb->contact_sides[k]] = 1;
    s.tim_side.resize(ni); s.tim_e1.resize(ni); s.tim_e2.resize(ni); s.tim_w1.resize(ni); s.tim_w2.resize(ni);
    s.tim_na.resize((size_t)ni * dim); s.tim_jump.resize(ni); s.tim_contact.resize(ni);
    for (int64_t t = 0; t < ni; ++t) {
      const int64_t sd = pb->internal[t];
      s.tim_side[t] = (int32_t)sd;
      s.tim_e1[t] = f_row[t];
      s.tim_e2[t] = f_nb[t];
      s.tim_w1[t] = reflect ? (int32_t)(nd0 + t) : -1;
      s.tim_w2[t] = reflect ? (int32_t)(nd0 + ni + t) : -1;
      for (int d = 0; d < dim; ++d) s.tim_na[(size_t)t * dim + d] = na[sd * dim + d];
      s.tim_jump[t] = is_per[sd] ? jump_of[sd] : 0.0;
      s.tim_contact[t] = is_contact[sd];
    }
  }

  // directed faces across kept periodic sides (the only ones whose inflow becomes a periodic source)
  std::vector<int32_t> cut_faces;
  for (int64_t f = 0; f < nfd; ++f)
    if (f_cut[f]) cut_faces.push_back((int32_t)f);

  // mixed sides are validated up front (the per-direction workers do not report errors for them)
  for (int64_t k = 0; k < pb->n_mixed; ++k)
    if (!in_range(pb->mixed_sides[k], ns)) { set_error("mixed side out of range"); return OBTE_ERR_BAD_ARG; }

  // ---- per-direction schedule: directions in parallel, merged in direction order ----
  // uninitialised here: each direction worker initialises and fills its own range
  s.cell.resize((size_t)n_dir * n);
  s.slot.resize((size_t)n_dir * n);
  s.xk.resize((size_t)n_dir * n);
  s.wout.resize((size_t)n_dir * n);
  s.contact.resize((size_t)n_dir * n);
  s.in_idx.resize((size_t)n_dir * n * nf);
  s.in_coef.resize((size_t)n_dir * n * nf);
  s.D.resize((size_t)n_dir * n);
  s.P.resize((size_t)n_dir * n);
  s.nlev.assign(n_dir, 0);
  s.nslots.assign(n_dir, 0);
  if (keep_tf) {
    tf.g0.assign((size_t)n_dir * n * nf, 0.0);
    tf.mode.assign((size_t)n_dir * n * nf, -1);
    const int64_t np = pb->n_periodic;
    tf.per_i.resize(np);
    tf.per_j.resize(np);
    tf.per_side.resize(np);
    for (int64_t k = 0; k < np; ++k) {
      const int64_t sd = pb->periodic_sides[k];
      tf.per_i[k] = (int32_t)sem[2 * sd];
      tf.per_j[k] = (int32_t)sem[2 * sd + 1];
      tf.per_side[k] = (int32_t)sd;
    }
    tf.per_a.assign((size_t)n_dir * np * 2, 0.0);
  }

  struct DirOut {
    std::vector<int32_t> lev, x_cell, wo_wall;
    std::vector<double> kcoef, scoef;
    int nslots = 0;
    obte_status st = OBTE_OK;
    std::string err;
  };
  std::vector<DirOut> outs(n_dir);

  auto build_dir = [&](int q, DirOut& o, std::vector<double>& D, std::vector<double>& P, std::vector<double>& g,
                       std::vector<int32_t>& indeg, std::vector<int32_t>& level, std::vector<int32_t>& order,
                       std::vector<int32_t>& last_use, std::vector<int32_t>& slot_of, std::vector<int64_t>& out_ptr,
                       std::vector<int64_t>& in_ptr, std::vector<int32_t>& out_adj, std::vector<int32_t>& in_face,
                       std::vector<std::vector<int32_t>>& wall_in, std::vector<std::vector<int32_t>>& wall_out,
                       std::vector<int32_t>& src_of) {
    const double* sq = mt->vmfp + (int64_t)q * dd;
    std::fill(D.begin(), D.end(), 0.0);
    std::fill(P.begin(), P.end(), 0.0);
    // internal faces: outflow into D (bte.py:58-62), same accumulation order as the reference
    for (int64_t f = 0; f < nfd; ++f) {
      double v = 0;
      for (int d = 0; d < dim; ++d) v += sq[d] * f_k[f * dim + d];
      g[f] = v;
      if (v > 0) D[f_row[f]] += v;
    }
    // diffuse walls (bte.py:80-84); reflecting walls sit on internal faces, whose outflow is in D already
    for (int64_t w = 0; w < nd0; ++w) {
      double v = 0;
      for (int d = 0; d < dim; ++d) v += sq[d] * w_db[w * dim + d];
      if (v > 0) D[w_cell[w]] += v;
    }
    // mixed walls (bte.py:90-96)
    for (int64_t k = 0; k < pb->n_mixed; ++k) {
      const int64_t sd = pb->mixed_sides[k];
      const int64_t i = sem[2 * sd];
      double v = 0;
      for (int d = 0; d < dim; ++d) v += sq[d] * na[sd * dim + d] / vol[i];
      if (v < 0) P[i] += -v * pb->mixed_value[k];
      if (v > 0) D[i] += v;
    }
    // periodic jump (bte.py:99-110)
    for (int64_t k = 0; k < pb->n_periodic; ++k) {
      const int64_t sd = pb->periodic_sides[k];
      const int64_t i = sem[2 * sd], j = sem[2 * sd + 1];
      const double jump = pb->periodic_jump[k];
      double v1 = 0, v2 = 0;
      for (int d = 0; d < dim; ++d) {
        v1 += sq[d] * na[sd * dim + d] / vol[i];
        v2 += sq[d] * (-na[sd * dim + d]) / vol[j];
      }
      P[i] += -std::min(v1, 0.0) * jump * t_side[sd];
      P[j] += std::min(v2, 0.0) * jump * t_side[sd];
      if (keep_tf) {
        tf.per_a[((size_t)q * pb->n_periodic + k) * 2] = -std::min(v1, 0.0) * jump;
        tf.per_a[((size_t)q * pb->n_periodic + k) * 2 + 1] = std::min(v2, 0.0) * jump;
      }
    }
    if (pb->is_nanowire)
      for (int64_t e = 0; e < n; ++e) P[e] += -sq[2];

    // DAG of uncut inflow edges nb -> row
    std::fill(indeg.begin(), indeg.end(), 0);
    std::fill(out_ptr.begin(), out_ptr.end(), 0);
    std::fill(in_ptr.begin(), in_ptr.end(), 0);
    for (int64_t f = 0; f < nfd; ++f)
      if (g[f] < 0) {
        in_ptr[f_row[f] + 1]++;
        if (!f_cut[f]) { indeg[f_row[f]]++; out_ptr[f_nb[f] + 1]++; }
      }
    for (int64_t e = 0; e < n; ++e) { out_ptr[e + 1] += out_ptr[e]; in_ptr[e + 1] += in_ptr[e]; }
    out_adj.assign(out_ptr[n], 0);
    in_face.assign(in_ptr[n], 0);
    {
      std::vector<int64_t> oc(out_ptr.begin(), out_ptr.end() - 1), ic(in_ptr.begin(), in_ptr.end() - 1);
      for (int64_t f = 0; f < nfd; ++f)
        if (g[f] < 0) {
          in_face[ic[f_row[f]]++] = (int32_t)f;
          if (!f_cut[f]) out_adj[oc[f_nb[f]]++] = f_row[f];
        }
    }
    // Kahn topological order + longest-path levels
    std::vector<int32_t> queue;
    queue.reserve(n);
    for (int64_t e = 0; e < n; ++e) { level[e] = 0; if (indeg[e] == 0) queue.push_back((int32_t)e); }
    for (size_t h = 0; h < queue.size(); ++h) {
      const int32_t c = queue[h];
      for (int64_t k = out_ptr[c]; k < out_ptr[c + 1]; ++k) {
        const int32_t d = out_adj[k];
        level[d] = std::max(level[d], level[c] + 1);
        if (--indeg[d] == 0) queue.push_back(d);
      }
    }
    if ((int64_t)queue.size() != n) {
      o.st = OBTE_ERR_CYCLE;
      o.err = "upwind graph of direction " + std::to_string(q) + " has a cycle not broken by periodic cuts";
      return;
    }
    // elements ordered by (level, element id): a counting sort on the level
    int32_t nl = 0;
    for (int64_t e = 0; e < n; ++e) nl = std::max(nl, level[e] + 1);
    o.lev.assign(nl + 1, 0);
    for (int64_t e = 0; e < n; ++e) o.lev[level[e] + 1]++;
    for (int L = 0; L < nl; ++L) o.lev[L + 1] += o.lev[L];
    {
      std::vector<int32_t> pos(o.lev.begin(), o.lev.end() - 1);
      for (int64_t e = 0; e < n; ++e) order[pos[level[e]]++] = (int32_t)e;
    }

    // periodic source cells of direction q (sorted unique upstream elements of cut inflow)
    std::vector<int32_t>& src = o.x_cell;
    for (int32_t f : cut_faces)
      if (g[f] < 0) src.push_back(f_nb[f]);
    std::sort(src.begin(), src.end());
    src.erase(std::unique(src.begin(), src.end()), src.end());
    for (size_t k = 0; k < src.size(); ++k) src_of[src[k]] = (int32_t)k;   // reset when the direction is done

    // inflow walls / wall outputs per element
    for (int64_t e = 0; e < n; ++e) { wall_in[e].clear(); wall_out[e].clear(); }
    for (int64_t w = 0; w < nd; ++w) {
      double v = 0;
      for (int d = 0; d < dim; ++d) v += sq[d] * w_db[w * dim + d];
      if (v < 0) wall_in[w_cell[w]].push_back((int32_t)w);
      if (key_out[(size_t)w_key[w] * n_dir + q]) wall_out[w_cell[w]].push_back((int32_t)w);
    }

    // slots: an element is alive from its level to the last level of its consumers; elements
    // with per-MFP outputs (periodic source, wall re-emission, contact) hold a slot for their
    // own level so their outputs can be read back after the MFP loop
    for (int64_t e = 0; e < n; ++e) {
      int32_t lu = -1;
      for (int64_t k = out_ptr[e]; k < out_ptr[e + 1]; ++k) lu = std::max(lu, level[out_adj[k]]);
      const bool special = src_of[e] >= 0 || !wall_out[e].empty() || ck == OBTE_CONTACT_NANOWIRE ||
                           co_ptr[e] != co_ptr[e + 1];
      if (special) lu = std::max(lu, level[e]);
      last_use[e] = lu;
      slot_of[e] = -1;
    }
    {
      std::vector<std::vector<int32_t>> release(nl + 1);
      std::vector<int32_t> free_slots;
      int32_t next = 0;
      int64_t p = 0;
      for (int L = 0; L < nl; ++L) {
        for (int32_t sl : release[L]) free_slots.push_back(sl);
        for (; p < n && level[order[p]] == L; ++p) {
          const int32_t e = order[p];
          if (last_use[e] < 0) continue;
          int32_t sl;
          if (!free_slots.empty()) { sl = free_slots.back(); free_slots.pop_back(); }
          else sl = next++;
          slot_of[e] = sl;
          release[last_use[e] + 1].push_back(sl);
        }
      }
      o.nslots = next;
    }

    // items in level order (wout and contact indices local to the direction; rebased on merge)
    const size_t base = (size_t)q * n;
    std::fill(s.xk.begin() + base, s.xk.begin() + base + n, -1);
    std::fill(s.wout.begin() + base, s.wout.begin() + base + n, 0);
    std::fill(s.contact.begin() + base, s.contact.begin() + base + n, -1);
    std::fill(s.in_idx.begin() + base * nf, s.in_idx.begin() + (base + n) * nf, 0);
    std::fill(s.in_coef.begin() + base * nf, s.in_coef.begin() + (base + n) * nf, 0.0);
    for (int64_t p = 0; p < n; ++p) {
      const int32_t e = order[p];
      const size_t it = base + p;
      s.cell[it] = e;
      s.slot[it] = slot_of[e];
      s.D[it] = D[e];
      s.P[it] = P[e];
      int k = 0;
      for (int64_t t = in_ptr[e]; t < in_ptr[e + 1]; ++t) {
        const int32_t f = in_face[t];
        if (k >= nf) { o.st = OBTE_ERR_BAD_ARG; o.err = "more inflow faces than element sides"; return; }
        if (f_cut[f]) s.in_idx[it * nf + k] = pack_item(ITEM_PERIODIC, src_of[f_nb[f]]);
        else s.in_idx[it * nf + k] = pack_item(ITEM_CELL, slot_of[f_nb[f]]);
        s.in_coef[it * nf + k] = g[f] * f_t[f];
        if (keep_tf) {
          tf.g0[it * nf + k] = g[f];
          tf.mode[it * nf + k] = (int32_t)pb->internal[f % ni];
        }
        ++k;
      }
      for (int32_t w : wall_in[e]) {
        if (k >= nf) { o.st = OBTE_ERR_BAD_ARG; o.err = "more inflow faces than element sides"; return; }
        double v = 0;
        for (int d = 0; d < dim; ++d) v += sq[d] * w_db[(int64_t)w * dim + d];
        s.in_idx[it * nf + k] = pack_item(ITEM_WALL, w);
        s.in_coef[it * nf + k] = v * w_scale[w];
        if (keep_tf) {
          tf.g0[it * nf + k] = v;
          tf.mode[it * nf + k] = w < nd0 ? -1 : -((int32_t)pb->internal[(w - nd0) % ni] + 2);
        }
        ++k;
      }
      if (src_of[e] >= 0) s.xk[it] = src_of[e];
      if (!wall_out[e].empty()) {
        const int32_t begin = (int32_t)o.wo_wall.size();
        if (wall_out[e].size() > 7) { o.st = OBTE_ERR_BAD_ARG; o.err = "too many wall sides on one element"; return; }
        for (int32_t w : wall_out[e]) o.wo_wall.push_back(w);
        s.wout[it] = (begin << 3) | (int32_t)wall_out[e].size();
      }
      // contact coefficients
      if (ck == OBTE_CONTACT_NANOWIRE || co_ptr[e] != co_ptr[e + 1]) {
        const int32_t ce = (int32_t)o.scoef.size();
        double sc = 0;
        for (int m = 0; m < m_pad; ++m) {
          double kc = 0;
          if (m < n_mfp) {
            if (ck == OBTE_CONTACT_NANOWIRE) {
              kc = mt->sigma[((int64_t)m * n_dir + q) * ds + 2] * vol[e];
            } else {
              for (int32_t c = co_ptr[e]; c < co_ptr[e + 1]; ++c) {
                const double sn = sigma_n(m, q, co_k[c]);
                kc += (co_role[c] == 1 ? std::max(sn, 0.0) : std::min(sn, 0.0)) * c_t[co_k[c]];
              }
            }
          }
          o.kcoef.push_back(kc * nrm);
        }
        if (ck != OBTE_CONTACT_NANOWIRE)
          for (int32_t c = co_ptr[e]; c < co_ptr[e + 1]; ++c)
            if (co_role[c] == 1) sc += c_area[co_k[c]];
        o.scoef.push_back(sc * nrm);
        s.contact[it] = ce;
        for (int m = 0; m < n_mfp; ++m) {
          s.kshift[(size_t)m * n_dir + q] += o.kcoef[(size_t)ce * m_pad + m];
          s.sshift[(size_t)m * n_dir + q] += sc * nrm;
        }
      }
    }
    // alpha term of K (bte.py:243)
    if (ck == OBTE_CONTACT_PERIODIC || ck == OBTE_CONTACT_MIXED)
      for (int m = 0; m < n_mfp; ++m) {
        double acc = 0;
        for (int64_t k = 0; k < nc; ++k) acc += std::min(sigma_n(m, q, k), 0.0) * c_t[k];
        s.kconst[(size_t)m * n_dir + q] = pb->contact_alpha * acc * nrm;
      }
  };

  int nthreads = (int)std::thread::hardware_concurrency();
  if (const char* env = std::getenv("OBTE_HOST_THREADS")) nthreads = std::atoi(env);
  nthreads = std::max(1, std::min({nthreads, n_dir, 32}));
  auto worker = [&](int tid) {
    std::vector<double> D(n), P(n), g(nfd);
    std::vector<int32_t> indeg(n), level(n), order(n), last_use(n), slot_of(n), out_adj, in_face;
    std::vector<int64_t> out_ptr(n + 1), in_ptr(n + 1);
    std::vector<std::vector<int32_t>> wall_in(n), wall_out(n);
    std::vector<int32_t> src_of(n, -1);   // periodic source index of an element in the current direction
    for (int q = tid; q < n_dir; q += nthreads) {
      build_dir(q, outs[q], D, P, g, indeg, level, order, last_use, slot_of, out_ptr, in_ptr, out_adj, in_face,
                wall_in, wall_out, src_of);
      for (int32_t e : outs[q].x_cell) src_of[e] = -1;
    }
  };
  if (nthreads == 1) {
    worker(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker, t);
    for (auto& th : pool) th.join();
  }

  // merge in direction order
  s.lev_ptr.clear();
  s.lev_off.assign(n_dir, 0);
  s.x_base.assign(n_dir + 1, 0);
  s.x_cell.clear();
  s.wo_wall.clear();
  s.wo_off.assign(n_dir + 1, 0);
  s.kcoef.clear();
  s.scoef.clear();
  s.max_slots = s.max_src = s.max_wo = 0;
  std::vector<int32_t> wo_base(n_dir), ce_base(n_dir);
  for (int q = 0; q < n_dir; ++q) {
    DirOut& o = outs[q];
    if (o.st != OBTE_OK) { set_error(o.err); return o.st; }
    s.lev_off[q] = (int64_t)s.lev_ptr.size();
    s.lev_ptr.insert(s.lev_ptr.end(), o.lev.begin(), o.lev.end());
    s.nlev[q] = (int32_t)o.lev.size() - 1;
    s.nslots[q] = o.nslots;
    s.max_slots = std::max(s.max_slots, o.nslots);
    s.x_base[q + 1] = s.x_base[q] + (int64_t)o.x_cell.size();
    s.x_cell.insert(s.x_cell.end(), o.x_cell.begin(), o.x_cell.end());
    s.max_src = std::max(s.max_src, (int)o.x_cell.size());
    const int32_t wo0 = (int32_t)s.wo_wall.size();
    const int32_t ce0 = (int32_t)s.scoef.size();
    s.wo_off[q] = wo0;
    wo_base[q] = wo0;
    ce_base[q] = ce0;
    s.wo_wall.insert(s.wo_wall.end(), o.wo_wall.begin(), o.wo_wall.end());
    s.kcoef.insert(s.kcoef.end(), o.kcoef.begin(), o.kcoef.end());
    s.scoef.insert(s.scoef.end(), o.scoef.begin(), o.scoef.end());
    s.wo_off[q + 1] = (int32_t)s.wo_wall.size();
    s.max_wo = std::max(s.max_wo, s.wo_off[q + 1] - wo0);
    std::vector<int32_t>().swap(o.lev);
  }
  // wall-output and contact indices from direction-local to global
  parallel_tasks(n_dir, [&](int64_t q) {
    const size_t base = (size_t)q * n;
    const int32_t wo0 = wo_base[q], ce0 = ce_base[q];
    for (int64_t p = 0; p < n; ++p) {
      const size_t it = base + p;
      if (s.wout[it]) s.wout[it] = (((s.wout[it] >> 3) + wo0) << 3) | (s.wout[it] & 7);
      if (s.contact[it] >= 0) s.contact[it] += ce0;
    }
  });
  return OBTE_OK;
}

// New transmissions: every coefficient that depends on t, from the factors kept by build_schedule and
// with the same arithmetic (inflow coefficients bte.py-style g t or g (1 - t), the periodic jump terms
// of P, the contact coefficients with their K shifts and alpha term, the offset weights of the walls).
obte_status set_transmission(Schedule& s, const double* t) {
  PhaseTimer timer("set_transmission");
  if (!t) { set_error("null side transmissions"); return OBTE_ERR_BAD_ARG; }
  if (!s.tim) { set_error("the plan was created without side transmissions"); return OBTE_ERR_BAD_ARG; }
  const Schedule::TransmissionFactors& tf = s.tf;
  if (!tf.ok) {
    set_error("new transmissions need a new plan when the problem has isothermal walls or nanowire terms");
    return OBTE_ERR_UNSUPPORTED;
  }
  for (int64_t k = 0; k < s.n_sides; ++k)
    if (!(t[k] > 0 && t[k] <= 1)) { set_error("side transmission outside (0, 1]"); return OBTE_ERR_BAD_ARG; }
  const int64_t n = s.n;
  const int nf = s.nf, n_dir = s.n_dir, n_mfp = s.n_mfp, m_pad = s.m_pad, ds = s.ds, dim = s.dim;
  parallel_for((int64_t)n_dir * n, [&](int64_t it) {
    for (int k = 0; k < nf; ++k) {
      const size_t e = (size_t)it * nf + k;
      const int32_t md = tf.mode[e];
      s.in_coef[e] = md >= 0 ? tf.g0[e] * t[md] : md == -1 ? tf.g0[e] * 1.0 : tf.g0[e] * (1.0 - t[-md - 2]);
    }
  });
  const int64_t np = (int64_t)tf.per_i.size();
  const int64_t nc = (int64_t)tf.c_side.size();
  const double nrm = s.normalization;
  auto sigma_n = [&](int m, int q, int64_t k) {
    double v = 0;
    for (int d = 0; d < dim; ++d) v += s.sig[((size_t)q * m_pad + m) * ds + d] * tf.c_na[k * dim + d];
    return v;
  };
  std::fill(s.kshift.begin(), s.kshift.end(), 0.0);
  parallel_tasks(n_dir, [&](int64_t qq) {
    const int q = (int)qq;
    std::vector<double> P(n, 0.0);
    for (int64_t k = 0; k < np; ++k) {
      const double tk = t[tf.per_side[k]];
      P[tf.per_i[k]] += tf.per_a[((size_t)q * np + k) * 2] * tk;
      P[tf.per_j[k]] += tf.per_a[((size_t)q * np + k) * 2 + 1] * tk;
    }
    const size_t base = (size_t)q * n;
    for (int64_t p = 0; p < n; ++p) {
      const size_t it = base + p;
      const int32_t e = s.cell[it];
      s.P[it] = P[e];
      const int32_t ce = s.contact[it];
      if (ce < 0) continue;
      for (int m = 0; m < m_pad; ++m) {
        double kc = 0;
        if (m < n_mfp)
          for (int32_t c = tf.co_ptr[e]; c < tf.co_ptr[e + 1]; ++c) {
            const int32_t k = tf.co_k[c];
            const double sn = sigma_n(m, q, k);
            kc += (tf.co_role[c] == 1 ? std::max(sn, 0.0) : std::min(sn, 0.0)) * t[tf.c_side[k]];
          }
        s.kcoef[(size_t)ce * m_pad + m] = kc * nrm;
      }
      for (int m = 0; m < n_mfp; ++m) s.kshift[(size_t)m * n_dir + q] += s.kcoef[(size_t)ce * m_pad + m];
    }
    if (tf.contact_kind == OBTE_CONTACT_PERIODIC || tf.contact_kind == OBTE_CONTACT_MIXED)
      for (int m = 0; m < n_mfp; ++m) {
        double acc = 0;
        for (int64_t k = 0; k < nc; ++k) acc += std::min(sigma_n(m, q, k), 0.0) * t[tf.c_side[k]];
        s.kconst[(size_t)m * n_dir + q] = s.contact_alpha * acc * nrm;
      }
  });
  for (int64_t w = 0; w < s.nd; ++w)
    s.ell_B[w] = tf.ell0[w] * (tf.w_side[w] < 0 ? 1.0 : 1.0 - t[tf.w_side[w]]);
  for (size_t k = 0; k < s.dsa.t.size(); ++k) s.dsa.t[k] = t[s.dsa.side[k]];
  return OBTE_OK;
}

}  // namespace obte
