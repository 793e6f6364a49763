// Host-side set-up of the assembly path (see host_model.hpp).
//
// The sparsity pattern is built row by row from mesh adjacency instead of the
// reference's pre-sized buffer + linear-scan insertion + per-row sort
// (SparseMatrix.cpp:44-114): the SET of registered (i, j) pairs is the same as
// FEStorage::initSolutionData registers (FEStorage.cpp:502-541) --
//   element DoF x node DoF for every node of the element,
//   node DoF x node DoF for every node pair sharing an element (all DoF types
//     registered on both nodes, including the node with itself),
//   element DoF x element DoF of the same element,
//   MPC equation x each term's DoF --
// mapped to the upper triangle and split into block(1) / block(1,2) / block(2)
// exactly as BlockSparseSymMatrix<2>::addEntry does (BlockSparseMatrix.h:139-152).
// Since the reference sorts every row, equal pair sets give bit-identical
// iofeir/columns arrays; the tests compare them against the reference's.
#include "host_model.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>

namespace nla3d_gpu {

namespace {

template <class F>
void parallel_for(uint64_t n, int n_threads, F&& f) {
  if (n == 0) return;
  int nt = n_threads;
  if ((uint64_t)nt > n) nt = (int)n;
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const uint64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    uint64_t b = t * chunk, e = std::min<uint64_t>(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& t : th) t.join();
}

inline int popcount8(uint8_t v) { return __builtin_popcount((unsigned)v); }

}  // namespace

std::vector<LocalPair> element_k_layout(int etype) {
  std::vector<LocalPair> L;
  if (etype == SOLID81) {
    // ElementSOLID81::assemble3 (SOLID81.h:54-94)
    for (int i = 0; i < 8; i++)
      for (int di = 0; di < 3; di++)
        for (int j = i; j < 8; j++)
          for (int dj = 0; dj < 3; dj++) {
            if (i == j && dj < di) continue;
            L.push_back({(int8_t)i, (int8_t)di, (int8_t)j, (int8_t)dj});
          }
    for (int i = 0; i < 8; i++)
      for (int di = 0; di < 3; di++)
        L.push_back({(int8_t)i, (int8_t)di, (int8_t)-1, (int8_t)HYDRO_PRESSURE});
    L.push_back({(int8_t)-1, (int8_t)HYDRO_PRESSURE, (int8_t)-1, (int8_t)HYDRO_PRESSURE});
  } else if (etype == PLANE41) {
    // ElementPLANE41::assembleK (PLANE41.h:54-95): node pairs j >= i, then the
    // two DoFs, the diagonal node blocks by their lower triangle (dj <= di)
    for (int i = 0; i < 4; i++)
      for (int j = i; j < 4; j++)
        for (int di = 0; di < 2; di++)
          for (int dj = 0; dj < 2; dj++) {
            if (i == j && dj > di) continue;
            L.push_back({(int8_t)i, (int8_t)di, (int8_t)j, (int8_t)dj});
          }
    for (int i = 0; i < 4; i++)
      for (int di = 0; di < 2; di++)
        L.push_back({(int8_t)i, (int8_t)di, (int8_t)-1, (int8_t)HYDRO_PRESSURE});
    L.push_back({(int8_t)-1, (int8_t)HYDRO_PRESSURE, (int8_t)-1, (int8_t)HYDRO_PRESSURE});
  } else {
    // Element::assembleK (element.h:281-303, 356-386)
    const int nn = 4;
    const int nd = etype == QUADTH ? 1 : 3;
    for (int i = 0; i < nn; i++)
      for (int di = 0; di < nd; di++)
        for (int j = i; j < nn; j++)
          for (int dj = 0; dj < nd; dj++) {
            if (i == j && dj < di) continue;
            int ti = etype == QUADTH ? TEMP : di, tj = etype == QUADTH ? TEMP : dj;
            L.push_back({(int8_t)i, (int8_t)ti, (int8_t)j, (int8_t)tj});
          }
  }
  return L;
}

std::vector<LocalPair> element_f_layout(int etype) {
  std::vector<LocalPair> L;
  if (etype == SOLID81) {
    for (int i = 0; i < 8; i++)
      for (int di = 0; di < 3; di++) L.push_back({(int8_t)i, (int8_t)di, 0, 0});
    L.push_back({(int8_t)-1, (int8_t)HYDRO_PRESSURE, 0, 0});
  } else if (etype == PLANE41) {
    for (int i = 0; i < 4; i++)
      for (int di = 0; di < 2; di++) L.push_back({(int8_t)i, (int8_t)di, 0, 0});
    L.push_back({(int8_t)-1, (int8_t)HYDRO_PRESSURE, 0, 0});
  } else if (etype == QUADTH) {
    for (int i = 0; i < 4; i++) L.push_back({(int8_t)i, (int8_t)TEMP, 0, 0});
  }
  return L;  // TETRA0 assembles no F from its fresh state (TETRA0.cpp:45-76)
}

std::string build_host_numbering(HostModel& m) {
  const uint32_t N = m.n_nodes, E = m.n_elems;
  if (N < 1 && E < 1) return "No any nodes or elements";
  m.npe = m.etype == SOLID81 ? 8 : 4;
  m.nodal_dofs = m.etype == QUADTH ? 1 : (m.etype == PLANE41 ? 2 : 3);
  for (uint64_t i = 0; i < (uint64_t)E * m.npe; i++)
    if (m.conn[i] < 1 || m.conn[i] > N) return "element connectivity refers to a missing node";

  // ---- DoF registration (Element::pre, RigidBodyMpc::pre) ----
  m.node_mask.assign(N, 0);
  m.elem_mask.assign(E, 0);
  const uint8_t node_bits = m.etype == QUADTH    ? (uint8_t)(1u << TEMP)
                            : m.etype == PLANE41 ? (uint8_t)((1u << UX) | (1u << UY))
                                              : (uint8_t)((1u << UX) | (1u << UY) | (1u << UZ));
  for (uint64_t i = 0; i < (uint64_t)E * m.npe; i++) m.node_mask[m.conn[i] - 1] |= node_bits;
  // SurfaceLINETH::pre (QUADTH.cpp:70-83): TEMP on the line's nodes
  if (m.n_lines() && m.etype != QUADTH) return "surface lines need a QUADTH mesh";
  for (uint32_t n : m.line_conn) {
    if (n < 1 || n > N) return "surface line connectivity refers to a missing node";
    m.node_mask[n - 1] |= (uint8_t)(1u << TEMP);
  }
  if (m.etype == SOLID81 || m.etype == PLANE41)
    for (uint32_t e = 0; e < E; e++) m.elem_mask[e] = (uint8_t)(1u << HYDRO_PRESSURE);
  m.mpcs.clear();
  for (uint32_t r = 0; r < m.rbs.size(); r++) {
    RigidBody& rb = m.rbs[r];
    if (rb.master < 1 || rb.master > N) return "rigid body master node out of range";
    rb.first_mpc = (uint32_t)m.mpcs.size();
    for (uint32_t s : rb.slaves) {
      if (s < 1 || s > N) return "rigid body slave node out of range";
      for (int d : rb.dofs) {
        if (d < UX || d > UZ) return "rigid body slave DoF must be UX, UY or UZ";
        MpcEq q;
        q.node[0] = s; q.dof[0] = d;
        q.node[1] = rb.master; q.dof[1] = d;
        q.node[2] = rb.master; q.dof[2] = ROTX;
        q.node[3] = rb.master; q.dof[3] = ROTY;
        q.node[4] = rb.master; q.dof[4] = ROTZ;
        q.rb = r;
        q.slave = s;
        q.slave_dof = d;
        m.mpcs.push_back(q);
      }
    }
    m.node_mask[rb.master - 1] |= 0x3F;  // UX..ROTZ
  }
  for (const MpcEq& q : m.mpcs)
    if (!(m.node_mask[q.node[0] - 1] & (1u << q.dof[0])))
      return "rigid body slave DoF is not registered by any element";
  for (const LinearMpc& q : m.lmpcs) {
    if (q.node.empty() || q.node.size() != q.dof.size() || q.node.size() != q.coef.size())
      return "linear MPC without terms";
    for (size_t t = 0; t < q.node.size(); t++)
      if (q.node[t] < 1 || q.node[t] > N || q.dof[t] < 0 || q.dof[t] >= kDofTypes ||
          !(m.node_mask[q.node[t] - 1] & (1u << q.dof[t])))
        return "linear MPC term on a DoF that no element or rigid body uses";
  }
  if (m.mpcs.size() + m.lmpcs.size() >= 0xFFFFFFFFull) return "too many MPC equations";
  m.n_mpc = (uint32_t)(m.lmpcs.size() + m.mpcs.size());
  uint64_t nd = 0;
  for (uint32_t n = 0; n < N; n++) nd += popcount8(m.node_mask[n]);
  for (uint32_t e = 0; e < E; e++) nd += popcount8(m.elem_mask[e]);
  if (nd == 0) return "no DoFs registered";
  if (nd + m.n_mpc >= 0xFFFFFFFFull) return "too many equations for 32-bit numbering";
  m.n_dofs = (uint32_t)nd;

  // ---- constraints (FEStorage::setConstrainedNodeDof) ----
  m.node_fix.assign(N, 0);
  m.n_con = 0;
  for (size_t f = 0; f < m.fix_node.size(); f++) {
    uint32_t n = m.fix_node[f];
    int d = m.fix_dof[f];
    if (n < 1 || n > N || d < 0 || d >= kDofTypes || !(m.node_mask[n - 1] & (1u << d)))
      return "constraint on an unregistered DoF";
    if (!(m.node_fix[n - 1] & (1u << d))) {
      m.node_fix[n - 1] |= (uint8_t)(1u << d);
      m.n_con++;
    }
  }
  m.n_unk = m.n_dofs - m.n_con;
  if (m.n_unk == 0) return "no unknown DoFs";

  // ---- equation numbers (FEStorage::assignEquationNumbers, FEStorage.cpp:382-432) ----
  m.node_eq.assign((size_t)N * kDofTypes, 0);
  m.elem_eq.assign((size_t)E * kDofTypes, 0);
  uint32_t next_solve = m.n_con + 1, next_const = 1;
  for (uint32_t e = 0; e < E; e++)
    for (int t = 0; t < kDofTypes; t++)
      if (m.elem_mask[e] & (1u << t)) m.elem_eq[(size_t)e * kDofTypes + t] = next_solve++;
  for (uint32_t n = 0; n < N; n++)
    for (int t = 0; t < kDofTypes; t++)
      if (m.node_mask[n] & (1u << t))
        m.node_eq[(size_t)n * kDofTypes + t] =
            (m.node_fix[n] & (1u << t)) ? next_const++ : next_solve++;
  for (LinearMpc& q : m.lmpcs) q.eq = next_solve++;  // FEStorage.cpp:424-426, list order
  for (MpcEq& q : m.mpcs) q.eq = next_solve++;
  return "";
}

void mpc_extras(const HostModel& m, std::vector<uint32_t>& mpc_ptr,
                std::vector<uint32_t>& mpc_eqs) {
  mpc_ptr.clear();
  mpc_eqs.clear();
  if (!m.n_mpc) return;
  mpc_ptr.assign((size_t)m.n_nodes * kDofTypes + 1, 0);
  for (const MpcEq& q : m.mpcs)
    for (int t = 0; t < 5; t++) mpc_ptr[(size_t)(q.node[t] - 1) * kDofTypes + q.dof[t] + 1]++;
  for (const LinearMpc& q : m.lmpcs)
    for (size_t t = 0; t < q.node.size(); t++)
      mpc_ptr[(size_t)(q.node[t] - 1) * kDofTypes + q.dof[t] + 1]++;
  for (size_t k = 0; k + 1 < mpc_ptr.size(); k++) mpc_ptr[k + 1] += mpc_ptr[k];
  mpc_eqs.resize(mpc_ptr.back());
  std::vector<uint32_t> pos(mpc_ptr.begin(), mpc_ptr.end() - 1);
  for (const MpcEq& q : m.mpcs)
    for (int t = 0; t < 5; t++) mpc_eqs[pos[(size_t)(q.node[t] - 1) * kDofTypes + q.dof[t]]++] = q.eq;
  for (const LinearMpc& q : m.lmpcs)
    for (size_t t = 0; t < q.node.size(); t++)
      mpc_eqs[pos[(size_t)(q.node[t] - 1) * kDofTypes + q.dof[t]]++] = q.eq;
  for (size_t k = 0; k + 1 < mpc_ptr.size(); k++) {
    auto b = mpc_eqs.begin() + mpc_ptr[k], e = mpc_eqs.begin() + mpc_ptr[k + 1];
    std::sort(b, e);  // ascending; duplicates removed at use
  }
}

bool host_slot_of(const HostModel& m, uint32_t i, uint32_t j, uint32_t* out) {
  const uint32_t nc = m.n_con;
  if (i > j) std::swap(i, j);
  int b;
  if (j <= nc) {
    b = 0;
  } else if (i <= nc) {
    b = 1;
    j -= nc;
  } else {
    b = 2;
    i -= nc;
    j -= nc;
  }
  const CsrBlock& B = m.blk[b];
  const uint32_t* beg = B.columns.data() + (B.iofeir[i - 1] - 1);
  const uint32_t* end = B.columns.data() + (B.iofeir[i] - 1);
  const uint32_t* p = std::lower_bound(beg, end, j);
  if (p == end || *p != j) return false;
  *out = (uint32_t)(m.val_off[b] + (uint64_t)(p - B.columns.data()));
  return true;
}

std::string host_mpc_slots(HostModel& m) {
  m.lmpc_slot.clear();
  for (const LinearMpc& q : m.lmpcs)
    for (size_t t = 0; t < q.node.size(); t++) {
      uint32_t sl = 0;
      if (!host_slot_of(m, q.eq, m.neq(q.node[t], q.dof[t]), &sl))
        return "an MPC term has no slot in the CSR pattern";
      m.lmpc_slot.push_back(sl);
    }
  m.mpc_slot.assign(m.mpcs.size() * 5, 0);
  for (uint32_t k = 0; k < (uint32_t)m.mpcs.size(); k++)
    for (int t = 0; t < 5; t++) {
      const MpcEq& q = m.mpcs[k];
      if (!host_slot_of(m, q.eq, m.neq(q.node[t], q.dof[t]), &m.mpc_slot[(size_t)k * 5 + t]))
        return "an MPC term has no slot in the CSR pattern";
    }
  return "";
}

std::string build_host_pattern(HostModel& m, int n_threads) {
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  const uint32_t N = m.n_nodes, E = m.n_elems;

  // ---- node -> element incidence (FEStorage::learnTopology) ----
  std::vector<uint32_t> inc_ptr(N + 1, 0), inc_el;
  for (uint64_t i = 0; i < (uint64_t)E * m.npe; i++) inc_ptr[m.conn[i]]++;
  for (uint32_t n = 0; n < N; n++) inc_ptr[n + 1] += inc_ptr[n];
  inc_el.resize(inc_ptr[N]);
  {
    std::vector<uint32_t> pos(inc_ptr.begin(), inc_ptr.end() - 1);
    for (uint32_t e = 0; e < E; e++)
      for (int a = 0; a < m.npe; a++) {
        uint32_t n = m.conn[(size_t)e * m.npe + a] - 1;
        bool dup = false;
        for (uint32_t k = inc_ptr[n]; k < pos[n]; k++) dup |= inc_el[k] == e + 1;
        if (!dup) inc_el[pos[n]++] = e + 1;
      }
    // compact away duplicate slots (repeated nodes within one element)
    std::vector<uint32_t> np(N + 1, 0), ne;
    ne.reserve(inc_el.size());
    for (uint32_t n = 0; n < N; n++) {
      for (uint32_t k = inc_ptr[n]; k < pos[n]; k++) ne.push_back(inc_el[k]);
      np[n + 1] = (uint32_t)ne.size();
    }
    inc_ptr.swap(np);
    inc_el.swap(ne);
  }

  // ---- MPC equations per (node, dof) ----
  std::vector<uint32_t> mpc_ptr, mpc_eqs;
  mpc_extras(m, mpc_ptr, mpc_eqs);

  // ---- pattern, row by row ----
  const uint32_t nc = m.n_con, ns = m.n_unk + m.n_mpc, ntot = m.n_total();
  // per equation row: counts per destination block
  std::vector<uint32_t> cnt_lo(ntot + 1, 0), cnt_hi(ntot + 1, 0);  // (block1 or block2), block(1,2)

  // node -> surface lines
  const uint32_t Lc = m.n_lines();
  std::vector<uint32_t> lptr(Lc ? N + 1 : 0, 0), lel;
  if (Lc) {
    for (uint32_t n : m.line_conn) lptr[n]++;
    for (uint32_t n = 0; n < N; n++) lptr[n + 1] += lptr[n];
    lel.resize(lptr[N]);
    std::vector<uint32_t> pos(lptr.begin(), lptr.end() - 1);
    for (uint32_t l = 0; l < Lc; l++) lel[pos[m.line_conn[2 * l] - 1]++] = l;
    for (uint32_t l = 0; l < Lc; l++)
      if (m.line_conn[2 * l + 1] != m.line_conn[2 * l]) lel[pos[m.line_conn[2 * l + 1] - 1]++] = l;
  }

  auto node_row_cols = [&](uint32_t n /*1-based*/, std::vector<uint32_t>& cand) {
    cand.clear();
    if (Lc)
      for (uint32_t k = lptr[n - 1]; k < lptr[n]; k++)
        for (int a = 0; a < 2; a++) cand.push_back(m.neq(m.line_conn[2 * lel[k] + a], TEMP));
    for (uint32_t k = inc_ptr[n - 1]; k < inc_ptr[n]; k++) {
      const uint32_t el = inc_el[k];
      for (int t = 0; t < kDofTypes; t++)
        if (m.elem_mask[el - 1] & (1u << t)) cand.push_back(m.eeq(el, t));
      for (int a = 0; a < m.npe; a++) {
        const uint32_t n2 = m.conn[(size_t)(el - 1) * m.npe + a];
        for (int t = 0; t < kDofTypes; t++)
          if (m.node_mask[n2 - 1] & (1u << t)) cand.push_back(m.neq(n2, t));
      }
    }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  };
  auto elem_row_cols = [&](uint32_t el /*1-based*/, std::vector<uint32_t>& cand) {
    cand.clear();
    for (int t = 0; t < kDofTypes; t++)
      if (m.elem_mask[el - 1] & (1u << t)) cand.push_back(m.eeq(el, t));
    for (int a = 0; a < m.npe; a++) {
      const uint32_t n2 = m.conn[(size_t)(el - 1) * m.npe + a];
      for (int t = 0; t < kDofTypes; t++)
        if (m.node_mask[n2 - 1] & (1u << t)) cand.push_back(m.neq(n2, t));
    }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  };
  // emit(row r, sorted candidate columns >= r from `cand`, plus sorted `extra`)
  auto for_row = [&](uint32_t r, const std::vector<uint32_t>& cand, const uint32_t* xb,
                     const uint32_t* xe, bool fill) {
    auto it = std::lower_bound(cand.begin(), cand.end(), r);
    uint32_t lo = 0, hi = 0;
    CsrBlock* B_lo = r <= nc ? &m.blk[0] : &m.blk[2];
    uint32_t* out_lo = nullptr;
    uint32_t* out_hi = nullptr;
    if (fill) {
      const uint32_t row_local = r <= nc ? r : r - nc;
      out_lo = B_lo->columns.data() + (B_lo->iofeir[row_local - 1] - 1);
      if (r <= nc) out_hi = m.blk[1].columns.data() + (m.blk[1].iofeir[r - 1] - 1);
    }
    uint32_t prev = 0;
    auto put = [&](uint32_t c) {
      if (c == prev) return;
      prev = c;
      if (r <= nc) {
        if (c <= nc) {
          if (fill) out_lo[lo] = c;
          lo++;
        } else {
          if (fill) out_hi[hi] = c - nc;
          hi++;
        }
      } else {
        if (fill) out_lo[lo] = c - nc;
        lo++;
      }
    };
    for (; it != cand.end(); ++it) put(*it);
    for (const uint32_t* p = xb; p != xe; ++p)
      if (*p >= r) put(*p);
    if (!fill) {
      cnt_lo[r] = lo;
      cnt_hi[r] = hi;
    }
  };

  auto pattern_pass = [&](bool fill) {
    parallel_for(N, n_threads, [&](uint64_t b, uint64_t e) {
      std::vector<uint32_t> cand;
      for (uint64_t i = b; i < e; i++) {
        const uint32_t n = (uint32_t)i + 1;
        if (!m.node_mask[n - 1]) continue;
        node_row_cols(n, cand);
        for (int t = 0; t < kDofTypes; t++) {
          if (!(m.node_mask[n - 1] & (1u << t))) continue;
          const uint32_t r = m.neq(n, t);
          const uint32_t* xb = nullptr;
          const uint32_t* xe = nullptr;
          if (m.n_mpc) {
            size_t key = (size_t)(n - 1) * kDofTypes + t;
            xb = mpc_eqs.data() + mpc_ptr[key];
            xe = mpc_eqs.data() + mpc_ptr[key + 1];
          }
          for_row(r, cand, xb, xe, fill);
        }
      }
    });
    parallel_for(E, n_threads, [&](uint64_t b, uint64_t e) {
      std::vector<uint32_t> cand;
      for (uint64_t i = b; i < e; i++) {
        const uint32_t el = (uint32_t)i + 1;
        if (!m.elem_mask[el - 1]) continue;
        elem_row_cols(el, cand);
        for (int t = 0; t < kDofTypes; t++)
          if (m.elem_mask[el - 1] & (1u << t)) for_row(m.eeq(el, t), cand, nullptr, nullptr, fill);
      }
    });
  };

  pattern_pass(false);
  // iofeir of the three blocks
  m.blk[0].rows = nc; m.blk[0].cols = nc;
  m.blk[1].rows = nc; m.blk[1].cols = ns;
  m.blk[2].rows = ns; m.blk[2].cols = ns;
  for (int b = 0; b < 3; b++) m.blk[b].iofeir.assign(m.blk[b].rows + 1, 1);
  uint64_t s0 = 0, s1 = 0, s2 = 0;
  for (uint32_t r = 1; r <= ntot; r++) {
    if (r <= nc) {
      s0 += cnt_lo[r];
      s1 += cnt_hi[r];
      m.blk[0].iofeir[r] = (uint32_t)(s0 + 1);
      m.blk[1].iofeir[r] = (uint32_t)(s1 + 1);
    } else {
      s2 += cnt_lo[r];
      m.blk[2].iofeir[r - nc] = (uint32_t)(s2 + 1);
    }
    if (s0 + s1 + s2 >= 0xFFFFFFF0ull) return "K has more than 2^32 nonzeros";
  }
  m.blk[0].columns.assign(s0, 0);
  m.blk[1].columns.assign(s1, 0);
  m.blk[2].columns.assign(s2, 0);
  pattern_pass(true);
  std::vector<uint32_t>().swap(cnt_lo);
  std::vector<uint32_t>().swap(cnt_hi);
  m.val_off[0] = 0;
  m.val_off[1] = s0;
  m.val_off[2] = s0 + s1;
  m.nnz_total = s0 + s1 + s2;

  auto slot_of = [&](uint32_t i, uint32_t j, uint32_t* out) -> bool {
    return host_slot_of(m, i, j, out);
  };

  // ---- element -> slot maps ----
  const std::vector<LocalPair> KL = element_k_layout(m.etype);
  const std::vector<LocalPair> FL = element_f_layout(m.etype);
  m.n_kc = (int)KL.size();
  m.n_fc = (int)FL.size();
  if ((uint64_t)E * (m.n_kc + m.n_fc) + (uint64_t)Lc * (kLineKc + kLineFc) >= 0xFFFFFFF0ull)
    return "too many element contributions";
  std::vector<uint32_t>& kslot = m.kslot;
  std::vector<uint32_t>& fslot = m.fslot;
  // contributions of the lines follow the elements' (the lines are created after them)
  kslot.assign((size_t)E * m.n_kc + (size_t)Lc * kLineKc, 0);
  fslot.assign((size_t)E * m.n_fc + (size_t)Lc * kLineFc, 0);
  std::atomic<int> bad(0);
  parallel_for(E, n_threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; i++) {
      const uint32_t el = (uint32_t)i + 1;
      const uint32_t* c = m.conn.data() + i * m.npe;
      auto eqof = [&](int ent, int t) -> uint32_t {
        return ent < 0 ? m.eeq(el, t) : m.neq(c[ent], t);
      };
      for (int k = 0; k < m.n_kc; k++) {
        const LocalPair& L = KL[k];
        if (!slot_of(eqof(L.ei, L.ti), eqof(L.ej, L.tj), &kslot[i * m.n_kc + k])) bad = 1;
      }
      for (int k = 0; k < m.n_fc; k++) fslot[i * m.n_fc + k] = eqof(FL[k].ei, FL[k].ti) - 1;
    }
  });
  // surface lines: assembleK(MatSym<2>, Vec<2>, {TEMP}) order (element.h:356-386)
  for (uint32_t l = 0; l < Lc; l++) {
    const uint32_t qa = m.neq(m.line_conn[2 * l], TEMP), qb = m.neq(m.line_conn[2 * l + 1], TEMP);
    const uint64_t kb = (uint64_t)E * m.n_kc + (uint64_t)l * kLineKc;
    if (!slot_of(qa, qa, &kslot[kb]) || !slot_of(qa, qb, &kslot[kb + 1]) ||
        !slot_of(qb, qb, &kslot[kb + 2]))
      bad = 1;
    const uint64_t fb = (uint64_t)E * m.n_fc + (uint64_t)l * kLineFc;
    fslot[fb] = qa - 1;
    fslot[fb + 1] = qb - 1;
  }
  if (bad) return "an element contribution has no slot in the CSR pattern";

  // ---- inverse: gather lists in ascending contribution order ----
  auto invert = [&](const std::vector<uint32_t>& slot, uint64_t n_slots, int per_elem,
                    std::vector<uint32_t>& ptr, std::vector<uint32_t>& ids) {
    ptr.assign(n_slots + 1, 0);
    uint32_t* P = ptr.data();
    parallel_for(slot.size(), n_threads, [&](uint64_t b, uint64_t e) {
      for (uint64_t i = b; i < e; i++) __atomic_fetch_add(&P[slot[i] + 1], 1u, __ATOMIC_RELAXED);
    });
    for (uint64_t s = 0; s < n_slots; s++) P[s + 1] += P[s];
    ids.assign(slot.size(), 0);
    std::vector<uint32_t> pos(ptr.begin(), ptr.end() - 1);
    uint32_t* Q = pos.data();
    parallel_for(slot.size(), n_threads, [&](uint64_t b, uint64_t e) {
      for (uint64_t i = b; i < e; i++) {
        uint32_t at = __atomic_fetch_add(&Q[slot[i]], 1u, __ATOMIC_RELAXED);
        ids[at] = (uint32_t)i;  // contribution id = element * per_elem + local
      }
    });
    parallel_for(n_slots, n_threads, [&](uint64_t b, uint64_t e) {
      for (uint64_t s = b; s < e; s++)
        if (P[s + 1] - P[s] > 1) std::sort(ids.begin() + P[s], ids.begin() + P[s + 1]);
    });
    (void)per_elem;
  };
  invert(kslot, m.nnz_total, m.n_kc, m.k_ptr, m.k_ids);
  invert(fslot, ntot, m.n_fc, m.f_ptr, m.f_ids);

  // ---- MPC term slots ----
  return host_mpc_slots(m);
}

std::string build_host_model(HostModel& m, int n_threads) {
  std::string msg = build_host_numbering(m);
  if (!msg.empty()) return msg;
  return build_host_pattern(m, n_threads);
}

}  // namespace nla3d_gpu
