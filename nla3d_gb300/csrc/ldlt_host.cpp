// Symbolic analysis of the supernodal multifrontal LDL^T (host, once per
// pattern).  See ldlt.hpp.
//
// Published methods used: the elimination tree by Liu's algorithm with path
// compression; a depth-first postorder; column counts by walking each row's
// subtree of the elimination tree (Liu, "The role of elimination trees in
// sparse factorization", 1990); fundamental supernodes (a column joins its
// child when it is the only child and the counts differ by one); relaxed
// amalgamation of a child supernode into its parent when the merged front
// stays small or gains few explicit zeros (the thresholds of Ashcraft and
// Grimes' relaxed supernodes as popularised by CHOLMOD: merge when the merged
// supernode has <= 4 columns, <= 16 columns and < 80 % zeros, <= 48 columns
// and < 10 % zeros, or < 5 % zeros).
#include "ldlt.hpp"

#include <algorithm>
#include <atomic>
#include <climits>
#include <thread>

namespace {

// Nested dissection of the rows idx: split at the median of the points'
// longest extent; the rows of the lower half that couple to the upper half
// form the separator, ordered after both halves; leaves of 64 rows.
struct NdState {
  const double* pts;
  const std::vector<int64_t>* ptr;
  const std::vector<int32_t>* adj;
  std::vector<uint8_t> upper;
  std::vector<int32_t> out;
};

void nd_split(NdState& st, std::vector<int32_t>& idx) {
  if (idx.size() <= 64) {
    st.out.insert(st.out.end(), idx.begin(), idx.end());
    return;
  }
  int ax = 0;
  double best = -1.0;
  for (int d = 0; d < 3; d++) {
    double lo = st.pts[3 * (size_t)idx[0] + d], hi = lo;
    for (int32_t r : idx) {
      lo = std::min(lo, st.pts[3 * (size_t)r + d]);
      hi = std::max(hi, st.pts[3 * (size_t)r + d]);
    }
    if (hi - lo > best) {
      best = hi - lo;
      ax = d;
    }
  }
  std::vector<double> x(idx.size());
  for (size_t i = 0; i < idx.size(); i++) x[i] = st.pts[3 * (size_t)idx[i] + ax];
  std::vector<double> sorted = x;
  const size_t mid = sorted.size() / 2;
  std::nth_element(sorted.begin(), sorted.begin() + mid, sorted.end());
  double med = sorted[mid];
  if (sorted.size() % 2 == 0)
    med = 0.5 * (*std::max_element(sorted.begin(), sorted.begin() + mid) + med);
  std::vector<int32_t> lower, up;
  for (size_t i = 0; i < idx.size(); i++) (x[i] < med ? lower : up).push_back(idx[i]);
  if (lower.empty() || up.empty()) {
    st.out.insert(st.out.end(), idx.begin(), idx.end());
    return;
  }
  std::vector<int32_t>().swap(idx);   // the halves hold the rows now
  for (int32_t r : up) st.upper[r] = 1;
  std::vector<int32_t> inner, sep;
  const std::vector<int64_t>& P = *st.ptr;
  const std::vector<int32_t>& A = *st.adj;
  for (int32_t r : lower) {
    bool touch = false;
    for (int64_t q = P[r]; q < P[r + 1] && !touch; q++) touch = st.upper[A[q]] != 0;
    (touch ? sep : inner).push_back(r);
  }
  for (int32_t r : up) st.upper[r] = 0;
  std::vector<int32_t>().swap(lower);
  nd_split(st, inner);
  nd_split(st, up);
  st.out.insert(st.out.end(), sep.begin(), sep.end());
}

}  // namespace

std::string ldlt_nd_order(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                          const double* points, int64_t n_dofs, int32_t* order) {
  if (n <= 0 || n >= INT32_MAX / 2) return "bad size";
  if (!iofeir || !points || !order || iofeir[0] != 1) return "bad argument";
  // both triangles, diagonal excluded
  std::vector<int64_t> ptr(n + 1, 0);
  for (int64_t r = 0; r < n; r++) {
    if (iofeir[r + 1] < iofeir[r]) return "iofeir is not monotone";
    for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
      const int64_t c = (int64_t)columns[q] - 1;
      if (c < r || c >= n) return "not an upper-triangle CSR";
      if (c != r) {
        ptr[r + 1]++;
        ptr[c + 1]++;
      }
    }
  }
  for (int64_t i = 0; i < n; i++) ptr[i + 1] += ptr[i];
  std::vector<int32_t> adj(ptr[n]);
  {
    std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t r = 0; r < n; r++)
      for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
        const int64_t c = (int64_t)columns[q] - 1;
        if (c != r) {
          adj[fill[r]++] = (int32_t)c;
          adj[fill[c]++] = (int32_t)r;
        }
      }
  }
  NdState st{points, &ptr, &adj, std::vector<uint8_t>(n, 0), {}};
  st.out.reserve(n);
  std::vector<int32_t> all(n);
  for (int64_t r = 0; r < n; r++) all[r] = (int32_t)r;
  nd_split(st, all);
  auto has_diag = [&](int64_t r) {
    return iofeir[r + 1] > iofeir[r] && (int64_t)columns[iofeir[r] - 1] == r + 1;
  };
  int64_t k = 0;
  for (int32_t r : st.out)
    if (r < n_dofs && has_diag(r)) order[k++] = r;
  for (int64_t r = std::max<int64_t>(n_dofs, 0); r < n; r++) order[k++] = (int32_t)r;
  for (int32_t r : st.out)
    if (r < n_dofs && !has_diag(r)) order[k++] = r;
  return k == n ? "" : "order is not a permutation";
}

std::string ldlt_analyze(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                         const int32_t* perm_in, LdltSymbolic* out) {
  LdltSymbolic& S = *out;
  S = LdltSymbolic();
  if (n <= 0) return "empty matrix";
  if (n >= INT32_MAX / 2) return "too many equations";
  if (!iofeir || iofeir[0] != 1) return "iofeir[0] must be 1";
  S.n = n;
  const uint64_t nnz = (uint64_t)iofeir[n] - 1;
  S.nnz = nnz;
  if (nnz && !columns) return "null columns";

  // ---- order 0: the caller's permutation ----
  std::vector<int32_t> p0(n), ip0(n, -1);
  for (int64_t i = 0; i < n; i++) p0[i] = perm_in ? perm_in[i] : (int32_t)i;
  for (int64_t i = 0; i < n; i++) {
    if (p0[i] < 0 || p0[i] >= n || ip0[p0[i]] != -1) return "perm is not a permutation";
    ip0[p0[i]] = (int32_t)i;
  }
  // strictly lower entries by row (order 0): row hi holds lo < hi
  std::vector<int64_t> lp(n + 1, 0);
  for (int64_t r = 0; r < n; r++) {
    if (iofeir[r + 1] < iofeir[r]) return "iofeir is not monotone";
    for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
      const int64_t c = (int64_t)columns[q] - 1;
      if (c < r || c >= n) return "not an upper-triangle CSR";
      const int32_t a = ip0[r], b = ip0[c];
      if (a != b) lp[std::max(a, b) + 1]++;
    }
  }
  for (int64_t i = 0; i < n; i++) lp[i + 1] += lp[i];
  std::vector<int32_t> li(lp[n]);
  {
    std::vector<int64_t> fill(lp.begin(), lp.end() - 1);
    for (int64_t r = 0; r < n; r++)
      for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
        const int32_t a = ip0[r], b = ip0[columns[q] - 1];
        if (a != b) li[fill[std::max(a, b)]++] = std::min(a, b);
      }
  }

  // ---- elimination tree (Liu, path compression) ----
  std::vector<int32_t> parent(n, -1);
  {
    std::vector<int32_t> anc(n, -1);
    for (int32_t k = 0; k < n; k++)
      for (int64_t q = lp[k]; q < lp[k + 1]; q++) {
        int32_t r = li[q];
        while (anc[r] != -1 && anc[r] != k) {
          const int32_t nx = anc[r];
          anc[r] = k;
          r = nx;
        }
        if (anc[r] == -1) {
          anc[r] = k;
          parent[r] = k;
        }
      }
  }
  // ---- postorder (children visited in ascending order) ----
  std::vector<int32_t> post(n), ipost(n);
  {
    std::vector<int32_t> head(n, -1), next(n, -1), stack;
    for (int32_t j = (int32_t)n - 1; j >= 0; j--)
      if (parent[j] != -1) {
        next[j] = head[parent[j]];
        head[parent[j]] = j;
      }
    int32_t t = 0;
    for (int32_t j = 0; j < n; j++) {
      if (parent[j] != -1) continue;
      stack.push_back(j);
      while (!stack.empty()) {
        const int32_t p = stack.back();
        const int32_t c = head[p];
        if (c == -1) {
          stack.pop_back();
          post[t++] = p;
        } else {
          head[p] = next[c];
          stack.push_back(c);
        }
      }
    }
    if (t != n) return "elimination tree is not a forest";
    for (int32_t i = 0; i < n; i++) ipost[post[i]] = i;
  }
  // ---- column counts, incl. the diagonal ----
  // c(j) = number of row subtrees T(i) (rows i > j of L) that contain j, plus
  // one.  As in Gilbert, Ng and Peyton ("An efficient algorithm to compute row
  // and column counts for sparse Cholesky factorization", 1994) each count is
  // a subtree sum of weights: +1 at every leaf of a row subtree, -1 at the
  // least common ancestor of consecutive leaves (in postorder) and at the
  // subtree's root i, and 1 - (number of children) for the diagonal.  A
  // column j is a leaf of T(i) when no earlier neighbour of row i lies in j's
  // subtree (first(j) > the last neighbour seen); the ancestors come from a
  // disjoint-set forest merged along the postorder.  Cost O(nnz(A)), where
  // walking every row subtree costs O(nnz(L)).
  std::vector<int64_t> cc(n, 1);
  {
    // upper neighbours of each column (order 0): k > j with A(k, j) != 0
    std::vector<int64_t> up(n + 1, 0);
    for (int32_t k = 0; k < n; k++)
      for (int64_t q = lp[k]; q < lp[k + 1]; q++) up[li[q] + 1]++;
    for (int64_t i = 0; i < n; i++) up[i + 1] += up[i];
    std::vector<int32_t> ui(up[n]);
    {
      std::vector<int64_t> fill(up.begin(), up.end() - 1);
      for (int32_t k = 0; k < n; k++)
        for (int64_t q = lp[k]; q < lp[k + 1]; q++) ui[fill[li[q]]++] = k;
    }
    // everything below in postorder positions
    std::vector<int32_t> pp(n), first(n, -1), prevnbr(n, -1), prevleaf(n, -1), anc(n);
    std::vector<int64_t> w(n, 1);
    for (int32_t t = 0; t < n; t++) {
      const int32_t p = parent[post[t]];
      pp[t] = p == -1 ? -1 : ipost[p];
      anc[t] = t;
    }
    for (int32_t t = 0; t < n; t++)
      if (pp[t] != -1) w[pp[t]]--;
    for (int32_t t = 0; t < n; t++)
      for (int32_t r = t; r != -1 && first[r] == -1; r = pp[r]) first[r] = t;
    for (int32_t t = 0; t < n; t++) {
      const int32_t j = post[t];
      for (int64_t q = up[j]; q < up[j + 1]; q++) {
        const int32_t ip = ipost[ui[q]];
        if (first[t] > prevnbr[ip]) {   // t is a leaf of row ip's subtree
          w[t]++;
          const int32_t pl = prevleaf[ip];
          if (pl == -1) {
            w[ip]--;
          } else {
            int32_t r = pl;
            while (anc[r] != r) r = anc[r];
            for (int32_t x = pl; anc[x] != r;) {
              const int32_t nx = anc[x];
              anc[x] = r;
              x = nx;
            }
            w[r]--;   // the least common ancestor of the previous leaf and t
          }
          prevleaf[ip] = t;
        }
        prevnbr[ip] = t;
      }
      if (pp[t] != -1) anc[t] = pp[t];
    }
    for (int32_t t = 0; t < n; t++)
      if (pp[t] != -1) w[pp[t]] += w[t];
    for (int32_t t = 0; t < n; t++) cc[post[t]] = w[t];
  }
  // ---- order 1: postorder labels ----
  std::vector<int32_t> par1(n), nch1(n, 0);
  std::vector<int64_t> cc1(n);
  for (int32_t t = 0; t < n; t++) {
    const int32_t p = parent[post[t]];
    par1[t] = p == -1 ? -1 : ipost[p];
    cc1[t] = cc[post[t]];
    if (par1[t] != -1) nch1[par1[t]]++;
  }
  // ---- fundamental supernodes ----
  std::vector<int32_t> ffirst;
  for (int32_t t = 0; t < n; t++) {
    const bool join = t > 0 && par1[t - 1] == t && cc1[t - 1] == cc1[t] + 1 && nch1[t] == 1;
    if (!join) ffirst.push_back(t);
  }
  const int32_t nf = (int32_t)ffirst.size();
  ffirst.push_back((int32_t)n);
  std::vector<int32_t> col2f(n);
  for (int32_t s = 0; s < nf; s++)
    for (int32_t t = ffirst[s]; t < ffirst[s + 1]; t++) col2f[t] = s;
  // ---- relaxed amalgamation: a child group ending right before its parent ----
  std::vector<int32_t> gfirst(nf), gk(nf);
  std::vector<int64_t> gm(nf), gtrue(nf);
  std::vector<char> merged(nf, 0);
  for (int32_t s = 0; s < nf; s++) {
    gfirst[s] = ffirst[s];
    gk[s] = ffirst[s + 1] - ffirst[s];
    gm[s] = cc1[ffirst[s]];
    int64_t tr = 0;
    for (int32_t t = ffirst[s]; t < ffirst[s + 1]; t++) tr += cc1[t];
    gtrue[s] = tr;
  }
  for (int32_t s = 0; s + 1 < nf; s++) {
    const int32_t lastc = ffirst[s + 1] - 1;
    if (par1[lastc] == -1 || col2f[par1[lastc]] != s + 1) continue;
    const int32_t t = s + 1;
    const int64_t k = (int64_t)gk[s] + gk[t];
    const int64_t m = (int64_t)gk[s] + gm[t];
    const double nzm = (double)k * m - (double)k * (k - 1) / 2.0;
    const double zeros = nzm - (double)(gtrue[s] + gtrue[t]);
    const bool merge = k <= 4 || (k <= 16 && zeros < 0.8 * nzm) ||
                       (k <= 48 && zeros < 0.1 * nzm) || zeros < 0.05 * nzm;
    if (!merge) continue;
    gfirst[t] = gfirst[s];
    gk[t] = (int32_t)k;
    gm[t] = m;
    gtrue[t] = gtrue[s] + gtrue[t];
    merged[s] = 1;
  }
  for (int32_t s = 0; s < nf; s++)
    if (!merged[s]) S.sn_first.push_back(gfirst[s]);
  const int32_t ns = (int32_t)S.sn_first.size();
  S.sn_first.push_back((int32_t)n);
  std::vector<int32_t> col2sn(n);
  for (int32_t s = 0; s < ns; s++)
    for (int32_t t = S.sn_first[s]; t < S.sn_first[s + 1]; t++) col2sn[t] = s;

  // ---- lower column structure of A in order 1 ----
  auto o1 = [&](int64_t input) { return ipost[ip0[input]]; };
  std::vector<int64_t> cp(n + 1, 0);
  for (int64_t r = 0; r < n; r++)
    for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
      const int32_t a = o1(r), b = o1(columns[q] - 1);
      if (a != b) cp[std::min(a, b) + 1]++;
    }
  for (int64_t i = 0; i < n; i++) cp[i + 1] += cp[i];
  std::vector<int32_t> ci(cp[n]);
  {
    std::vector<int64_t> fill(cp.begin(), cp.end() - 1);
    for (int64_t r = 0; r < n; r++)
      for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
        const int32_t a = o1(r), b = o1(columns[q] - 1);
        if (a != b) ci[fill[std::min(a, b)]++] = std::max(a, b);
      }
  }
  // ---- supernodal tree and row structures ----
  S.sn_parent.assign(ns, -1);
  for (int32_t s = 0; s < ns; s++) {
    const int32_t p = par1[S.sn_first[s + 1] - 1];
    S.sn_parent[s] = p == -1 ? -1 : col2sn[p];
    if (S.sn_parent[s] != -1 && S.sn_parent[s] <= s) return "supernodal tree out of order";
  }
  S.child_ptr.assign(ns + 1, 0);
  for (int32_t s = 0; s < ns; s++)
    if (S.sn_parent[s] != -1) S.child_ptr[S.sn_parent[s] + 1]++;
  for (int32_t s = 0; s < ns; s++) S.child_ptr[s + 1] += S.child_ptr[s];
  S.child_list.resize(S.child_ptr[ns]);
  {
    std::vector<int32_t> fill(S.child_ptr.begin(), S.child_ptr.end() - 1);
    for (int32_t s = 0; s < ns; s++)
      if (S.sn_parent[s] != -1) S.child_list[fill[S.sn_parent[s]]++] = s;
  }
  S.row_ptr.assign(ns + 1, 0);
  {
    std::vector<int32_t> mark(n, -1), beyond;
    for (int32_t s = 0; s < ns; s++) {
      const int32_t f = S.sn_first[s], l = S.sn_first[s + 1] - 1;
      beyond.clear();
      for (int32_t j = f; j <= l; j++)
        for (int64_t q = cp[j]; q < cp[j + 1]; q++) {
          const int32_t r = ci[q];
          if (r > l && mark[r] != s) {
            mark[r] = s;
            beyond.push_back(r);
          }
        }
      for (int32_t q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) {
        const int32_t c = S.child_list[q];
        for (int64_t t = S.row_ptr[c] + S.k(c); t < S.row_ptr[c + 1]; t++) {
          const int32_t r = S.rows[t];
          if (r < f) return "child row below its parent";
          if (r > l && mark[r] != s) {
            mark[r] = s;
            beyond.push_back(r);
          }
        }
      }
      std::sort(beyond.begin(), beyond.end());
      for (int32_t j = f; j <= l; j++) S.rows.push_back(j);
      S.rows.insert(S.rows.end(), beyond.begin(), beyond.end());
      S.row_ptr[s + 1] = (int64_t)S.rows.size();
    }
  }
  // ---- relative indices of each child's update rows in its parent ----
  S.rel_ptr.assign(ns + 1, 0);
  for (int32_t s = 0; s < ns; s++)
    S.rel_ptr[s + 1] = S.rel_ptr[s] + (S.sn_parent[s] == -1 ? 0 : S.m(s) - S.k(s));
  S.rel.resize(S.rel_ptr[ns]);
  {
    std::vector<int32_t> pos(n, -1), stamp(n, -1);
    for (int32_t p = 0; p < ns; p++) {
      for (int64_t t = S.row_ptr[p]; t < S.row_ptr[p + 1]; t++) {
        pos[S.rows[t]] = (int32_t)(t - S.row_ptr[p]);
        stamp[S.rows[t]] = p;
      }
      for (int32_t q = S.child_ptr[p]; q < S.child_ptr[p + 1]; q++) {
        const int32_t c = S.child_list[q];
        int64_t w = S.rel_ptr[c];
        for (int64_t t = S.row_ptr[c] + S.k(c); t < S.row_ptr[c + 1]; t++) {
          const int32_t r = S.rows[t];
          if (stamp[r] != p) return "child row missing from its parent";
          S.rel[w++] = (uint32_t)pos[r];
        }
      }
    }
  }
  // ---- offsets, statistics, levels ----
  S.front_off.assign(ns + 1, 0);
  S.vec_off.assign(ns + 1, 0);
  S.level.assign(ns, 0);
  int32_t max_level = 0;
  for (int32_t s = 0; s < ns; s++) {
    const int64_t m = S.m(s), k = S.k(s);
    S.front_off[s + 1] = S.front_off[s] + (uint64_t)(m * m);
    S.vec_off[s + 1] = S.vec_off[s] + (uint64_t)m;
    S.nnz_L += (uint64_t)(k * m - k * (k - 1) / 2);
    for (int64_t c = 0; c < k; c++) {
      const double r = (double)(m - c - 1);
      S.flops += r + r * (r + 1.0);
    }
    S.max_front = std::max<int32_t>(S.max_front, (int32_t)m);
    S.max_children = std::max(S.max_children, S.child_ptr[s + 1] - S.child_ptr[s]);
    for (int32_t q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++)
      S.level[s] = std::max(S.level[s], S.level[S.child_list[q]] + 1);
    max_level = std::max(max_level, S.level[s]);
  }
  S.level_ptr.assign(max_level + 2, 0);
  for (int32_t s = 0; s < ns; s++) S.level_ptr[S.level[s] + 1]++;
  for (int32_t L = 0; L <= max_level; L++) S.level_ptr[L + 1] += S.level_ptr[L];
  S.level_list.resize(ns);
  {
    std::vector<int32_t> fill(S.level_ptr.begin(), S.level_ptr.end() - 1);
    for (int32_t s = 0; s < ns; s++) S.level_list[fill[S.level[s]]++] = s;
  }
  // ---- where each stored value lands: front of the lower column's supernode ----
  // (rows split over the host threads; every entry is independent)
  S.a_dest.resize(nnz);
  {
    std::atomic<bool> outside{false};
    auto dest_rows = [&](int64_t r0, int64_t r1) {
      for (int64_t r = r0; r < r1; r++)
        for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
          const int32_t a = o1(r), b = o1(columns[q] - 1);
          const int32_t hi = std::max(a, b), lo = std::min(a, b);
          const int32_t s = col2sn[lo];
          const int32_t f = S.sn_first[s], l = S.sn_first[s + 1] - 1;
          int64_t lrow;
          if (hi <= l) {
            lrow = hi - f;
          } else {
            const int32_t* b0 = S.rows.data() + S.row_ptr[s] + S.k(s);
            const int32_t* b1 = S.rows.data() + S.row_ptr[s + 1];
            const int32_t* it = std::lower_bound(b0, b1, hi);
            if (it == b1 || *it != hi) {
              outside = true;
              return;
            }
            lrow = (int64_t)(it - (S.rows.data() + S.row_ptr[s]));
          }
          S.a_dest[q] = S.front_off[s] + (uint64_t)lrow + (uint64_t)(lo - f) * (uint64_t)S.m(s);
        }
    };
    const int nt = (int)std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()),
                                          std::max<int64_t>(1, n / 4096));
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (int t = 1; t < nt; t++) {
      const int64_t r0 = t * chunk, r1 = std::min<int64_t>(n, r0 + chunk);
      if (r0 < r1) th.emplace_back(dest_rows, r0, r1);
    }
    dest_rows(0, std::min<int64_t>(n, chunk));
    for (auto& x : th) x.join();
    if (outside) return "entry outside its front";
  }
  // ---- both triangles in input numbering (refinement SpMV) ----
  // Row c holds the transposed upper entries (r, c), r < c, in ascending r,
  // then its own upper entries.  The rows are split in chunks over the host
  // threads; each chunk's count per column gives its write offsets, so the
  // layout is the sequential one whatever the thread count.
  {
    const int nt = (int)std::min<int64_t>(
        std::min(16u, std::max(1u, std::thread::hardware_concurrency())),
        std::max<int64_t>(1, n / 65536));
    const int64_t chunk = (n + nt - 1) / nt;
    // per chunk and column: a count, then a write offset within the column's
    // row of the full pattern (both bounded by one row's length: 32 bits)
    std::vector<std::vector<uint32_t>> cnt(nt, std::vector<uint32_t>(n, 0));
    auto run = [&](auto&& body) {
      std::vector<std::thread> th;
      for (int t = 1; t < nt; t++) th.emplace_back(body, t);
      body(0);
      for (auto& x : th) x.join();
    };
    run([&](int t) {
      const int64_t r0 = t * chunk, r1 = std::min<int64_t>(n, r0 + chunk);
      for (int64_t r = r0; r < r1; r++)
        for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
          const int64_t c = columns[q] - 1;
          if (c != r) cnt[t][c]++;
        }
    });
    S.full_ptr.assign(n + 1, 0);
    for (int64_t r = 0; r < n; r++) {
      int64_t tr = 0;
      for (int t = 0; t < nt; t++) tr += cnt[t][r];
      S.full_ptr[r + 1] = S.full_ptr[r] + tr + (int64_t)(iofeir[r + 1] - iofeir[r]);
    }
    // cnt[t][c] becomes chunk t's first write offset in row c
    for (int64_t c = 0; c < n; c++) {
      uint32_t at = 0;
      for (int t = 0; t < nt; t++) {
        const uint32_t k = cnt[t][c];
        cnt[t][c] = at;
        at += k;
      }
    }
    S.full_col.resize(S.full_ptr[n]);
    S.full_slot.resize(S.full_ptr[n]);
    run([&](int t) {
      const int64_t r0 = t * chunk, r1 = std::min<int64_t>(n, r0 + chunk);
      for (int64_t r = r0; r < r1; r++) {
        int64_t own = S.full_ptr[r + 1] - (int64_t)(iofeir[r + 1] - iofeir[r]);
        for (uint64_t q = iofeir[r] - 1; q < (uint64_t)iofeir[r + 1] - 1; q++) {
          const int64_t c = columns[q] - 1;
          S.full_col[own] = (int32_t)c;
          S.full_slot[own++] = (uint32_t)q;
          if (c != r) {
            const int64_t w = S.full_ptr[c] + (int64_t)cnt[t][c]++;
            S.full_col[w] = (int32_t)r;
            S.full_slot[w] = (uint32_t)q;
          }
        }
      }
    });
  }
  S.perm.resize(n);
  for (int32_t t = 0; t < n; t++) S.perm[t] = p0[post[t]];
  return "";
}
