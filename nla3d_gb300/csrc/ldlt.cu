// Supernodal multifrontal LDL^T on the device for a symmetric K(2) held in
// the reference's upper CSR layout (SparseSymMatrix, SparseMatrix.h:206-221):
// the GPU counterpart of EquationSolver::factorizeEquations /
// substituteEquations (EquationSolver.h:19-34).  No counterpart exists in the
// reference's own sources for the device; its host PARDISO / dense Gauss
// solvers are what this replaces.
//
// Numeric factorisation, level by level of the supernodal tree (all fronts
// of a level are independent):
//   1. every front is zeroed and the matrix values are scattered into it
//      (one map entry per stored value, computed by the symbolic analysis);
//   2. extend-add: each child's update matrix is added into its parent's
//      front; children are taken one ordinal at a time (first children of all
//      parents of the level, then second children, ...) so that no two
//      threads add into one entry and the sums keep a fixed order;
//   3. partial LDL^T of the front's k pivot columns, right-looking, without
//      pivoting (the u/p blocks are quasi-definite: K_uu > 0, K_pp < 0, and
//      constraint rows are ordered last by the caller); a pivot below
//      tau = pivot_rel * max|A| is replaced by +-tau and counted, and the
//      solve's iterative refinement recovers the accuracy.
//      Fronts of <= kSmallFront rows: one thread block per front, the front
//      in shared memory, all fronts of the level in one launch.  Larger
//      fronts: all of the level's together, blocked, 64 columns per panel
//      (diagonal block and its inverse, panel rows) in outer blocks of 256
//      columns: each panel's rank-64 update reaches only the rest of its
//      outer block; the columns after the block take one rank-256 update
//      per block, so each trailing tile is read and written once per 256
//      pivots instead of once per 64 (FMA tiles, or tcgen05 TF32 split MMAs
//      for FP32 fronts with precision 2).
// Solve (multifrontal, vectors): forward by levels with the same extend-add
// on the update vectors, D^-1, backward by levels top-down gathering the
// solved ancestor entries; FP64 refinement r = b - A x with A's
// both-triangle CSR in the input numbering (plain steps, then GMRES
// preconditioned by the factor).  Factorisation and solve are captured once
// into CUDA graphs and replayed.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/nla3d_gpu.h"
#include "ldlt.hpp"

namespace {

constexpr int kThreads = 256;
constexpr int kSmallFront = 128;   // fronts up to this many rows: one block each, in smem
constexpr int kPanel = 64;         // panel width of the blocked path
constexpr int kOuter = 256;        // outer block of the blocked path (4 panels)
constexpr int kTile = 64;          // panel-row tile of the blocked path

struct LdltDev {
  const uint64_t* front_off;
  const uint64_t* vec_off;
  const int64_t* row_ptr;
  const int32_t* rows;
  const int32_t* sn_first;
  const int32_t* sn_parent;
  const int64_t* rel_ptr;
  const uint32_t* rel;
};

// ---- factorisation kernels ----

template <typename T>
__global__ void scatter_values_kernel(uint64_t nnz, const uint64_t* __restrict__ dest,
                                      const double* __restrict__ values, T* __restrict__ front) {
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (uint64_t)gridDim.x * blockDim.x)
    front[dest[q]] = (T)values[q];
}

// max |A| over the stored values: per-block maxima, then one block over them
constexpr int kMaxBlocks = 1024;
__global__ void maxabs_kernel(uint64_t nnz, const double* __restrict__ values,
                              double* __restrict__ part) {
  __shared__ double red[kThreads];
  double m = 0.0;
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (uint64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(values[q]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void maxabs_final_kernel(int n, const double* __restrict__ part, double* out) {
  __shared__ double red[kThreads];
  double m = 0.0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) m = fmax(m, part[q]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// children[blockIdx.x]: add its update matrix into its parent's front
template <typename T>
__global__ void extend_add_kernel(const int32_t* __restrict__ children, int n, LdltDev d,
                                  T* __restrict__ front) {
  const int c = children[blockIdx.x];
  const int p = d.sn_parent[c];
  const int64_t mc = d.row_ptr[c + 1] - d.row_ptr[c];
  const int64_t kc = d.sn_first[c + 1] - d.sn_first[c];
  const int64_t mp = d.row_ptr[p + 1] - d.row_ptr[p];
  const int64_t u = mc - kc;
  const T* Fc = front + d.front_off[c];
  T* Fp = front + d.front_off[p];
  const uint32_t* rel = d.rel + d.rel_ptr[c];
  for (int64_t j = blockIdx.y; j < u; j += gridDim.y) {
    const int64_t pj = rel[j];
    const T* src = Fc + (kc + j) * mc + kc;
    T* dst = Fp + pj * mp;
    for (int64_t i = j + threadIdx.x; i < u; i += blockDim.x) dst[rel[i]] += src[i];
  }
}

// the guarded pivot without counting it
template <typename T>
__device__ __forceinline__ T guard_value(T dv, T tau) {
  if (!(fabs(dv) >= tau) && dv == dv) return dv < T(0) ? -tau : tau;
  return dv;
}

template <typename T>
__device__ __forceinline__ T guard_pivot(T dv, T tau, int* perturbed) {
  if (!(fabs(dv) >= tau)) {   // also catches NaN
    if (dv != dv) {
      atomicAdd(perturbed + 1, 1);
      return dv;
    }
    atomicAdd(perturbed, 1);
    return dv < T(0) ? -tau : tau;
  }
  return dv;
}

// one block per front (m <= kSmallFront), the front held in shared memory
// (column-major, leading dimension m+1): right-looking LDL^T of the k pivot
// columns, the trailing (m-k)^2 block left as the update matrix.  Threads
// cover the trailing triangle as 32 rows x 8 columns.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    factor_small_kernel(const int32_t* __restrict__ list, LdltDev d, T* __restrict__ front,
                        const double* __restrict__ tau_p, double pivot_rel, int* perturbed) {
  extern __shared__ unsigned char smem_raw[];
  T* S = reinterpret_cast<T*>(smem_raw);
  const int s = list[blockIdx.x];
  const int m = (int)(d.row_ptr[s + 1] - d.row_ptr[s]);
  const int k = d.sn_first[s + 1] - d.sn_first[s];
  const int ld = m + 1;
  T* F = front + d.front_off[s];
  for (int c = 0; c < m; c++)
    for (int r = c + threadIdx.x; r < m; r += blockDim.x) S[r + c * ld] = F[r + (int64_t)c * m];
  __syncthreads();
  // the pivot bound in the front's precision (the guards compare in it)
  const T tau = (T)(pivot_rel * tau_p[0]);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  // one barrier per pivot: the columns right of p are updated with the
  // unscaled column p (A_ij -= w_i w_j / d), which no later step writes; the
  // pivot columns are scaled after the loop
  for (int p = 0; p < k; p++) {
    // every thread guards the pivot itself (thread 0 counts)
    const T raw = S[p + p * ld];
    const T dv = threadIdx.x == 0 ? guard_pivot(raw, tau, perturbed) : guard_value(raw, tau);
    const T* colp = S + p * ld;
    for (int j = p + 1 + ty; j < m; j += 8) {
      const T lj = colp[j] / dv;
      T* col = S + j * ld;
      for (int i = j + tx; i < m; i += 32) col[i] -= colp[i] * lj;
    }
    __syncthreads();
  }
  // scale column p by its guarded pivot (its diagonal is unchanged since
  // step p), one warp per column
  for (int p = ty; p < k; p += 8) {
    T* colp = S + p * ld;
    const T dv = guard_value(colp[p], tau);
    for (int i = p + 1 + tx; i < m; i += 32) colp[i] = colp[i] / dv;
    __syncwarp();
    if (tx == 0) colp[p] = dv;
  }
  __syncthreads();
  for (int c = 0; c < m; c++)
    for (int r = c + threadIdx.x; r < m; r += blockDim.x) F[r + (int64_t)c * m] = S[r + c * ld];
}

// Blocked path for the fronts above kSmallFront rows, batched: every launch
// works on panel p0 of all large fronts of one level (blockIdx.z / .x picks
// the front; fronts with k <= p0 return).  W: per front an m x min(kOuter,
// k rounded up to kPanel) block, W[i + c m] = (L D)[i][o0 + c] for the rows
// i past the panel of column o0 + c (o0: the current outer block).
struct BigBatch {
  const int32_t* list;
  const uint64_t* w_off;
  const uint64_t* li_off;   // the front's inverted diagonal blocks, 64 x 64 per panel
  const uint64_t* pk_off;   // tensor-core fronts: the front's packed outer-block operands
};

// step 1: LDL^T of the pb x pb diagonal block, and the inverse of its unit
// lower factor (64 x 64 column-major, kept per panel for step 2 and the solves)
template <typename T>
__global__ void __launch_bounds__(kThreads)
    batched_diag_kernel(BigBatch b, LdltDev d, T* __restrict__ front, int64_t p0,
                        T* __restrict__ Linv, const double* __restrict__ tau_p, double pivot_rel,
                        int* perturbed) {
  extern __shared__ unsigned char diag_smem_raw[];
  T(*B)[kPanel + 1] = reinterpret_cast<T(*)[kPanel + 1]>(diag_smem_raw);   // B[col][row]
  unsigned char* diag_smem = diag_smem_raw + sizeof(T) * kPanel * (kPanel + 1);
  const int s = b.list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (p0 >= k) return;
  const int pb = (int)(k - p0 < kPanel ? k - p0 : kPanel);
  T* F = front + d.front_off[s];
  const int tc = threadIdx.x % kPanel, tr = threadIdx.x / kPanel;   // 64 columns x 4
  for (int r = tr; r < pb; r += kThreads / kPanel)
    if (tc < pb) B[tc][r] = r >= tc ? F[(p0 + r) + (p0 + tc) * m] : T(0);
  __syncthreads();
  // the pivot bound in the front's precision (the guards compare in it)
  const T tau = (T)(pivot_rel * tau_p[0]);
  // one barrier per pivot: every thread guards the pivot itself (only thread
  // 0 counts); the columns right of p are updated with the unscaled column p
  // (A_rc -= w_r w_c / d), which no later step writes, and every column is
  // scaled by its pivot after the loop
  for (int p = 0; p < pb; p++) {
    const T raw = B[p][p];
    const T dv = threadIdx.x == 0 ? guard_pivot(raw, tau, perturbed) : guard_value(raw, tau);
    if (tc > p && tc < pb) {
      const T lc = B[p][tc] / dv;
      for (int r = tc + tr; r < pb; r += kThreads / kPanel) B[tc][r] -= B[p][r] * lc;
    }
    __syncthreads();
  }
  if (tc < pb) {
    // column tc's diagonal is unchanged since its own step
    const T dc = guard_value(B[tc][tc], tau);
    for (int r = tc + 1 + tr; r < pb; r += kThreads / kPanel) B[tc][r] = B[tc][r] / dc;
  }
  __syncthreads();
  if (threadIdx.x < pb) B[threadIdx.x][threadIdx.x] = guard_value(B[threadIdx.x][threadIdx.x], tau);
  __syncthreads();
  for (int r = tr; r < pb; r += kThreads / kPanel)
    if (tc < pb && r >= tc) F[(p0 + r) + (p0 + tc) * m] = B[tc][r];
  // inverse of the unit lower L11 in shared memory (X[col][row]): column c by
  // the four consecutive lanes 4c .. 4c+3, row after row, each row's dot
  // product split over the four lanes and summed by shuffles, so that only
  // warp-level barriers separate the rows; then stored for step 2 and the solves
  T(*X)[kPanel + 1] = reinterpret_cast<T(*)[kPanel + 1]>(diag_smem);
  {
    const int c = threadIdx.x >> 2, sub = threadIdx.x & 3;
    if (c < pb)
      for (int r = sub; r <= c; r += 4) X[c][r] = r == c ? T(1) : T(0);
    __syncwarp();
    for (int r = 1; r < pb; r++) {
      T part = T(0);
      if (c < r)
        for (int q = c + sub; q < r; q += 4) part += B[q][r] * X[c][q];
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      if (sub == 0 && c < r) X[c][r] = -part;
      __syncwarp();
    }
  }
  __syncthreads();
  T* Li = Linv + b.li_off[blockIdx.x] + (uint64_t)(p0 / kPanel) * kPanel * kPanel;
  for (int t = threadIdx.x; t < pb * kPanel; t += blockDim.x) {
    const int r = t % kPanel, c = t / kPanel;
    if (r < pb) Li[r + c * kPanel] = X[c][r];
  }
}

// step 2: the panel rows i >= q0 = p0+pb: W = F21 Linv^T (W = L21 D), F21 <- W D^-1;
// 64-row tiles, 4 rows x 4 columns per thread
template <typename T>
__global__ void __launch_bounds__(kThreads)
    batched_panel_kernel(BigBatch b, LdltDev d, T* __restrict__ front, int64_t p0,
                         const T* __restrict__ Linv, T* __restrict__ Wbuf) {
  __shared__ T As[16][kTile + 1];
  __shared__ T Bs[16][kPanel + 1];
  __shared__ T Dv[kPanel];
  const int s = b.list[blockIdx.y];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (p0 >= k) return;
  const int pb = (int)(k - p0 < kPanel ? k - p0 : kPanel);
  const int64_t q0 = p0 + pb;
  const int64_t i0 = q0 + (int64_t)blockIdx.x * kTile;
  if (i0 >= m) return;
  T* F = front + d.front_off[s];
  T* W = Wbuf + b.w_off[blockIdx.y];
  const T* Li = Linv + b.li_off[blockIdx.y] + (uint64_t)(p0 / kPanel) * kPanel * kPanel;
  for (int t = threadIdx.x; t < pb; t += blockDim.x) Dv[t] = F[(p0 + t) + (p0 + t) * m];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T acc[4][4] = {};
  for (int c0 = 0; c0 < pb; c0 += 16) {
    for (int t = threadIdx.x; t < 16 * kTile; t += blockDim.x) {
      const int cc = t / kTile, rr = t % kTile;
      const int c2 = c0 + cc;
      const int64_t i = i0 + rr;
      As[cc][rr] = (c2 < pb && i < m) ? F[i + (p0 + c2) * m] : T(0);
      // Bs[c2][c] = Linv[c][c2]
      Bs[cc][rr] = (c2 < pb && rr < pb) ? Li[rr + c2 * kPanel] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int cc = 0; cc < 16; cc++) {
      T a[4], bb[4];
#pragma unroll
      for (int u = 0; u < 4; u++) a[u] = As[cc][ty * 4 + u];
#pragma unroll
      for (int v = 0; v < 4; v++) bb[v] = Bs[cc][tx * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * bb[v];
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const int64_t i = i0 + ty * 4 + u;
    if (i >= m) continue;
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int c = tx * 4 + v;
      if (c >= pb) continue;
      W[i + (int64_t)(p0 % kOuter + c) * m] = acc[u][v];
      F[i + (p0 + c) * m] = acc[u][v] / Dv[c];
    }
  }
}

// step 3: update of the lower triangle, F[i][j] -= sum_c L[i][lc0 + c] W[j][wc0 + c]
// for jb <= j < je, i >= j:
//   inner (outer == 0, after panel p0): the panel's kw = pb columns into the
//     rest of its outer block, jb = p0 + pb, je = min(o0 + kOuter, k);
//   outer (outer == 1, p0 = o0): the whole outer block, kw = min(k, o0 +
//     kOuter) - o0 columns, into everything after it, jb = o0 + kw, je = m.
// Every front's (lc0, wc0, kw, jb, je) follow from its own k and m.
struct UpdateRange {
  int64_t lc0, wc0, kw, jb, je;
};

__device__ __forceinline__ bool update_range(int64_t p0, int outer, int64_t k, int64_t m,
                                             UpdateRange& u) {
  if (p0 >= k) return false;
  if (!outer) {
    const int64_t pb = k - p0 < kPanel ? k - p0 : kPanel;
    const int64_t o0 = p0 - p0 % kOuter;
    u.lc0 = p0;
    u.wc0 = p0 % kOuter;
    u.kw = pb;
    u.jb = p0 + pb;
    u.je = o0 + kOuter < k ? o0 + kOuter : k;
  } else {
    const int64_t oe = p0 + kOuter < k ? p0 + kOuter : k;
    u.lc0 = p0;
    u.wc0 = 0;
    u.kw = oe - p0;
    u.jb = oe;
    u.je = m;
  }
  return u.jb < u.je;
}

// BT x BT tiles (blockIdx.x rows, .y columns, both from jb), front
// blockIdx.z, RT x RT outputs per thread (64 / 4 for FP64, whose FMA pipe
// bounds it anyway; 128 / 8 for FP32).  A thread owns rows tx + 16u and
// columns ty + 16v: shared-memory reads are conflict-free or broadcast and
// the stores run down the columns.  The next 16-wide slice of the operands
// is loaded into registers while the current one is multiplied.
template <typename T, int BT, int RT>
__global__ void __launch_bounds__(kThreads)
    batched_trailing_kernel(BigBatch b, LdltDev d, T* __restrict__ front, int64_t p0, int outer,
                            const T* __restrict__ Wbuf) {
  static_assert((BT / RT) * (BT / RT) == kThreads, "one output block per thread");
  static_assert(BT / RT == 16, "16 x 16 threads");
  constexpr int LPT = 16 * BT / kThreads;   // slice elements each thread loads per operand
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (tj > ti) return;
  const int s = b.list[blockIdx.z];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  UpdateRange ur;
  if (!update_range(p0, outer, k, m, ur)) return;
  const int64_t i0 = ur.jb + (int64_t)ti * BT, j0 = ur.jb + (int64_t)tj * BT;
  if (i0 >= m || j0 >= ur.je) return;
  T* F = front + d.front_off[s];
  const T* W = Wbuf + b.w_off[blockIdx.z];
  const int kw = (int)ur.kw;
  __shared__ T As[16][BT];
  __shared__ T Bs[16][BT];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T acc[RT][RT] = {};
  T ra[LPT], rb[LPT];
  auto load = [&](int c0) {
#pragma unroll
    for (int q = 0; q < LPT; q++) {
      const int t = threadIdx.x + q * kThreads;
      const int cc = t / BT, rr = t % BT;
      const int c = c0 + cc;
      const int64_t i = i0 + rr, j = j0 + rr;
      ra[q] = (c < kw && i < m) ? F[i + (ur.lc0 + c) * m] : T(0);
      rb[q] = (c < kw && j < ur.je) ? W[j + (ur.wc0 + c) * m] : T(0);
    }
  };
  load(0);
  for (int c0 = 0; c0 < kw; c0 += 16) {
#pragma unroll
    for (int q = 0; q < LPT; q++) {
      const int t = threadIdx.x + q * kThreads;
      As[t / BT][t % BT] = ra[q];
      Bs[t / BT][t % BT] = rb[q];
    }
    __syncthreads();
    if (c0 + 16 < kw) load(c0 + 16);
#pragma unroll
    for (int cc = 0; cc < 16; cc++) {
      T a[RT], bb[RT];
#pragma unroll
      for (int u = 0; u < RT; u++) a[u] = As[cc][tx + 16 * u];
#pragma unroll
      for (int v = 0; v < RT; v++) bb[v] = Bs[cc][ty + 16 * v];
#pragma unroll
      for (int u = 0; u < RT; u++)
#pragma unroll
        for (int v = 0; v < RT; v++) acc[u][v] += a[u] * bb[v];
    }
    __syncthreads();
  }
#pragma unroll
  for (int v = 0; v < RT; v++) {
    const int64_t j = j0 + ty + 16 * v;
    if (j >= ur.je) continue;
#pragma unroll
    for (int u = 0; u < RT; u++) {
      const int64_t i = i0 + tx + 16 * u;
      if (i < m && j <= i) F[i + j * m] -= acc[u][v];
    }
  }
}

template <typename T>
struct TrailingShape {
  static constexpr int BT = 64, RT = 4;
};
template <>
struct TrailingShape<float> {
  static constexpr int BT = 128, RT = 8;
};

// ---- tensor-core helpers (tcgen05, kind::tf32) ----
//
// Operands are split into TF32 high and low parts (x = hi + lo, hi = x
// rounded to TF32) and staged in shared memory in the canonical K-major
// layout without swizzle (8-row x 16-byte core matrices; K-adjacent cores
// 128 B apart, 8-row groups 1 KB apart); an update tile is 128 x 128, its
// operands taken in chunks of 32 columns, each chunk 4 k-steps x 3 MMAs
// (hi.hi + hi.lo + lo.hi, FP32 accumulation in TMEM).
constexpr int kTcM = 128, kTcN = 128, kTcKH = 32;   // tile rows, columns, K per chunk
constexpr int kTcThreads = 256;                      // the packing kernel's block
constexpr uint32_t kTcTileFloats = kTcM * kTcKH;     // one 128 x 32 operand chunk
// instruction descriptor: D F32 (bit 4), A and B TF32 (bits 7, 10), both
// K-major, N / 8 at bit 17, M / 16 at bit 24
constexpr uint32_t kTcIdesc =
    (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
constexpr long long kTcSpinLimit = 1ll << 26;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, leading (K) and stride (8-row) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// offset (floats) of element (row r, k) of a 128 x 32 K-major operand chunk
__device__ __forceinline__ uint32_t tc_off(int r, int k) {
  return (uint32_t)(((r >> 3) * (kTcKH / 4) + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3));
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t phase) {
  for (long long it = 0; it < kTcSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kTcIdesc), "r"(acc));
}

// ---- the updates from packed operands (tensor-core fronts) ----
//
// An update (update_range: the rank-256 one after an outer block, or a
// panel's rank-64 one inside its block) reads the same operands from every
// tile of a row or column: L[jb + 128 r .. +127][lc0 .. lc0 + kw) and
// W[jb + 128 r .. +127][wc0 .. wc0 + kw).  pack_update_kernel splits them
// into TF32 high and low parts once per update and stores them, per 128-row
// block r and 32-column chunk c, as four 16 KB tiles (A hi, A lo, B hi, B lo)
// in the MMA's shared-memory layout (tc_off).  tc_packed_kernel is persistent
// (one CTA per SM walking a host-built list of the level's tiles) and
// warp-specialised:
//   warp 0 (one lane): copies each chunk's four tiles into a ring of
//     kPkStages shared-memory stages with asynchronous bulk copies
//     (cp.async.bulk, completion counted on the stage's `full` mbarrier);
//   warp 1 (one lane): waits for a stage, issues its 12 MMAs (hi.hi, hi.lo,
//     lo.hi per 8-wide k step) into one of two 128-column TMEM
//     accumulators and commits them to the stage's `empty` mbarrier (the
//     stage is refilled once they have read it) and, after a tile's last
//     chunk, to the accumulator's `acc_full` mbarrier;
//   warps 2-9: load their 32 rows x 64 columns of the front tile into
//     registers while the tile's MMAs run, then read the same part of the
//     finished accumulator from TMEM, release it (`acc_empty`, one arrival
//     per warp) and store the difference, while the MMAs of the next tile
//     run into the other accumulator.
// Every wait is bounded: on a timeout the role stops, err[0] is set and the
// copies and MMAs still in flight get one more bounded wait each before the
// CTA releases its shared memory and TMEM.
constexpr int kPkChunks = kOuter / kTcKH;                  // 8 chunks of 32 columns
constexpr uint32_t kPkTile = kTcTileFloats;                // floats per 128 x 32 tile
constexpr uint32_t kPkBlock = 4 * kPkTile * kPkChunks;    // floats per 128-row block
constexpr int kPkStages = 3;
constexpr size_t kPkSmem = (size_t)kPkStages * 4 * kPkTile * sizeof(float) + 256;
constexpr int kOuterThreads = 320;   // tc_packed_kernel: producer, MMA, 8 epilogue warps

__global__ void __launch_bounds__(kTcThreads)
    pack_update_kernel(BigBatch b, LdltDev d, const float* __restrict__ front, int64_t p0,
                       int outer, const float* __restrict__ Wbuf, float* __restrict__ packed) {
  const int s = b.list[blockIdx.z];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  UpdateRange ur;
  if (!update_range(p0, outer, k, m, ur)) return;
  const int rb = blockIdx.x, ch = blockIdx.y;
  const int64_t r0 = ur.jb + (int64_t)rb * kTcM;
  if (r0 >= m || ch * kTcKH >= ur.kw) return;
  const float* F = front + d.front_off[s];
  const float* W = Wbuf + b.w_off[blockIdx.z];
  float* P = packed + b.pk_off[blockIdx.z] + (uint64_t)(rb * kPkChunks + ch) * 4 * kPkTile;
  // thread: row r, four groups of 4 consecutive columns (16-byte stores)
  const int r = threadIdx.x % kTcM, g0 = (threadIdx.x / kTcM) * 4;
  const int64_t i = r0 + r;
#pragma unroll
  for (int g = g0; g < g0 + 4; g++) {
    float4 ah, al, wh, wl;
    float* ahp = &ah.x;
    float* alp = &al.x;
    float* whp = &wh.x;
    float* wlp = &wl.x;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int c = ch * kTcKH + g * 4 + e;
      const bool in = c < ur.kw && i < m;
      const float av = in ? F[i + (ur.lc0 + c) * m] : 0.0f;
      const float wv = in && i < ur.je ? W[i + (ur.wc0 + c) * m] : 0.0f;   // B: columns < je
      ahp[e] = tf32_hi(av);
      alp[e] = av - ahp[e];
      whp[e] = tf32_hi(wv);
      wlp[e] = wv - whp[e];
    }
    const uint32_t o = tc_off(r, g * 4);
    *reinterpret_cast<float4*>(P + o) = ah;
    *reinterpret_cast<float4*>(P + kPkTile + o) = al;
    *reinterpret_cast<float4*>(P + 2 * kPkTile + o) = wh;
    *reinterpret_cast<float4*>(P + 3 * kPkTile + o) = wl;
  }
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst), "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ void expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
               : "memory");
}

// one update tile of the level's outer-block list: large front z (index in
// the level's list), tile row ti >= tile column tj
struct OuterTile {
  uint32_t z, tij;   // tij = ti << 16 | tj
};

__global__ void __launch_bounds__(kOuterThreads, 1)
    tc_packed_kernel(BigBatch b, LdltDev d, float* __restrict__ front, int64_t p0, int outer,
                     const float* __restrict__ packed, const OuterTile* __restrict__ tiles,
                     int n_tiles, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char pk_smem[];
  float* stage0 = reinterpret_cast<float*>(pk_smem);
  uint64_t* full = reinterpret_cast<uint64_t*>(stage0 + (size_t)kPkStages * 4 * kPkTile);
  uint64_t* empty = full + kPkStages;
  uint64_t* acc_full = empty + kPkStages;
  uint64_t* acc_empty = acc_full + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(2 * kTcN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 32) {
    for (int q = 0; q < kPkStages; q++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(full + q)), "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(empty + q)), "r"(1));
    }
    for (int q = 0; q < 2; q++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(acc_full + q)),
                   "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(acc_empty + q)),
                   "r"(8));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t kTileBytes = kPkTile * sizeof(float);
  auto stage_addr = [&](int q, int t) {   // t: 0 A hi, 1 A lo, 2 B hi, 3 B lo
    return smem_addr(stage0 + (size_t)(q * 4 + t) * kPkTile);
  };
  // the front of a tile: rows m, update range, chunks
  struct TileInfo {
    int64_t m, je, i0, j0;
    int nch;
    const float* pa;
    const float* pb;
    float* F;
  };
  auto info = [&](int t, TileInfo& ti) {
    const OuterTile ot = tiles[t];
    const int s = b.list[ot.z];
    const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
    const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
    UpdateRange ur;
    update_range(p0, outer, k, m, ur);   // the host listed only fronts whose range is not empty
    const uint32_t rI = ot.tij >> 16, rJ = ot.tij & 0xFFFFu;
    ti.m = m;
    ti.je = ur.je;
    ti.i0 = ur.jb + (int64_t)rI * kTcM;
    ti.j0 = ur.jb + (int64_t)rJ * kTcN;
    ti.nch = (int)((ur.kw + kTcKH - 1) / kTcKH);
    ti.pa = packed + b.pk_off[ot.z] + (uint64_t)rI * kPkBlock;
    ti.pb = packed + b.pk_off[ot.z] + (uint64_t)rJ * kPkBlock;
    ti.F = front + d.front_off[s];
  };
  bool ok = true;
  if (warp == 0) {
    if (lane == 0) {
      // producer: the ring of stages, in the MMA warp's order
      uint32_t g = 0, issued = 0;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        TileInfo ti;
        info(t, ti);
        for (int c = 0; c < ti.nch && ok; c++, g++) {
          const int q = g % kPkStages;
          if (g >= kPkStages) ok = tc_wait(smem_addr(empty + q), (g / kPkStages - 1) & 1u);
          if (!ok) break;
          const uint32_t fb = smem_addr(full + q);
          expect_tx(fb, 4 * kTileBytes);
          const float* a = ti.pa + (size_t)c * 4 * kPkTile;
          const float* bb = ti.pb + (size_t)c * 4 * kPkTile;
          bulk_copy(stage_addr(q, 0), a, kTileBytes, fb);
          bulk_copy(stage_addr(q, 1), a + kPkTile, kTileBytes, fb);
          bulk_copy(stage_addr(q, 2), bb + 2 * kPkTile, kTileBytes, fb);
          bulk_copy(stage_addr(q, 3), bb + 3 * kPkTile, kTileBytes, fb);
          issued = g + 1;
        }
      }
      if (!ok) {
        atomicExch(err, 1);
        // the copies of the last kPkStages chunks may still be in flight
        for (uint32_t h = issued > kPkStages ? issued - kPkStages : 0; h < issued; h++)
          tc_wait(smem_addr(full + h % kPkStages), (h / kPkStages) & 1u);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      const uint32_t lbo = 128, sbo = (kTcKH / 4) * 128;
      uint32_t g = 0, it = 0, committed_acc = 0;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, it++) {
        TileInfo ti;
        info(t, ti);
        const uint32_t a = it & 1u;
        if (it >= 2) ok = tc_wait(smem_addr(acc_empty + a), (it / 2 - 1) & 1u);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + a * kTcN;
        for (int c = 0; c < ti.nch && ok; c++, g++) {
          const int q = g % kPkStages;
          ok = tc_wait(smem_addr(full + q), (g / kPkStages) & 1u);
          if (!ok) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          for (int st = 0; st < kTcKH / 8; st++) {
            const uint32_t koff = st * 256;   // 8 K values = two core matrices
            const uint64_t dah = tc_desc(stage_addr(q, 0) + koff, lbo, sbo);
            const uint64_t dal = tc_desc(stage_addr(q, 1) + koff, lbo, sbo);
            const uint64_t dbh = tc_desc(stage_addr(q, 2) + koff, lbo, sbo);
            const uint64_t dbl = tc_desc(stage_addr(q, 3) + koff, lbo, sbo);
            tc_mma(acc, dah, dbh, (c > 0 || st > 0) ? 1u : 0u);
            tc_mma(acc, dah, dbl, 1u);
            tc_mma(acc, dal, dbh, 1u);
          }
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                  smem_addr(empty + q))
              : "memory");
        }
        if (!ok) break;
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_addr(acc_full + a))
            : "memory");
        committed_acc = it + 1;
      }
      if (!ok) {
        atomicExch(err, 1);
        // MMAs complete in order: the last chunk commit covers every MMA issued
        if (g > 0) tc_wait(smem_addr(empty + (g - 1) % kPkStages), ((g - 1) / kPkStages) & 1u);
      } else if (committed_acc > 0) {
        tc_wait(smem_addr(acc_full + ((committed_acc - 1) & 1u)), ((committed_acc - 1) / 2) & 1u);
      }
    }
  } else {
    // epilogue warp (warps 2-9): TMEM lanes 32 (warp % 4) .. +31 = tile rows
    // (a warp reaches only its own lane quarter), columns 64 ((warp - 2) / 4)
    // .. +63
    const int lq = warp & 3, cb = ((warp - 2) >> 2) * 64;
    const int row = lq * 32 + lane;
    uint32_t it = 0;
    for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, it++) {
      TileInfo ti;
      info(t, ti);
      const uint32_t a = it & 1u;
      const int64_t i = ti.i0 + row;
      const bool row_in = i < ti.m;
      // the front's values of the first 32 columns first: their loads overlap
      // the tile's MMAs; the second 32 load while the first are stored
      float* fp = ti.F + i + (ti.j0 + cb) * ti.m;   // (i, j0 + cb); column stride m
      const int64_t jlim = (row_in ? (i < ti.je - 1 ? i : ti.je - 1) : -1) - (ti.j0 + cb);
      float cv[32];
#pragma unroll
      for (int q = 0; q < 32; q++) cv[q] = q <= jlim ? fp[q * ti.m] : 0.0f;
      ok = tc_wait(smem_addr(acc_full + a), (it / 2) & 1u);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int h = 0; h < 2; h++) {
        uint32_t v[32];
#pragma unroll
        for (int c2 = 0; c2 < 2; c2++) {
          const uint32_t taddr = tmem + ((uint32_t)(lq * 32) << 16) + a * kTcN +
                                 (uint32_t)(cb + h * 32 + c2 * 16);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, "
              "%10, %11, %12, %13, %14, %15}, [%16];"
              : "=r"(v[c2 * 16 + 0]), "=r"(v[c2 * 16 + 1]), "=r"(v[c2 * 16 + 2]),
                "=r"(v[c2 * 16 + 3]), "=r"(v[c2 * 16 + 4]), "=r"(v[c2 * 16 + 5]),
                "=r"(v[c2 * 16 + 6]), "=r"(v[c2 * 16 + 7]), "=r"(v[c2 * 16 + 8]),
                "=r"(v[c2 * 16 + 9]), "=r"(v[c2 * 16 + 10]), "=r"(v[c2 * 16 + 11]),
                "=r"(v[c2 * 16 + 12]), "=r"(v[c2 * 16 + 13]), "=r"(v[c2 * 16 + 14]),
                "=r"(v[c2 * 16 + 15])
              : "r"(taddr));
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (h == 1) {
          // the accumulator is in registers: the MMAs of the tile after next may reuse it
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(acc_empty + a))
                         : "memory");
        }
        float nv[32];
        if (h == 0) {
#pragma unroll
          for (int q = 0; q < 32; q++) nv[q] = 32 + q <= jlim ? fp[(32 + q) * ti.m] : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 32; q++)
          if (h * 32 + q <= jlim) fp[(h * 32 + q) * ti.m] = cv[q] - __uint_as_float(v[q]);
        if (h == 0) {
#pragma unroll
          for (int q = 0; q < 32; q++) cv[q] = nv[q];
        }
      }
    }
    if (!ok && lane == 0) atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * kTcN));
}

// ---- solve kernels ----

__global__ void solve_init_kernel(int64_t n, const int32_t* __restrict__ perm,
                                  const int32_t* __restrict__ col2sn, LdltDev d,
                                  const double* __restrict__ b, double* __restrict__ vec) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int s = col2sn[j];
  vec[d.vec_off[s] + (j - d.sn_first[s])] = b[perm[j]];
}

__global__ void vec_extend_add_kernel(const int32_t* __restrict__ children, LdltDev d,
                                      double* __restrict__ vec) {
  const int c = children[blockIdx.x];
  const int p = d.sn_parent[c];
  const int64_t mc = d.row_ptr[c + 1] - d.row_ptr[c];
  const int64_t kc = d.sn_first[c + 1] - d.sn_first[c];
  const double* src = vec + d.vec_off[c] + kc;
  double* dst = vec + d.vec_off[p];
  const uint32_t* rel = d.rel + d.rel_ptr[c];
  for (int64_t i = threadIdx.x; i < mc - kc; i += blockDim.x) dst[rel[i]] += src[i];
}

// forward: v[0:k] <- D^-1 L11^-1 v[0:k], v[k:m] <- v[k:m] - L21 (L11^-1 v[0:k]);
// blocks of 64 pivots: the block's unit triangle in shared memory, then one
// pass over the rows below it
template <typename T>
__global__ void __launch_bounds__(kThreads)
    forward_kernel(const int32_t* __restrict__ list, LdltDev d, const T* __restrict__ front,
                   double* __restrict__ vec) {
  __shared__ double yb[kPanel];
  const int s = list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  const T* F = front + d.front_off[s];
  double* v = vec + d.vec_off[s];
  for (int64_t c0 = 0; c0 < k; c0 += kPanel) {
    const int cb = (int)(k - c0 < kPanel ? k - c0 : kPanel);
    if (threadIdx.x < cb) yb[threadIdx.x] = v[c0 + threadIdx.x];
    __syncthreads();
    for (int c = 0; c < cb; c++) {
      const int t = threadIdx.x;
      if (t > c && t < cb) yb[t] -= (double)F[(c0 + t) + (c0 + c) * m] * yb[c];
      __syncthreads();
    }
    if (threadIdx.x < cb) v[c0 + threadIdx.x] = yb[threadIdx.x];
    for (int64_t i = c0 + cb + threadIdx.x; i < m; i += blockDim.x) {
      double acc = 0.0;
      for (int c = 0; c < cb; c++) acc += (double)F[i + (c0 + c) * m] * yb[c];
      v[i] -= acc;
    }
    __syncthreads();
  }
  for (int64_t c = threadIdx.x; c < k; c += blockDim.x) v[c] /= (double)F[c + c * m];
}

// backward: x[0:k] = L11^-T (v[0:k] - L21^T x_rest), x_rest gathered from the
// solved ancestors (factor order), written to xf; blocks of 64 pivots from the
// last: the contributions of the solved pivots below the block (a warp per
// column), then the block's triangle in shared memory
template <typename T>
__global__ void __launch_bounds__(kThreads)
    backward_kernel(const int32_t* __restrict__ list, LdltDev d, const T* __restrict__ front,
                    double* __restrict__ vec, double* __restrict__ xf) {
  __shared__ double xb[kPanel];
  const int s = list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  const int32_t* rows = d.rows + d.row_ptr[s];
  const T* F = front + d.front_off[s];
  double* v = vec + d.vec_off[s];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x / 32;
  for (int64_t c = warp; c < k; c += nwarps) {
    double acc = 0.0, acc2 = 0.0;
    int64_t i = k + lane;
    for (; i + 32 < m; i += 64) {
      acc += (double)F[i + c * m] * xf[rows[i]];
      acc2 += (double)F[i + 32 + c * m] * xf[rows[i + 32]];
    }
    if (i < m) acc += (double)F[i + c * m] * xf[rows[i]];
    acc += acc2;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) v[c] -= acc;
  }
  __syncthreads();
  for (int64_t c0 = ((k - 1) / kPanel) * kPanel; c0 >= 0; c0 -= kPanel) {
    const int cb = (int)(k - c0 < kPanel ? k - c0 : kPanel);
    for (int c = warp; c < cb; c += nwarps) {
      double acc = 0.0;
      for (int64_t i = c0 + cb + lane; i < k; i += 32) acc += (double)F[i + (c0 + c) * m] * v[i];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if (lane == 0) xb[c] = v[c0 + c] - acc;
    }
    __syncthreads();
    for (int c = cb - 1; c >= 0; c--) {
      const int t = threadIdx.x;
      if (t < c) xb[t] -= (double)F[(c0 + c) + (c0 + t) * m] * xb[c];
      __syncthreads();
    }
    if (threadIdx.x < cb) v[c0 + threadIdx.x] = xb[threadIdx.x];
    __syncthreads();
  }
  const int32_t f = d.sn_first[s];
  for (int64_t c = threadIdx.x; c < k; c += blockDim.x) xf[f + c] = v[c];
}

// Solves of the large supernodes, batched per level like their factorisation
// (blockIdx picks the supernode in the level's large list; each 64-pivot
// diagonal block applied through its stored inverse).

// after the forward panels: v[0:k] <- D^-1 v[0:k]
template <typename T>
__global__ void scale_pivots_kernel(BigBatch b, LdltDev d, const T* __restrict__ front,
                                    double* __restrict__ vec) {
  const int s = b.list[blockIdx.y];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const T* F = front + d.front_off[s];
  vec[d.vec_off[s] + c] /= (double)F[c + c * m];
}

// Products of the large supernodes' solves.  With FP64 fronts they are FP64
// FMAs.  With FP32 fronts the FP64 pipe (1/64 of the FP32 rate on this part,
// and the float -> double conversion runs on it too) would bound every pass,
// so a product f x of a front entry f and a vector entry x = xh + xl (two
// floats, |xl| <= ulp(xh)/2) is formed exactly in FP32 (p = f xh, e = fma(f,
// xh, -p)) and summed into a double-word accumulator (h, l) by TwoSum, l
// collecting the rounding errors and f xl: the compensated dot product Dot2
// of Ogita, Rump and Oishi (2005), error <= u |sum| + gamma_n^2 sum |f x|
// with u = 2^-24, far below the FP32 factor's own error.  Each accumulator
// adds in a fixed order, so a pass is run-to-run identical.
template <typename T>
struct Dot;

template <>
struct Dot<double> {
  using X = double;
  double s = 0.0;
  __device__ static X split(double x) { return x; }
  __device__ void add(double f, X x) { s = fma(f, x, s); }
  __device__ void merge(const Dot& o) { s += o.s; }
  __device__ void shfl_xor(int lanemask) { s += __shfl_xor_sync(0xffffffffu, s, lanemask); }
  __device__ void shfl_down(int delta) { s += __shfl_down_sync(0xffffffffu, s, delta); }
  __device__ double value() const { return s; }
};

template <>
struct Dot<float> {
  using X = float2;
  float h = 0.0f, l = 0.0f;
  __device__ static X split(double x) {
    const float xh = __double2float_rn(x);
    return make_float2(xh, __double2float_rn(x - (double)xh));
  }
  // h + l += b (TwoSum of h and b; the error joins l)
  __device__ void two_sum(float b, float bl) {
    const float sum = __fadd_rn(h, b);
    const float bv = __fsub_rn(sum, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(sum, bv)), __fsub_rn(b, bv));
    h = sum;
    l = __fadd_rn(l, __fadd_rn(err, bl));
  }
  __device__ void add(float f, X x) {
    const float p = __fmul_rn(f, x.x);
    two_sum(p, __fmaf_rn(f, x.y, __fmaf_rn(f, x.x, -p)));
  }
  __device__ void merge(const Dot& o) { two_sum(o.h, o.l); }
  __device__ void shfl_xor(int lanemask) {
    Dot o;
    o.h = __shfl_xor_sync(0xffffffffu, h, lanemask);
    o.l = __shfl_xor_sync(0xffffffffu, l, lanemask);
    merge(o);
  }
  __device__ void shfl_down(int delta) {
    Dot o;
    o.h = __shfl_down_sync(0xffffffffu, h, delta);
    o.l = __shfl_down_sync(0xffffffffu, l, delta);
    merge(o);
  }
  __device__ double value() const { return (double)h + (double)l; }
};

// FP32 fronts, FP64 products (the accurate mode of the refinement): the
// entry widened exactly by integer operations (re-biased exponent, shifted
// mantissa; zero by a select, subnormals and non-finite values by the
// conversion instruction), so that each product takes one FP64 FMA
__device__ __forceinline__ double widen(float f) {
  const uint32_t bits = __float_as_uint(f);
  const uint32_t mag = bits & 0x7FFFFFFFu;
  const uint32_t ex = bits & 0x7F800000u;
  if (mag != 0u && (ex == 0u || ex == 0x7F800000u)) return (double)f;
  const uint32_t sign = bits & 0x80000000u;
  const uint32_t hi = mag ? (sign | ((mag >> 3) + (896u << 20))) : sign;
  const uint32_t lo = mag ? (bits << 29) : 0u;
  return __hiloint2double((int)hi, (int)lo);
}

struct DotWide {
  using X = double;
  double s = 0.0;
  __device__ static X split(double x) { return x; }
  __device__ void add(float f, X x) { s = fma(widen(f), x, s); }
  __device__ void merge(const DotWide& o) { s += o.s; }
  __device__ void shfl_xor(int lanemask) { s += __shfl_xor_sync(0xffffffffu, s, lanemask); }
  __device__ void shfl_down(int delta) { s += __shfl_down_sync(0xffffffffu, s, delta); }
  __device__ double value() const { return s; }
};

// backward, before the large supernodes' triangles: the solved ancestor
// entries x[rows[i]], i >= k, gathered into v[k:m] (the update rows' slots,
// free once the forward pass has added them into the parent), in the
// products' operand form (a double, or its two-float split in its 8 bytes)
template <typename T, typename D>
__global__ void gather_rest_kernel(BigBatch b, LdltDev d, double* __restrict__ vec,
                                   const double* __restrict__ xf) {
  using X = typename D::X;
  static_assert(sizeof(X) == sizeof(double), "operand form fills a vector slot");
  const int s = b.list[blockIdx.y];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  const int64_t i = k + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  reinterpret_cast<X*>(vec + d.vec_off[s])[i] = D::split(xf[d.rows[d.row_ptr[s] + i]]);
}

// backward: t_c = v_c - sum_{i >= k} L[i][c] xr_i (xr gathered into v[k:m]),
// a warp per column: the column's contiguous segment and xr read by the
// lanes, eight loads of each in flight, eight partial sums merged in a fixed
// order
template <typename T, typename D>
__global__ void __launch_bounds__(kThreads)
    bwd_rest_kernel(BigBatch b, LdltDev d, const T* __restrict__ front,
                    double* __restrict__ vec) {
  using X = typename D::X;
  const int s = b.list[blockIdx.y];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t c = (int64_t)blockIdx.x * (kThreads / 32) + warp;
  if (c >= k) return;   // warp-uniform; no block barrier follows
  const T* Fc = front + d.front_off[s] + c * m;
  double* v = vec + d.vec_off[s];
  const X* xr = reinterpret_cast<const X*>(v);
  D acc[8];
  int64_t i = k + lane;
  for (; i + 7 * 32 < m; i += 8 * 32) {
    T f[8];
    X x[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      f[u] = Fc[i + 32 * u];
      x[u] = xr[i + 32 * u];
    }
#pragma unroll
    for (int u = 0; u < 8; u++) acc[u].add(f[u], x[u]);
  }
  for (; i < m; i += 32) acc[0].add(Fc[i], xr[i]);
#pragma unroll
  for (int u = 1; u < 8; u++) acc[0].merge(acc[u]);
  for (int o = 16; o > 0; o >>= 1) acc[0].shfl_down(o);
  if (lane == 0) v[c] -= acc[0].value();
}

// The forward and backward passes go by outer blocks of kOuter pivots (four
// panels), two launches per outer block and level: the block's own triangle
// by one CTA per supernode (panel by panel through the stored inverses, the
// rows / columns inside the block updated in shared memory), then the rows
// below it (forward) or the pivots before it (backward) with up to kOuter
// products per entry.  Every product chain is split so that its loads are
// issued together (the passes are bound by load latency, not bandwidth), and
// the partial sums are merged in a fixed order (run-to-run identical).

// forward, outer block o0: v_B <- L_BB^-1 v_B for the block's ob pivots.
// Per panel: y = Linv v_p, then the rows below the panel inside the block,
// both by four threads per row (16 products each, merged by shuffles).
template <typename T, typename D>
__global__ void __launch_bounds__(kThreads)
    fwd_block_kernel(BigBatch b, LdltDev d, const T* __restrict__ front,
                     const T* __restrict__ Linv, int64_t o0, double* __restrict__ vec) {
  using X = typename D::X;
  __shared__ double vb[kOuter];
  __shared__ X xs[kPanel];
  const int s = b.list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (o0 >= k) return;
  const int ob = (int)(k - o0 < kOuter ? k - o0 : kOuter);
  const T* F = front + d.front_off[s];
  double* v = vec + d.vec_off[s];
  const int t = threadIdx.x;
  if (t < ob) vb[t] = v[o0 + t];
  __syncthreads();
  const int r = t >> 2, q = t & 3;   // kThreads = 4 x kPanel
  for (int p = 0; p < ob; p += kPanel) {
    const int cb = ob - p < kPanel ? ob - p : kPanel;
    const T* Li = Linv + b.li_off[blockIdx.x] + (uint64_t)((o0 + p) / kPanel) * kPanel * kPanel;
    // (entries past cb are zero: the row products below read all kPanel)
    if (t < kPanel) xs[t] = D::split(t < cb ? vb[p + t] : 0.0);
    __syncthreads();
    // y_r = sum_c Linv[r][c] v_c (Linv's strict upper triangle holds zeros)
    D y;
    if (r < cb) {
      D y1;
#pragma unroll
      for (int j = 0; j < kPanel / 4; j += 2) {
        const int c0 = q + 4 * j, c1 = c0 + 4;
        if (c0 < cb) y.add(Li[r + c0 * kPanel], xs[c0]);
        if (c1 < cb) y1.add(Li[r + c1 * kPanel], xs[c1]);
      }
      y.merge(y1);
    }
    y.shfl_xor(1);
    y.shfl_xor(2);
    __syncthreads();
    if (r < cb && q == 0) {
      const double yv = y.value();
      vb[p + r] = yv;
      xs[r] = D::split(yv);
    }
    __syncthreads();
    // the rows below the panel inside the block: four threads per row, 16
    // columns each
    for (int i0 = p + cb; i0 < ob; i0 += kThreads / 4) {
      const int i = i0 + r;
      D a;
      if (i < ob) {
        const T* Fi = F + (o0 + i) + (o0 + p) * m;
        const int c0 = q * (kPanel / 4);
        T f[kPanel / 4];
#pragma unroll
        for (int u = 0; u < kPanel / 4; u++)
          f[u] = c0 + u < cb ? Fi[(int64_t)(c0 + u) * m] : T(0);
        D a1;
#pragma unroll
        for (int u = 0; u < kPanel / 4; u += 2) {
          a.add(f[u], xs[c0 + u]);
          a1.add(f[u + 1], xs[c0 + u + 1]);
        }
        a.merge(a1);
      }
      a.shfl_xor(1);
      a.shfl_xor(2);
      if (i < ob && q == 0) vb[i] -= a.value();
    }
    __syncthreads();
  }
  if (t < ob) v[o0 + t] = vb[t];
}

// forward, outer block o0: v[i] -= sum_c L[i][o0+c] y_c for the rows below the
// block, 32 rows per CTA: warp w takes the columns [32 w, 32 w + 32), lane =
// row (each load one coalesced 32-row segment of a column, 32 in flight),
// and the eight warps' partial sums are merged in a fixed order
template <typename T, typename D>
__global__ void __launch_bounds__(kThreads)
    fwd_rows_block_kernel(BigBatch b, LdltDev d, const T* __restrict__ front, int64_t o0,
                          double* __restrict__ vec) {
  using X = typename D::X;
  constexpr int kWarps = kThreads / 32;
  static_assert(kWarps * 32 == kOuter, "one warp per 32 columns of the outer block");
  __shared__ X yb[kOuter];
  __shared__ D part[kWarps][32];
  const int s = b.list[blockIdx.y];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (o0 >= k) return;
  const int ob = (int)(k - o0 < kOuter ? k - o0 : kOuter);
  const int64_t r0 = o0 + ob + (int64_t)blockIdx.x * 32;
  if (r0 >= m) return;
  const T* F = front + d.front_off[s];
  double* v = vec + d.vec_off[s];
  if (threadIdx.x < ob) yb[threadIdx.x] = D::split(v[o0 + threadIdx.x]);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i = r0 + lane;
  const int cbeg = warp * 32;
  D a0, a1, a2, a3;
  if (i < m && cbeg < ob) {
    const T* Fi = F + i + (o0 + cbeg) * m;
    if (ob - cbeg >= 32) {
      T f[32];
#pragma unroll
      for (int u = 0; u < 32; u++) f[u] = Fi[(int64_t)u * m];
#pragma unroll
      for (int u = 0; u < 32; u += 4) {
        a0.add(f[u], yb[cbeg + u]);
        a1.add(f[u + 1], yb[cbeg + u + 1]);
        a2.add(f[u + 2], yb[cbeg + u + 2]);
        a3.add(f[u + 3], yb[cbeg + u + 3]);
      }
    } else {
      for (int u = 0; u < ob - cbeg; u++) a0.add(Fi[(int64_t)u * m], yb[cbeg + u]);
    }
  }
  a0.merge(a1);
  a2.merge(a3);
  a0.merge(a2);
  part[warp][lane] = a0;
  __syncthreads();
  if (warp == 0 && i < m) {
    D sum = part[0][lane];
#pragma unroll
    for (int w = 1; w < kWarps; w++) sum.merge(part[w][lane]);
    v[i] -= sum.value();
  }
}

// backward, outer block o0: x_B = L_BB^-T t_B for the block's pivots.  Per
// panel (last first): the panel's inverse staged in shared memory (coalesced),
// x = Linv^T t_p by four threads per pivot, then t_j -= sum_c L[p+c][j] x_c
// for the block's pivots j before the panel by four threads per j (16
// contiguous products each), the partial sums merged by shuffles
template <typename T, typename D>
__global__ void __launch_bounds__(kThreads)
    bwd_block_kernel(BigBatch b, LdltDev d, const T* __restrict__ front,
                     const T* __restrict__ Linv, int64_t o0, double* __restrict__ vec) {
  using X = typename D::X;
  __shared__ double tb[kOuter];
  __shared__ X xs[kPanel];
  __shared__ T Ls[kPanel][kPanel + 1];   // Ls[c][r] = Linv[r][c]
  const int s = b.list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (o0 >= k) return;
  const int ob = (int)(k - o0 < kOuter ? k - o0 : kOuter);
  const T* F = front + d.front_off[s];
  double* v = vec + d.vec_off[s];
  const int t = threadIdx.x;
  if (t < ob) tb[t] = v[o0 + t];
  const int r = t >> 2, q = t & 3;   // kThreads = 4 x kPanel
  for (int p = ((ob - 1) / kPanel) * kPanel; p >= 0; p -= kPanel) {
    const int cb = ob - p < kPanel ? ob - p : kPanel;
    const T* Li = Linv + b.li_off[blockIdx.x] + (uint64_t)((o0 + p) / kPanel) * kPanel * kPanel;
#pragma unroll 4
    for (int e = t; e < kPanel * kPanel; e += kThreads) {
      const int er = e % kPanel, ec = e / kPanel;
      Ls[ec][er] = er < cb && ec < cb ? Li[er + ec * kPanel] : T(0);
    }
    __syncthreads();
    // (entries past cb are zero: the products below read all kPanel)
    if (t < kPanel) xs[t] = D::split(t < cb ? tb[p + t] : 0.0);
    __syncthreads();
    // x_r = sum_{c >= r} Linv[c][r] t_c
    D x;
    if (r < cb) {
      D x1;
#pragma unroll
      for (int j = 0; j < kPanel / 4; j += 2) {
        const int c0 = q + 4 * j, c1 = c0 + 4;
        if (c0 < cb) x.add(Ls[r][c0], xs[c0]);
        if (c1 < cb) x1.add(Ls[r][c1], xs[c1]);
      }
      x.merge(x1);
    }
    x.shfl_xor(1);
    x.shfl_xor(2);
    __syncthreads();
    if (r < cb && q == 0) {
      const double xv = x.value();
      tb[p + r] = xv;
      xs[r] = D::split(xv);
    }
    __syncthreads();
    // the pivots before the panel: column j's rows p .. p+cb, contiguous
    for (int j0 = 0; j0 < p; j0 += kThreads / 4) {
      const int j = j0 + r;
      D a;
      if (j < p) {
        const T* Fj = F + (o0 + p) + (o0 + j) * m;
        const int c0 = q * (kPanel / 4);
        T f[kPanel / 4];
#pragma unroll
        for (int u = 0; u < kPanel / 4; u++) f[u] = c0 + u < cb ? Fj[c0 + u] : T(0);
        D a1;
#pragma unroll
        for (int u = 0; u < kPanel / 4; u += 2) {
          a.add(f[u], xs[c0 + u]);
          a1.add(f[u + 1], xs[c0 + u + 1]);
        }
        a.merge(a1);
      }
      a.shfl_xor(1);
      a.shfl_xor(2);
      if (j < p && q == 0) tb[j] -= a.value();
    }
    __syncthreads();
  }
  if (t < ob) v[o0 + t] = tb[t];
}

// backward, outer block o0: t[j] -= sum_c L[o0+c][j] x_c for the pivots j < o0
// (a warp per column j, lanes over the block's rows, eight loads in flight)
template <typename T, typename D>
__global__ void __launch_bounds__(kThreads)
    bwd_cols_block_kernel(BigBatch b, LdltDev d, const T* __restrict__ front, int64_t o0,
                          double* __restrict__ vec) {
  using X = typename D::X;
  __shared__ X xb[kOuter];
  const int s = b.list[blockIdx.y];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (o0 >= k) return;
  const int64_t jbeg = (int64_t)blockIdx.x * 32;
  if (jbeg >= o0) return;
  const int ob = (int)(k - o0 < kOuter ? k - o0 : kOuter);
  const T* F = front + d.front_off[s];
  double* v = vec + d.vec_off[s];
  if (threadIdx.x < ob) xb[threadIdx.x] = D::split(v[o0 + threadIdx.x]);
  else if (threadIdx.x < kOuter) xb[threadIdx.x] = D::split(0.0);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t jend = jbeg + 32 < o0 ? jbeg + 32 : o0;
  for (int64_t j = jbeg + warp; j < jend; j += blockDim.x / 32) {
    const T* Fj = F + o0 + j * m;
    T f[kOuter / 32];
#pragma unroll
    for (int u = 0; u < kOuter / 32; u++) f[u] = lane + 32 * u < ob ? Fj[lane + 32 * u] : T(0);
    D a0, a1;
#pragma unroll
    for (int u = 0; u < kOuter / 32; u += 2) {
      a0.add(f[u], xb[lane + 32 * u]);
      a1.add(f[u + 1], xb[lane + 32 * (u + 1)]);
    }
    a0.merge(a1);
    for (int o = 16; o > 0; o >>= 1) a0.shfl_down(o);
    if (lane == 0) v[j] -= a0.value();
  }
}

// FP32 fronts: the block triangles with their operands staged in shared
// memory by asynchronous copies issued when the CTA starts (the stored
// inverses of the block's four panels and the block's strictly lower part,
// 166 KB), in the order the panels use them, so that the pass waits for one
// copy latency per block instead of a chain of them; everything after
// reads shared memory.  Columns are padded to 65 floats (two-way bank
// conflicts at most for the four-threads-per-row products).
constexpr int kLd = kPanel + 1;
constexpr int kStageLi = 4 * kPanel * kLd;    // the four inverses
constexpr int kStageTri = 6 * kPanel * kLd;   // panel pi >= 1: its rows x the 64 pi columns before it
constexpr size_t kStagedSmem = sizeof(float) * (kStageLi + kStageTri) + sizeof(double) * kOuter +
                               sizeof(double) * kPanel;
static_assert(kOuter == 4 * kPanel, "four panels per outer block");

__device__ __forceinline__ int tri_off(int pi) { return kPanel * kLd * (pi * (pi - 1) / 2); }

__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// this thread's copies of all but the `pending` most recent groups have landed
__device__ __forceinline__ void cp_async_wait(int pending) {
  switch (pending) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
  }
}

// forward, outer block o0, FP32 fronts (fwd_block_kernel's arithmetic): copy
// group g holds panel g's inverse and the columns of panel g in the rows of
// the later panels
template <typename D>
__global__ void __launch_bounds__(kThreads)
    fwd_block_staged_kernel(BigBatch b, LdltDev d, const float* __restrict__ front,
                            const float* __restrict__ Linv, int64_t o0,
                            double* __restrict__ vec) {
  using X = typename D::X;
  static_assert(sizeof(X) == sizeof(double), "operand slots of 8 bytes");
  extern __shared__ __align__(16) unsigned char staged_raw[];
  float* Ls = reinterpret_cast<float*>(staged_raw);
  float* Tb = Ls + kStageLi;
  double* vb = reinterpret_cast<double*>(Tb + kStageTri);
  X* xs = reinterpret_cast<X*>(vb + kOuter);
  const int s = b.list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (o0 >= k) return;
  const int ob = (int)(k - o0 < kOuter ? k - o0 : kOuter);
  const int np = (ob + kPanel - 1) / kPanel;
  const float* F = front + d.front_off[s];
  const float* Li0 = Linv + b.li_off[blockIdx.x] + (uint64_t)(o0 / kPanel) * kPanel * kPanel;
  double* v = vec + d.vec_off[s];
  const int t = threadIdx.x;
  for (int g = 0; g < np; g++) {
    const int cbg = ob - g * kPanel < kPanel ? ob - g * kPanel : kPanel;
    const float* Li = Li0 + (uint64_t)g * kPanel * kPanel;
    for (int e = t; e < kPanel * kPanel; e += kThreads) {
      const int er = e % kPanel, ec = e / kPanel;
      if (er < cbg && ec < cbg) cp_async4(Ls + g * kPanel * kLd + ec * kLd + er, Li + e);
    }
    for (int pi = g + 1; pi < np; pi++) {
      const int cbp = ob - pi * kPanel < kPanel ? ob - pi * kPanel : kPanel;
      for (int e = t; e < kPanel * kPanel; e += kThreads) {
        const int er = e % kPanel, ec = e / kPanel;
        if (er < cbp)
          cp_async4(Tb + tri_off(pi) + (g * kPanel + ec) * kLd + er,
                    F + (o0 + pi * kPanel + er) + (o0 + g * kPanel + ec) * m);
      }
    }
    cp_async_commit();
  }
  if (t < ob) vb[t] = v[o0 + t];
  const int r = t >> 2, q = t & 3;   // kThreads = 4 x kPanel
  for (int g = 0; g < np; g++) {
    const int p = g * kPanel;
    const int cb = ob - p < kPanel ? ob - p : kPanel;
    cp_async_wait(np - 1 - g);
    __syncthreads();
    if (t < kPanel) xs[t] = D::split(t < cb ? vb[p + t] : 0.0);
    __syncthreads();
    // y_r = sum_c Linv[r][c] v_c
    const float* L = Ls + g * kPanel * kLd;
    D y;
    if (r < cb) {
      D y1;
#pragma unroll
      for (int j = 0; j < kPanel / 4; j += 2) {
        const int c0 = q * (kPanel / 4) + j, c1 = c0 + 1;
        if (c0 < cb) y.add(L[c0 * kLd + r], xs[c0]);
        if (c1 < cb) y1.add(L[c1 * kLd + r], xs[c1]);
      }
      y.merge(y1);
    }
    y.shfl_xor(1);
    y.shfl_xor(2);
    __syncthreads();
    if (r < cb && q == 0) {
      const double yv = y.value();
      vb[p + r] = yv;
      xs[r] = D::split(yv);
    }
    __syncthreads();
    // the rows of the later panels: four threads per row, 16 columns each
    for (int i0 = p + cb; i0 < ob; i0 += kThreads / 4) {
      const int i = i0 + r;
      D a;
      if (i < ob) {
        const int pi = i / kPanel, rr = i - pi * kPanel;
        const float* Tr = Tb + tri_off(pi) + p * kLd + rr;
        D a1;
#pragma unroll
        for (int u = 0; u < kPanel / 4; u += 2) {
          const int c0 = q * (kPanel / 4) + u, c1 = c0 + 1;
          if (c0 < cb) a.add(Tr[c0 * kLd], xs[c0]);
          if (c1 < cb) a1.add(Tr[c1 * kLd], xs[c1]);
        }
        a.merge(a1);
      }
      a.shfl_xor(1);
      a.shfl_xor(2);
      if (i < ob && q == 0) vb[i] -= a.value();
    }
    __syncthreads();
  }
  if (t < ob) v[o0 + t] = vb[t];
}

// backward, outer block o0, FP32 fronts (bwd_block_kernel's arithmetic):
// copy groups in the backward order, group n = panel np-1-n's inverse and its
// rows in the columns before it
template <typename D>
__global__ void __launch_bounds__(kThreads)
    bwd_block_staged_kernel(BigBatch b, LdltDev d, const float* __restrict__ front,
                            const float* __restrict__ Linv, int64_t o0,
                            double* __restrict__ vec) {
  using X = typename D::X;
  static_assert(sizeof(X) == sizeof(double), "operand slots of 8 bytes");
  extern __shared__ __align__(16) unsigned char staged_raw[];
  float* Ls = reinterpret_cast<float*>(staged_raw);
  float* Tb = Ls + kStageLi;
  double* tb = reinterpret_cast<double*>(Tb + kStageTri);
  X* xs = reinterpret_cast<X*>(tb + kOuter);
  const int s = b.list[blockIdx.x];
  const int64_t m = d.row_ptr[s + 1] - d.row_ptr[s];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  if (o0 >= k) return;
  const int ob = (int)(k - o0 < kOuter ? k - o0 : kOuter);
  const int np = (ob + kPanel - 1) / kPanel;
  const float* F = front + d.front_off[s];
  const float* Li0 = Linv + b.li_off[blockIdx.x] + (uint64_t)(o0 / kPanel) * kPanel * kPanel;
  double* v = vec + d.vec_off[s];
  const int t = threadIdx.x;
  for (int g = np - 1; g >= 0; g--) {
    const int cbg = ob - g * kPanel < kPanel ? ob - g * kPanel : kPanel;
    const float* Li = Li0 + (uint64_t)g * kPanel * kPanel;
    for (int e = t; e < kPanel * kPanel; e += kThreads) {
      const int er = e % kPanel, ec = e / kPanel;
      if (er < cbg && ec < cbg) cp_async4(Ls + g * kPanel * kLd + ec * kLd + er, Li + e);
    }
    for (int e = t; e < kPanel * g * kPanel; e += kThreads) {
      const int er = e % kPanel, ec = e / kPanel;   // row er of panel g, column ec < 64 g
      if (er < cbg)
        cp_async4(Tb + tri_off(g) + ec * kLd + er, F + (o0 + g * kPanel + er) + (o0 + ec) * m);
    }
    cp_async_commit();
  }
  if (t < ob) tb[t] = v[o0 + t];
  const int r = t >> 2, q = t & 3;   // kThreads = 4 x kPanel
  for (int g = np - 1; g >= 0; g--) {
    const int p = g * kPanel;
    const int cb = ob - p < kPanel ? ob - p : kPanel;
    cp_async_wait(g);
    __syncthreads();
    if (t < kPanel) xs[t] = D::split(t < cb ? tb[p + t] : 0.0);
    __syncthreads();
    // x_r = sum_{c >= r} Linv[c][r] t_c (column r of the inverse)
    const float* L = Ls + g * kPanel * kLd + r * kLd;
    D x;
    if (r < cb) {
      D x1;
#pragma unroll
      for (int j = 0; j < kPanel / 4; j += 2) {
        const int c0 = q * (kPanel / 4) + j, c1 = c0 + 1;
        if (c0 < cb) x.add(L[c0], xs[c0]);
        if (c1 < cb) x1.add(L[c1], xs[c1]);
      }
      x.merge(x1);
    }
    x.shfl_xor(1);
    x.shfl_xor(2);
    __syncthreads();
    if (r < cb && q == 0) {
      const double xv = x.value();
      tb[p + r] = xv;
      xs[r] = D::split(xv);
    }
    __syncthreads();
    // the pivots before the panel: t_j -= sum_c L[p+c][j] x_c
    for (int j0 = 0; j0 < p; j0 += kThreads / 4) {
      const int j = j0 + r;
      D a;
      if (j < p) {
        const float* Tj = Tb + tri_off(g) + j * kLd;
        D a1;
#pragma unroll
        for (int u = 0; u < kPanel / 4; u += 2) {
          const int c0 = q * (kPanel / 4) + u, c1 = c0 + 1;
          if (c0 < cb) a.add(Tj[c0], xs[c0]);
          if (c1 < cb) a1.add(Tj[c1], xs[c1]);
        }
        a.merge(a1);
      }
      a.shfl_xor(1);
      a.shfl_xor(2);
      if (j < p && q == 0) tb[j] -= a.value();
    }
    __syncthreads();
  }
  if (t < ob) v[o0 + t] = tb[t];
}

// the solved pivots of the large supernodes into xf (factor order)
__global__ void store_pivots_kernel(BigBatch b, LdltDev d, const double* __restrict__ vec,
                                    double* __restrict__ xf) {
  const int s = b.list[blockIdx.y];
  const int64_t k = d.sn_first[s + 1] - d.sn_first[s];
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  xf[d.sn_first[s] + c] = vec[d.vec_off[s] + c];
}

__global__ void solve_finish_kernel(int64_t n, const int32_t* __restrict__ perm,
                                    const double* __restrict__ xf, double* __restrict__ x,
                                    int accumulate) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  if (accumulate)
    x[perm[j]] += xf[j];
  else
    x[perm[j]] = xf[j];
}

// r = b - A x, A by both-triangle rows (a warp per row, fixed order); per-block
// partial sums of r^2 and b^2 for the norms
__global__ void residual_kernel(int64_t n, const int64_t* __restrict__ ptr,
                                const int32_t* __restrict__ col, const uint32_t* __restrict__ slot,
                                const double* __restrict__ A, const double* __restrict__ x,
                                const double* __restrict__ b, double* __restrict__ r,
                                double* __restrict__ part) {
  __shared__ double red[2][kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row = blockIdx.x * (int64_t)(blockDim.x / 32) + warp;
  double rr = 0.0, bb = 0.0;
  if (row < n) {
    double acc = 0.0;
    for (int64_t q = ptr[row] + lane; q < ptr[row + 1]; q += 32) acc += A[slot[q]] * x[col[q]];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const double ri = b[row] - acc;
      r[row] = ri;
      rr = ri * ri;
      bb = b[row] * b[row];
    }
  }
  if (lane == 0) {
    red[0][warp] = rr;
    red[1][warp] = bb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int w = 0; w < kThreads / 32; w++) {
      a += red[0][w];
      c += red[1][w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = c;
  }
}

// ---- vector kernels of the GMRES refinement (fixed-order reductions) ----
constexpr int kDotBlocks = 1024;

__global__ void dot_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ part) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// y += alpha x
__global__ void axpy_kernel(int64_t n, double alpha, const double* __restrict__ x,
                            double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += alpha * x[i];
}

// y = alpha x
__global__ void scale_kernel(int64_t n, double alpha, const double* __restrict__ x,
                             double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = alpha * x[i];
}

// y = A x, A by both-triangle rows, a warp per row
__global__ void spmv_kernel(int64_t n, const int64_t* __restrict__ ptr,
                            const int32_t* __restrict__ col, const uint32_t* __restrict__ slot,
                            const double* __restrict__ A, const double* __restrict__ x,
                            double* __restrict__ y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row = blockIdx.x * (int64_t)(blockDim.x / 32) + warp;
  if (row >= n) return;
  double acc = 0.0;
  for (int64_t q = ptr[row] + lane; q < ptr[row + 1]; q += 32) acc += A[slot[q]] * x[col[q]];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc;
}

}  // namespace

struct nla3d_ldlt {
  LdltSymbolic S;
  int prec = 0;   // 0: FP64 fronts, 1: FP32 fronts (FP64 refinement)
  bool tc = false;   // FP32 fronts with the trailing updates on the tensor cores
  int* d_err = nullptr;
  double pivot_rel = 1e-13;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::vector<void*> allocs;
  void* d_front = nullptr;
  double* d_vec = nullptr;
  double* d_xf = nullptr;
  double* d_r = nullptr;
  double* d_dx = nullptr;
  double* d_part = nullptr;
  double* d_V = nullptr;        // GMRES basis, (kRestart + 1) x n, allocated on first use
  double* d_dot = nullptr;
  double* d_maxabs = nullptr;
  double* d_maxpart = nullptr;
  int* d_perturbed = nullptr;
  void* d_W = nullptr;
  void* d_Linv = nullptr;
  double* d_rhs = nullptr;      // the solve graph's right-hand side
  double* d_hb = nullptr;       // nla3d_ldlt_solve_host: b and x on the device
  double* d_hx = nullptr;
  cudaGraphExec_t factor_exec = nullptr, solve_exec = nullptr;
  // FP32 fronts: the solve with FP64 products (the refinement's accurate
  // mode, after the compensated-FP32 one stalls), and the mode in use
  cudaGraphExec_t solve_exec_acc = nullptr;
  int solve_accurate = 0;
  const double* factor_graph_values = nullptr;
  uint64_t* d_wo = nullptr;
  uint64_t* d_lio = nullptr;
  uint64_t* d_pko = nullptr;    // tensor-core fronts: packed outer-block operand offsets
  float* d_pk = nullptr;
  OuterTile* d_tiles = nullptr; // tensor-core fronts: every level's outer-block tile lists
  int n_sm = 0;
  uint64_t* d_adest = nullptr;
  int32_t* d_perm = nullptr;
  int32_t* d_col2sn = nullptr;
  int32_t* d_lists = nullptr;   // level lists, small lists, extend-add child lists
  int64_t* d_fptr = nullptr;
  int32_t* d_fcol = nullptr;
  uint32_t* d_fslot = nullptr;
  LdltDev dev{};
  // host schedule per level
  struct Level {
    int64_t all_off = 0, all_cnt = 0;     // every supernode of the level
    int64_t small_off = 0, small_cnt = 0;
    int32_t small_max_m = 0;
    int64_t large_off = 0, large_cnt = 0; // fronts above kSmallFront rows
    int64_t wo_off = 0;                   // their W offsets in d_wo
    int64_t large_max_m = 0, large_max_k = 0;
    std::vector<int64_t> tile_off, tile_cnt;  // tensor-core fronts: per outer block, its tiles
    std::vector<int64_t> itile_off, itile_cnt;  // and per panel, its in-block update's tiles
    std::vector<int64_t> ea_off, ea_cnt;  // children of the level's parents, by ordinal
    std::vector<uint32_t> ea_gy;          // column blocks per child (its update's size)
  };
  std::vector<Level> levels;
  bool factored = false;
  int perturbed[2] = {0, 0};
  uint64_t front_entries = 0;
};

namespace {

int fail(nla3d_ldlt* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(nla3d_ldlt* h, cudaError_t e, const char* where) {
  return fail(h, NLA3D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename X>
cudaError_t dalloc(nla3d_ldlt* h, X** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, sizeof(X) * (count ? count : 1));
  if (e == cudaSuccess) {
    h->allocs.push_back(q);
    *p = static_cast<X*>(q);
  }
  return e;
}

template <typename X>
cudaError_t upload(nla3d_ldlt* h, X** p, const std::vector<X>& v) {
  cudaError_t e = dalloc(h, p, v.size());
  if (e == cudaSuccess && !v.empty())
    e = cudaMemcpyAsync(*p, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice, h->stream);
  return e;
}

template <typename T>
cudaError_t enqueue_factor(nla3d_ldlt* h, const double* values) {
  const LdltSymbolic& S = h->S;
  T* front = static_cast<T*>(h->d_front);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemsetAsync(front, 0, sizeof(T) * h->front_entries, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(h->d_perturbed, 0, 2 * sizeof(int), st);
  if (e != cudaSuccess) return e;
  {
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(
        kMaxBlocks, (S.nnz + kThreads - 1) / kThreads));
    maxabs_kernel<<<blocks, kThreads, 0, st>>>(S.nnz, values, h->d_maxpart);
    maxabs_final_kernel<<<1, kThreads, 0, st>>>(blocks, h->d_maxpart, h->d_maxabs);
  }
  if (S.nnz) {
    const unsigned blocks = (unsigned)std::min<uint64_t>((S.nnz + kThreads - 1) / kThreads, 152 * 16);
    scatter_values_kernel<T><<<blocks, kThreads, 0, st>>>(S.nnz, h->d_adest, values, front);
  }
  for (const auto& L : h->levels) {
    for (size_t q = 0; q < L.ea_off.size(); q++) {
      if (!L.ea_cnt[q]) continue;
      const dim3 grid((unsigned)L.ea_cnt[q], L.ea_gy[q]);
      extend_add_kernel<T><<<grid, kThreads, 0, st>>>(h->d_lists + L.ea_off[q], (int)L.ea_cnt[q],
                                                      h->dev, front);
    }
    if (L.small_cnt) {
      const size_t smem = sizeof(T) * (size_t)L.small_max_m * (L.small_max_m + 1);
      factor_small_kernel<T><<<(unsigned)L.small_cnt, kThreads, smem, st>>>(
          h->d_lists + L.small_off, h->dev, front, h->d_maxabs, h->pivot_rel, h->d_perturbed);
    }
    if (L.large_cnt) {
      const BigBatch bb{h->d_lists + L.large_off, h->d_wo + L.wo_off, h->d_lio + L.wo_off,
                        h->d_pko ? h->d_pko + L.wo_off : nullptr};
      T* W = static_cast<T*>(h->d_W);
      T* Li = static_cast<T*>(h->d_Linv);
      const unsigned nf = (unsigned)L.large_cnt;
      constexpr int BT = TrailingShape<T>::BT, RT = TrailingShape<T>::RT;
      const bool tc = std::is_same<T, float>::value && h->tc;
      // one FMA update launch: rows from its range's first column to the
      // largest front's last row, `col_tiles` tiles of columns
      auto update = [&](int64_t p, int outer, int64_t rows, unsigned col_tiles) {
        const unsigned rt = (unsigned)((rows + BT - 1) / BT);
        const dim3 grid(rt, std::min(rt, col_tiles), nf);
        batched_trailing_kernel<T, BT, RT><<<grid, kThreads, 0, st>>>(bb, h->dev, front, p,
                                                                       outer, W);
      };
      for (int64_t o0 = 0; o0 < L.large_max_k; o0 += kOuter) {
        const int64_t o_end = std::min<int64_t>(o0 + kOuter, L.large_max_k);
        for (int64_t p0 = o0; p0 < o_end; p0 += kPanel) {
          batched_diag_kernel<T><<<nf, kThreads, 2 * sizeof(T) * kPanel * (kPanel + 1), st>>>(
              bb, h->dev, front, p0, Li, h->d_maxabs, h->pivot_rel, h->d_perturbed);
          const int64_t rest = L.large_max_m - p0 - 1;   // rows past the smallest panel
          if (rest <= 0) continue;
          const unsigned tiles = (unsigned)((rest + kTile - 1) / kTile);
          batched_panel_kernel<T><<<dim3(tiles, nf), kThreads, 0, st>>>(bb, h->dev, front, p0,
                                                                         Li, W);
          // the panel's columns into the rest of its outer block (at most
          // kOuter - kPanel columns)
          if (p0 + kPanel < o_end) {
            const int64_t pi = p0 / kPanel;
            if (tc && L.itile_cnt[pi] > 0) {
              const unsigned rb = (unsigned)((rest + kTcM - 1) / kTcM);
              pack_update_kernel<<<dim3(rb, kPanel / kTcKH, nf), kTcThreads, 0, st>>>(
                  bb, h->dev, reinterpret_cast<const float*>(front), p0, 0,
                  reinterpret_cast<const float*>(W), h->d_pk);
              const int nt = (int)L.itile_cnt[pi];
              tc_packed_kernel<<<(unsigned)std::min(nt, h->n_sm), kOuterThreads, kPkSmem, st>>>(
                  bb, h->dev, reinterpret_cast<float*>(front), p0, 0, h->d_pk,
                  h->d_tiles + L.itile_off[pi], nt, h->d_err);
            } else if (!tc) {
              update(p0, 0, rest, (unsigned)((kOuter - kPanel + BT - 1) / BT));
            }
          }
        }
        // the outer block into every column after it (tensor-core fronts:
        // its operands packed once, then the tiles with bulk copies)
        const int64_t rest = L.large_max_m - o0 - 1;
        if (rest > 0 && tc) {
          const unsigned rb = (unsigned)((rest + kTcM - 1) / kTcM);
          pack_update_kernel<<<dim3(rb, kPkChunks, nf), kTcThreads, 0, st>>>(
              bb, h->dev, reinterpret_cast<const float*>(front), o0, 1,
              reinterpret_cast<const float*>(W), h->d_pk);
          const int64_t ob = o0 / kOuter;
          const int nt = (int)L.tile_cnt[ob];
          if (nt > 0)
            tc_packed_kernel<<<(unsigned)std::min(nt, h->n_sm), kOuterThreads, kPkSmem, st>>>(
                bb, h->dev, reinterpret_cast<float*>(front), o0, 1, h->d_pk,
                h->d_tiles + L.tile_off[ob], nt, h->d_err);
        } else if (rest > 0) {
          update(o0, 1, rest, ~0u);
        }
      }
    }
  }
  return cudaGetLastError();
}

template <typename T, typename D>
cudaError_t enqueue_solve_core(nla3d_ldlt* h, const double* b) {
  const LdltSymbolic& S = h->S;
  const T* front = static_cast<const T*>(h->d_front);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemsetAsync(h->d_vec, 0, sizeof(double) * S.vec_off.back(), st);
  if (e != cudaSuccess) return e;
  const unsigned nb = (unsigned)((S.n + kThreads - 1) / kThreads);
  solve_init_kernel<<<nb, kThreads, 0, st>>>(S.n, h->d_perm, h->d_col2sn, h->dev, b, h->d_vec);
  const T* Li = static_cast<const T*>(h->d_Linv);
  for (const auto& L : h->levels) {
    for (size_t q = 0; q < L.ea_off.size(); q++)
      if (L.ea_cnt[q])
        vec_extend_add_kernel<<<(unsigned)L.ea_cnt[q], kThreads, 0, st>>>(h->d_lists + L.ea_off[q],
                                                                           h->dev, h->d_vec);
    if (L.small_cnt)
      forward_kernel<T><<<(unsigned)L.small_cnt, kThreads, 0, st>>>(h->d_lists + L.small_off,
                                                                    h->dev, front, h->d_vec);
    if (L.large_cnt) {
      const BigBatch bb{h->d_lists + L.large_off, h->d_wo + L.wo_off, h->d_lio + L.wo_off};
      const unsigned nf = (unsigned)L.large_cnt;
      for (int64_t o0 = 0; o0 < L.large_max_k; o0 += kOuter) {
        if constexpr (std::is_same<T, float>::value)
          fwd_block_staged_kernel<D><<<nf, kThreads, kStagedSmem, st>>>(bb, h->dev, front, Li, o0,
                                                                        h->d_vec);
        else
          fwd_block_kernel<T, D><<<nf, kThreads, 0, st>>>(bb, h->dev, front, Li, o0, h->d_vec);
        const int64_t rest = L.large_max_m - o0 - 1;
        if (rest > 0)
          fwd_rows_block_kernel<T, D><<<dim3((unsigned)((rest + 31) / 32), nf),
                                     kThreads, 0, st>>>(bb, h->dev, front, o0, h->d_vec);
      }
      scale_pivots_kernel<T><<<dim3((unsigned)((L.large_max_k + kThreads - 1) / kThreads), nf),
                               kThreads, 0, st>>>(bb, h->dev, front, h->d_vec);
    }
  }
  for (auto it = h->levels.rbegin(); it != h->levels.rend(); ++it) {
    const auto& L = *it;
    if (L.small_cnt)
      backward_kernel<T><<<(unsigned)L.small_cnt, kThreads, 0, st>>>(h->d_lists + L.small_off,
                                                                     h->dev, front, h->d_vec,
                                                                     h->d_xf);
    if (L.large_cnt) {
      const BigBatch bb{h->d_lists + L.large_off, h->d_wo + L.wo_off, h->d_lio + L.wo_off};
      const unsigned nf = (unsigned)L.large_cnt;
      const int64_t rest = L.large_max_m - 1;
      gather_rest_kernel<T, D><<<dim3((unsigned)((rest + kThreads - 1) / kThreads), nf), kThreads,
                              0, st>>>(bb, h->dev, h->d_vec, h->d_xf);
      bwd_rest_kernel<T, D><<<dim3((unsigned)((L.large_max_k + kThreads / 32 - 1) / (kThreads / 32)),
                                nf),
                           kThreads, 0, st>>>(bb, h->dev, front, h->d_vec);
      for (int64_t o0 = ((L.large_max_k - 1) / kOuter) * kOuter; o0 >= 0; o0 -= kOuter) {
        if constexpr (std::is_same<T, float>::value)
          bwd_block_staged_kernel<D><<<nf, kThreads, kStagedSmem, st>>>(bb, h->dev, front, Li, o0,
                                                                        h->d_vec);
        else
          bwd_block_kernel<T, D><<<nf, kThreads, 0, st>>>(bb, h->dev, front, Li, o0, h->d_vec);
        if (o0 > 0)
          bwd_cols_block_kernel<T, D><<<dim3((unsigned)((o0 + 31) / 32), nf), kThreads, 0, st>>>(
              bb, h->dev, front, o0, h->d_vec);
      }
      store_pivots_kernel<<<dim3((unsigned)((L.large_max_k + kThreads - 1) / kThreads), nf),
                            kThreads, 0, st>>>(bb, h->dev, h->d_vec, h->d_xf);
    }
  }
  return cudaGetLastError();
}

cudaError_t enqueue_residual(nla3d_ldlt* h, const double* A, const double* x, const double* b) {
  const LdltSymbolic& S = h->S;
  const int64_t rows_per_block = kThreads / 32;
  const unsigned blocks = (unsigned)((S.n + rows_per_block - 1) / rows_per_block);
  residual_kernel<<<blocks, kThreads, 0, h->stream>>>(S.n, h->d_fptr, h->d_fcol, h->d_fslot, A, x,
                                                     b, h->d_r, h->d_part);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int nla3d_ldlt_order(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                     const double* points, int64_t n_dofs, int32_t* order) {
  const std::string msg = ldlt_nd_order(n, iofeir, columns, points, n_dofs, order);
  return msg.empty() ? NLA3D_OK : NLA3D_ERR_ARG;
}

int nla3d_ldlt_analyze(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                       const int32_t* perm, double* stats, int32_t* perm_out, int32_t* sn_first_out,
                       int64_t* row_ptr_out, int32_t* rows_out) {
  if (!stats) return NLA3D_ERR_ARG;
  LdltSymbolic S;
  const std::string msg = ldlt_analyze(n, iofeir, columns, perm, &S);
  if (!msg.empty()) return NLA3D_ERR_ARG;
  stats[0] = (double)S.n_sn();
  stats[1] = (double)(S.level_ptr.size() - 1);
  stats[2] = (double)S.max_front;
  stats[3] = (double)S.nnz_L;
  stats[4] = S.flops;
  stats[5] = (double)S.front_off.back();
  stats[6] = (double)S.max_children;
  stats[7] = (double)S.rows.size();
  if (perm_out) std::copy(S.perm.begin(), S.perm.end(), perm_out);
  if (sn_first_out) std::copy(S.sn_first.begin(), S.sn_first.end(), sn_first_out);
  if (row_ptr_out) std::copy(S.row_ptr.begin(), S.row_ptr.end(), row_ptr_out);
  if (rows_out) std::copy(S.rows.begin(), S.rows.end(), rows_out);
  return NLA3D_OK;
}

int nla3d_ldlt_create(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                      const int32_t* perm, int precision, void* stream, nla3d_ldlt** out) {
  if (!out || precision < 0 || precision > 2) return NLA3D_ERR_ARG;
  *out = nullptr;
  nla3d_ldlt* h = new nla3d_ldlt();
  h->tc = precision == 2;
  if (precision == 2) precision = 1;
  h->prec = precision;
  if (precision == 1) h->pivot_rel = 1e-7;
  const std::string msg = ldlt_analyze(n, iofeir, columns, perm, &h->S);
  if (!msg.empty()) {
    delete h;
    return NLA3D_ERR_ARG;
  }
  const LdltSymbolic& S = h->S;
  h->front_entries = S.front_off.back();
  // the schedule: per level, all / small / large supernodes, children by ordinal
  const int64_t ns = S.n_sn();
  const int nlev = (int)S.level_ptr.size() - 1;
  std::vector<int32_t> lists;
  std::vector<int32_t> col2sn(S.n);
  for (int64_t s = 0; s < ns; s++)
    for (int32_t t = S.sn_first[s]; t < S.sn_first[s + 1]; t++) col2sn[t] = (int32_t)s;
  std::vector<uint64_t> wo, lio, pko;
  std::vector<OuterTile> tiles;
  int64_t max_w = 0, max_large_cnt = 0, max_pk = 0;
  uint64_t li_total = 0;
  h->levels.resize(nlev);
  for (int L = 0; L < nlev; L++) {
    auto& lv = h->levels[L];
    lv.all_off = (int64_t)lists.size();
    for (int32_t q = S.level_ptr[L]; q < S.level_ptr[L + 1]; q++) lists.push_back(S.level_list[q]);
    lv.all_cnt = (int64_t)lists.size() - lv.all_off;
    lv.small_off = (int64_t)lists.size();
    for (int32_t q = S.level_ptr[L]; q < S.level_ptr[L + 1]; q++) {
      const int32_t s = S.level_list[q];
      if (S.m(s) <= kSmallFront) {
        lists.push_back(s);
        lv.small_max_m = std::max(lv.small_max_m, S.m(s));
      }
    }
    lv.small_cnt = (int64_t)lists.size() - lv.small_off;
    lv.large_off = (int64_t)lists.size();
    lv.wo_off = (int64_t)wo.size();
    int64_t w = 0, pk = 0;
    for (int32_t q = S.level_ptr[L]; q < S.level_ptr[L + 1]; q++) {
      const int32_t s = S.level_list[q];
      if (S.m(s) > kSmallFront) {
        lists.push_back(s);
        wo.push_back((uint64_t)w);
        w += (int64_t)S.m(s) *
             std::min<int64_t>(kOuter, ((int64_t)S.k(s) + kPanel - 1) / kPanel * kPanel);
        lio.push_back(li_total);
        pko.push_back((uint64_t)pk);
        pk += ((int64_t)S.m(s) + kTcM - 1) / kTcM * (int64_t)kPkBlock;
        li_total += (uint64_t)((S.k(s) + kPanel - 1) / kPanel) * kPanel * kPanel;
        lv.large_max_m = std::max<int64_t>(lv.large_max_m, S.m(s));
        lv.large_max_k = std::max<int64_t>(lv.large_max_k, S.k(s));
      }
    }
    lv.large_cnt = (int64_t)lists.size() - lv.large_off;
    if (h->tc) {
      // every outer block's update tiles (the rule of update_range, outer):
      // per front with k > o0, rows and columns from jb = min(o0 + kOuter, k)
      for (int64_t o0 = 0; o0 < lv.large_max_k; o0 += kOuter) {
        lv.tile_off.push_back((int64_t)tiles.size());
        for (int64_t z = 0; z < lv.large_cnt; z++) {
          const int32_t s = lists[lv.large_off + z];
          const int64_t k = S.k(s), m = S.m(s);
          if (o0 >= k) continue;
          const int64_t jb = std::min<int64_t>(o0 + kOuter, k);
          if (jb >= m) continue;
          const int64_t rb = (m - jb + kTcM - 1) / kTcM;
          for (int64_t ti = 0; ti < rb; ti++)
            for (int64_t tj = 0; tj <= ti; tj++)
              tiles.push_back(OuterTile{(uint32_t)z, (uint32_t)(ti << 16 | tj)});
        }
        lv.tile_cnt.push_back((int64_t)tiles.size() - lv.tile_off.back());
      }
      // every panel's in-block update (update_range, inner): rows from
      // jb = p0 + pb, columns jb .. min(o0 + kOuter, k)
      for (int64_t p0 = 0; p0 < lv.large_max_k; p0 += kPanel) {
        lv.itile_off.push_back((int64_t)tiles.size());
        const int64_t o0 = p0 - p0 % kOuter;
        for (int64_t z = 0; z < lv.large_cnt; z++) {
          const int32_t s = lists[lv.large_off + z];
          const int64_t k = S.k(s), m = S.m(s);
          if (p0 >= k) continue;
          const int64_t jb = p0 + std::min<int64_t>(kPanel, k - p0);
          const int64_t je = std::min<int64_t>(o0 + kOuter, k);
          if (jb >= je) continue;
          const int64_t rb = (m - jb + kTcM - 1) / kTcM, cb = (je - jb + kTcN - 1) / kTcN;
          for (int64_t ti = 0; ti < rb; ti++)
            for (int64_t tj = 0; tj <= ti && tj < cb; tj++)
              tiles.push_back(OuterTile{(uint32_t)z, (uint32_t)(ti << 16 | tj)});
        }
        lv.itile_cnt.push_back((int64_t)tiles.size() - lv.itile_off.back());
      }
    }
    max_w = std::max(max_w, w);
    max_pk = std::max(max_pk, pk);
    max_large_cnt = std::max(max_large_cnt, lv.large_cnt);
    int maxc = 0;
    for (int32_t q = S.level_ptr[L]; q < S.level_ptr[L + 1]; q++) {
      const int32_t s = S.level_list[q];
      maxc = std::max(maxc, S.child_ptr[s + 1] - S.child_ptr[s]);
    }
    for (int o = 0; o < maxc; o++) {
      lv.ea_off.push_back((int64_t)lists.size());
      int64_t umax = 0;
      for (int32_t q = S.level_ptr[L]; q < S.level_ptr[L + 1]; q++) {
        const int32_t s = S.level_list[q];
        if (S.child_ptr[s + 1] - S.child_ptr[s] > o) {
          const int32_t c = S.child_list[S.child_ptr[s] + o];
          lists.push_back(c);
          umax = std::max<int64_t>(umax, S.m(c) - S.k(c));
        }
      }
      lv.ea_cnt.push_back((int64_t)lists.size() - lv.ea_off.back());
      // about 32 update columns per block, 16 .. 1024 blocks per child
      lv.ea_gy.push_back((uint32_t)std::min<int64_t>(1024, std::max<int64_t>(16, (umax + 31) / 32)));
    }
  }
  if (lists.size() >= (size_t)INT32_MAX || max_large_cnt > 65535) {
    delete h;
    return NLA3D_ERR_RANGE;
  }
  cudaError_t e = cudaSuccess;
  if (stream) {
    h->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete h;
      return NLA3D_ERR_CUDA;
    }
    h->own_stream = true;
  }
  size_t free_b = 0, total_b = 0;
  e = cudaMemGetInfo(&free_b, &total_b);
  const size_t tsize = precision ? sizeof(float) : sizeof(double);
  const double need = (double)h->front_entries * tsize + (double)S.nnz * 8 + (double)S.n * 64 +
                      (double)S.full_col.size() * 8 + (double)S.rows.size() * 8;
  int rc = NLA3D_OK;
  if (e != cudaSuccess)
    rc = cuda_fail(h, e, "cudaMemGetInfo");
  else if (need > 0.9 * (double)free_b)
    rc = fail(h, NLA3D_ERR_NOMEM, "fronts need more device memory than is free");
#define LCK(x)                                  \
  do {                                          \
    if (rc == NLA3D_OK) {                       \
      cudaError_t _e = (x);                     \
      if (_e != cudaSuccess) rc = cuda_fail(h, _e, #x); \
    }                                           \
  } while (0)
  if (precision)
    LCK(dalloc(h, reinterpret_cast<float**>(&h->d_front), h->front_entries));
  else
    LCK(dalloc(h, reinterpret_cast<double**>(&h->d_front), h->front_entries));
  const size_t nlinv = (size_t)std::max<uint64_t>(li_total, 1);
  if (precision) {
    LCK(dalloc(h, reinterpret_cast<float**>(&h->d_W), (size_t)max_w));
    LCK(dalloc(h, reinterpret_cast<float**>(&h->d_Linv), nlinv));
    LCK(cudaFuncSetAttribute(batched_diag_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(2 * sizeof(float) * kPanel * (kPanel + 1))));
    LCK(cudaFuncSetAttribute(factor_small_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(float) * kSmallFront * (kSmallFront + 1))));
  } else {
    LCK(dalloc(h, reinterpret_cast<double**>(&h->d_W), (size_t)max_w));
    LCK(dalloc(h, reinterpret_cast<double**>(&h->d_Linv), nlinv));
    LCK(cudaFuncSetAttribute(batched_diag_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(2 * sizeof(double) * kPanel * (kPanel + 1))));
    LCK(cudaFuncSetAttribute(factor_small_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double) * kSmallFront * (kSmallFront + 1))));
  }
  LCK(upload(h, &h->d_wo, wo));
  LCK(upload(h, &h->d_lio, lio));
  LCK(dalloc(h, &h->d_vec, S.vec_off.back()));
  LCK(dalloc(h, &h->d_xf, S.n));
  LCK(dalloc(h, &h->d_rhs, S.n));
  LCK(dalloc(h, &h->d_r, S.n));
  LCK(dalloc(h, &h->d_dx, S.n));
  LCK(dalloc(h, &h->d_part, 2 * ((S.n + 7) / 8 + 1)));
  LCK(dalloc(h, &h->d_dot, kDotBlocks));
  LCK(dalloc(h, &h->d_maxabs, 1));
  LCK(dalloc(h, &h->d_maxpart, kMaxBlocks));
  LCK(dalloc(h, &h->d_perturbed, 2));
  LCK(dalloc(h, &h->d_err, 1));
  LCK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
  if (h->tc) {
    LCK(cudaFuncSetAttribute(tc_packed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kPkSmem));
    LCK(upload(h, &h->d_pko, pko));
    LCK(dalloc(h, &h->d_pk, (size_t)std::max<int64_t>(max_pk, 1)));
    LCK(upload(h, &h->d_tiles, tiles));
    int dev = 0;
    LCK(cudaGetDevice(&dev));
    LCK(cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, dev));
  }
  LCK(upload(h, &h->d_adest, S.a_dest));
  LCK(upload(h, &h->d_perm, S.perm));
  LCK(upload(h, &h->d_col2sn, col2sn));
  LCK(upload(h, &h->d_lists, lists));
  LCK(upload(h, &h->d_fptr, S.full_ptr));
  LCK(upload(h, &h->d_fcol, S.full_col));
  LCK(upload(h, &h->d_fslot, S.full_slot));
  uint64_t *fo = nullptr, *vo = nullptr;
  int64_t *rp = nullptr, *relp = nullptr;
  int32_t *rw = nullptr, *sf = nullptr, *sp = nullptr;
  uint32_t* rl = nullptr;
  LCK(upload(h, &fo, S.front_off));
  LCK(upload(h, &vo, S.vec_off));
  LCK(upload(h, &rp, S.row_ptr));
  LCK(upload(h, &rw, S.rows));
  LCK(upload(h, &sf, S.sn_first));
  LCK(upload(h, &sp, S.sn_parent));
  LCK(upload(h, &relp, S.rel_ptr));
  LCK(upload(h, &rl, S.rel));
  LCK(cudaStreamSynchronize(h->stream));
#undef LCK
  h->dev = LdltDev{fo, vo, rp, rw, sf, sp, relp, rl};
  if (rc != NLA3D_OK) {
    // keep the handle so that the caller can read the message, then destroy it
    *out = h;
    return rc;
  }
  *out = h;
  return NLA3D_OK;
}

const char* nla3d_ldlt_last_error(const nla3d_ldlt* h) { return h ? h->err.c_str() : "null handle"; }

int nla3d_ldlt_info(const nla3d_ldlt* h, double* out) {
  if (!h || !out) return NLA3D_ERR_ARG;
  const LdltSymbolic& S = h->S;
  out[0] = (double)S.n_sn();
  out[1] = (double)h->levels.size();
  out[2] = (double)S.max_front;
  out[3] = (double)S.nnz_L;
  out[4] = S.flops;
  out[5] = (double)h->front_entries * (h->prec ? 4.0 : 8.0);
  out[6] = (double)h->perturbed[0];
  out[7] = (double)h->perturbed[1];
  return NLA3D_OK;
}

int nla3d_ldlt_factor(nla3d_ldlt* h, const double* values) {
  if (!h || !values) return fail(h, NLA3D_ERR_ARG, "ldlt_factor: null argument");
  if (!h->d_front) return fail(h, NLA3D_ERR_ARG, "ldlt_factor: the handle was not set up");
  // the factorisation's kernel sequence is captured once per values array
  // into a CUDA graph and replayed
  cudaError_t e = cudaSuccess;
  if (!h->factor_exec || h->factor_graph_values != values) {
    if (h->factor_exec) cudaGraphExecDestroy(h->factor_exec);
    h->factor_exec = nullptr;
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const cudaError_t ec = h->prec ? enqueue_factor<float>(h, values)
                                     : enqueue_factor<double>(h, values);
      e = cudaStreamEndCapture(h->stream, &g);
      if (ec != cudaSuccess) e = ec;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&h->factor_exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) h->factor_exec = nullptr;
      h->factor_graph_values = values;
    }
  }
  if (e == cudaSuccess) e = cudaGraphLaunch(h->factor_exec, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->perturbed, h->d_perturbed, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                        h->stream);
  int tc_err = 0;
  if (e == cudaSuccess && h->tc)
    e = cudaMemcpyAsync(&tc_err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "ldlt_factor");
  if (tc_err) {
    h->factored = false;
    return fail(h, NLA3D_ERR_CUDA, "ldlt_factor: a tensor-core tile timed out waiting for its MMAs");
  }
  h->factored = true;
  if (h->perturbed[1]) return fail(h, NLA3D_ERR_ELEMENT, "ldlt_factor: a non-finite pivot");
  return NLA3D_OK;
}

}  // extern "C"

namespace {

constexpr int kRestart = 30;

unsigned vec_blocks(int64_t n) {
  return (unsigned)std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 8);
}

// the solve's kernel sequence (a few thousand launches on large models) is
// captured once into a CUDA graph reading d_rhs and leaving the factor-order
// solution in d_xf; each solve copies its right-hand side in, replays the
// graph and scatters (or adds) the result into `out`
cudaError_t enqueue_solve_any(nla3d_ldlt* h, const double* rhs, double* out, int acc) {
  cudaError_t e = cudaSuccess;
  // FP64 fronts have one mode; FP32 fronts: compensated FP32 products, or
  // FP64 ones in the accurate mode
  const bool accurate = h->prec && h->solve_accurate;
  cudaGraphExec_t& exec = accurate ? h->solve_exec_acc : h->solve_exec;
  if (!exec) {
    if (h->prec) {
      // the staged block triangles take more than the default 48 KB
      const void* kf[4] = {(const void*)fwd_block_staged_kernel<Dot<float>>,
                           (const void*)bwd_block_staged_kernel<Dot<float>>,
                           (const void*)fwd_block_staged_kernel<DotWide>,
                           (const void*)bwd_block_staged_kernel<DotWide>};
      for (const void* f : kf) {
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStagedSmem);
        if (e != cudaSuccess) return e;
      }
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const cudaError_t ec =
        !h->prec ? enqueue_solve_core<double, Dot<double>>(h, h->d_rhs)
        : accurate ? enqueue_solve_core<float, DotWide>(h, h->d_rhs)
                   : enqueue_solve_core<float, Dot<float>>(h, h->d_rhs);
    e = cudaStreamEndCapture(h->stream, &g);
    if (ec != cudaSuccess) e = ec;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      exec = nullptr;
      return e;
    }
  }
  if (rhs != h->d_rhs)
    e = cudaMemcpyAsync(h->d_rhs, rhs, sizeof(double) * h->S.n, cudaMemcpyDeviceToDevice,
                        h->stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, h->stream);
  if (e != cudaSuccess) return e;
  const unsigned nb = (unsigned)((h->S.n + kThreads - 1) / kThreads);
  solve_finish_kernel<<<nb, kThreads, 0, h->stream>>>(h->S.n, h->d_perm, h->d_xf, out, acc);
  return cudaGetLastError();
}

// <a, b> with a fixed reduction order (per-block partial sums, summed on the host)
cudaError_t dot(nla3d_ldlt* h, const double* a, const double* b, double* out) {
  double part[kDotBlocks];
  dot_kernel<<<kDotBlocks, kThreads, 0, h->stream>>>(h->S.n, a, b, h->d_dot);
  cudaError_t e = cudaMemcpyAsync(part, h->d_dot, sizeof(part), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  double acc = 0.0;
  for (int q = 0; q < kDotBlocks; q++) acc += part[q];
  *out = acc;
  return e;
}

// ||b - A x|| and ||b|| (the residual kernel leaves b - A x in d_r)
cudaError_t residual_norms(nla3d_ldlt* h, const double* values, const double* x, const double* b,
                           double* rnorm, double* bnorm) {
  const int64_t nblk = (h->S.n + 7) / 8;
  std::vector<double> part(2 * nblk);
  cudaError_t e = enqueue_residual(h, values, x, b);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part.data(), h->d_part, sizeof(double) * 2 * nblk, cudaMemcpyDeviceToHost,
                        h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  double rr = 0.0, bb = 0.0;
  for (int64_t q = 0; q < nblk; q++) {
    rr += part[2 * q];
    bb += part[2 * q + 1];
  }
  *rnorm = std::sqrt(rr);
  *bnorm = std::sqrt(bb);
  return e;
}

// Right-preconditioned restarted GMRES with the factor as the preconditioner
// (GMRES-based iterative refinement), modified Gram-Schmidt, Givens rotations;
// x is improved in place until ||b - A x|| <= tol ||b|| or `budget`
// preconditioner applications are spent.
cudaError_t gmres_refine(nla3d_ldlt* h, const double* values, const double* b, double* x,
                         double tol, int budget, int* apps, double* rel) {
  const LdltSymbolic& S = h->S;
  const int64_t n = S.n;
  cudaStream_t st = h->stream;
  cudaError_t e = cudaSuccess;
  if (!h->d_V) {
    e = dalloc(h, &h->d_V, (size_t)(kRestart + 1) * n);
    if (e != cudaSuccess) return e;
  }
  const unsigned vb = vec_blocks(n);
  const unsigned mb = (unsigned)((n + kThreads / 32 - 1) / (kThreads / 32));
  double rnorm = 0.0, bnorm = 0.0;
  while (true) {
    e = residual_norms(h, values, x, b, &rnorm, &bnorm);
    if (e != cudaSuccess) return e;
    const double scale = bnorm > 0.0 ? bnorm : 1.0;
    *rel = rnorm / scale;
    if (!(*rel > tol) || *apps >= budget) return cudaSuccess;
    double H[kRestart + 1][kRestart] = {};
    double cs[kRestart] = {}, sn[kRestart] = {}, g[kRestart + 1] = {};
    g[0] = rnorm;
    scale_kernel<<<vb, kThreads, 0, st>>>(n, 1.0 / rnorm, h->d_r, h->d_V);
    int j = 0;
    for (; j < kRestart && *apps < budget; j++) {
      double* vj = h->d_V + (size_t)j * n;
      double* w = h->d_V + (size_t)(j + 1) * n;
      e = enqueue_solve_any(h, vj, h->d_dx, 0);   // z = M^-1 v_j
      (*apps)++;
      if (e != cudaSuccess) return e;
      spmv_kernel<<<mb, kThreads, 0, st>>>(n, h->d_fptr, h->d_fcol, h->d_fslot, values, h->d_dx, w);
      for (int i = 0; i <= j; i++) {
        double hij = 0.0;
        e = dot(h, w, h->d_V + (size_t)i * n, &hij);
        if (e != cudaSuccess) return e;
        H[i][j] = hij;
        axpy_kernel<<<vb, kThreads, 0, st>>>(n, -hij, h->d_V + (size_t)i * n, w);
      }
      double ww = 0.0;
      e = dot(h, w, w, &ww);
      if (e != cudaSuccess) return e;
      const double hn = std::sqrt(ww);
      H[j + 1][j] = hn;
      if (hn > 0.0) scale_kernel<<<vb, kThreads, 0, st>>>(n, 1.0 / hn, w, w);
      for (int i = 0; i < j; i++) {
        const double t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
        H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
        H[i][j] = t;
      }
      const double a = H[j][j], c = H[j + 1][j];
      const double rho = std::sqrt(a * a + c * c);
      cs[j] = rho > 0.0 ? a / rho : 1.0;
      sn[j] = rho > 0.0 ? c / rho : 0.0;
      H[j][j] = rho;
      H[j + 1][j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      if (std::fabs(g[j + 1]) <= 0.5 * tol * scale || hn == 0.0) {
        j++;
        break;
      }
    }
    // y = H^-1 g, t = V y, x += M^-1 t
    double y[kRestart] = {};
    for (int i = j - 1; i >= 0; i--) {
      double acc = g[i];
      for (int q = i + 1; q < j; q++) acc -= H[i][q] * y[q];
      y[i] = H[i][i] != 0.0 ? acc / H[i][i] : 0.0;
    }
    e = cudaMemsetAsync(h->d_r, 0, sizeof(double) * n, st);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < j; i++)
      axpy_kernel<<<vb, kThreads, 0, st>>>(n, y[i], h->d_V + (size_t)i * n, h->d_r);
    e = enqueue_solve_any(h, h->d_r, x, 1);
    (*apps)++;
    if (e != cudaSuccess) return e;
  }
}

}  // namespace

extern "C" {

int nla3d_ldlt_solve(nla3d_ldlt* h, const double* values, const double* b, double* x,
                     int max_refine, double tol, int* steps, double* rel_residual) {
  if (!h || !values || !b || !x || max_refine < 0)
    return fail(h, NLA3D_ERR_ARG, "ldlt_solve: bad argument");
  if (!h->factored) return fail(h, NLA3D_ERR_ARG, "ldlt_solve: factor first");
  h->solve_accurate = 0;
  cudaError_t e = enqueue_solve_any(h, b, x, 0);
  double rel = 0.0, prev = 0.0, rnorm = 0.0, bnorm = 0.0;
  int it = 0;
  // plain refinement while it converges fast; GMRES with the same factor
  // after, its preconditioner applied with FP64 products (FP32 fronts: the
  // compensated FP32 products carry 2^-48 per operation, which a hard
  // system's Krylov iteration can feel)
  for (;;) {
    if (e == cudaSuccess) e = residual_norms(h, values, x, b, &rnorm, &bnorm);
    if (e != cudaSuccess) return cuda_fail(h, e, "ldlt_solve");
    rel = rnorm / (bnorm > 0.0 ? bnorm : 1.0);
    if (!(rel > tol) || it >= max_refine) break;
    if (it > 0 && !(rel < 0.1 * prev)) {
      h->solve_accurate = 1;
      e = gmres_refine(h, values, b, x, tol, max_refine, &it, &rel);
      if (e != cudaSuccess) return cuda_fail(h, e, "ldlt_solve (GMRES)");
      break;
    }
    prev = rel;
    e = enqueue_solve_any(h, h->d_r, x, 1);   // x += A^-1 r with the same factors
    it++;
  }
  if (steps) *steps = it;
  if (rel_residual) *rel_residual = rel;
  if (!(rel <= tol)) return fail(h, NLA3D_ERR_RANGE, "ldlt_solve: refinement did not reach tol");
  return NLA3D_OK;
}

int nla3d_ldlt_solve_host(nla3d_ldlt* h, const double* values, const double* b_host,
                          double* x_host, int max_refine, double tol, int* steps,
                          double* rel_residual) {
  if (!h || !values || !b_host || !x_host) return fail(h, NLA3D_ERR_ARG, "ldlt_solve_host: bad argument");
  const size_t n = (size_t)h->S.n;
  cudaError_t e = cudaSuccess;
  if (!h->d_hb) e = dalloc(h, &h->d_hb, n);
  if (e == cudaSuccess && !h->d_hx) e = dalloc(h, &h->d_hx, n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->d_hb, b_host, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "ldlt_solve_host");
  const int rc = nla3d_ldlt_solve(h, values, h->d_hb, h->d_hx, max_refine, tol, steps, rel_residual);
  if (rc != NLA3D_OK && rc != NLA3D_ERR_RANGE) return rc;
  // the refined x also when tol was not reached (the caller reads the residual)
  e = cudaMemcpyAsync(x_host, h->d_hx, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "ldlt_solve_host");
  return rc;
}

int nla3d_ldlt_tc_check(int m, double* out) {
  // one front of m rows whose first kb pivots (one outer block: 256 when
  // m > 512, else 64) are done: the update of rows / columns kb .. m-1 by the
  // FMA kernel and by the tensor cores (operands packed, then bulk-copied by
  // the persistent kernel) from the same random data; out[0] = max
  // |difference|, out[1] = max |update|
  if (m < kPanel + 1 || m > 4096 || !out) return NLA3D_ERR_ARG;
  const int kb = m > 2 * kOuter ? kOuter : kPanel;
  const size_t mm = (size_t)m * m, mw = (size_t)m * kb;
  std::vector<float> F0(mm), W(mw);
  uint64_t x = 88172645463325252ull;   // xorshift, fixed seed
  auto rnd = [&]() {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return (float)((double)(x >> 11) / 9007199254740992.0 * 2.0 - 1.0);
  };
  for (auto& v : F0) v = rnd();
  for (auto& v : W) v = rnd();
  std::vector<void*> allocs;
  auto dal = [&](void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) allocs.push_back(*p);
    return e;
  };
  float *F1 = nullptr, *F3 = nullptr, *dW = nullptr, *dP = nullptr;
  const size_t mp = (size_t)((m + kTcM - 1) / kTcM) * kPkBlock;
  std::vector<OuterTile> tl;   // the outer update's tiles, as the factorisation lists them
  const int rbk = (m - kb + kTcM - 1) / kTcM;
  for (int ti = 0; ti < rbk; ti++)
    for (int tj = 0; tj <= ti; tj++) tl.push_back(OuterTile{0u, (uint32_t)(ti << 16 | tj)});
  OuterTile* dT = nullptr;
  int n_sm = 1, dev = 0;
  int* err = nullptr;
  int32_t* list = nullptr;
  uint64_t *woff = nullptr, *foff = nullptr;
  int64_t* rowp = nullptr;
  int32_t* snf = nullptr;
  cudaError_t e = dal((void**)&F1, mm * 4);
  if (e == cudaSuccess) e = dal((void**)&F3, mm * 4);
  if (e == cudaSuccess) e = dal((void**)&dP, mp * 4);
  if (e == cudaSuccess) e = dal((void**)&dT, tl.size() * sizeof(OuterTile));
  if (e == cudaSuccess)
    e = cudaMemcpy(dT, tl.data(), tl.size() * sizeof(OuterTile), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = dal((void**)&dW, mw * 4);
  if (e == cudaSuccess) e = dal((void**)&err, 4);
  if (e == cudaSuccess) e = dal((void**)&list, 4);
  if (e == cudaSuccess) e = dal((void**)&woff, 8);
  if (e == cudaSuccess) e = dal((void**)&foff, 16);
  if (e == cudaSuccess) e = dal((void**)&rowp, 16);
  if (e == cudaSuccess) e = dal((void**)&snf, 8);
  const int32_t zero32 = 0;
  const uint64_t zero64[2] = {0, (uint64_t)mm};
  const int64_t rp[2] = {0, m};
  const int32_t sf[2] = {0, kb};
  if (e == cudaSuccess) e = cudaMemcpy(F1, F0.data(), mm * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(F3, F0.data(), mm * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dW, W.data(), mw * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(err, 0, 4);
  if (e == cudaSuccess) e = cudaMemcpy(list, &zero32, 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(woff, zero64, 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(foff, zero64, 16, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(rowp, rp, 16, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(snf, sf, 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(tc_packed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kPkSmem);
  int tc_err = 0;
  if (e == cudaSuccess) {
    LdltDev d{};
    d.front_off = foff;
    d.row_ptr = rowp;
    d.sn_first = snf;
    const BigBatch bb{list, woff, woff, woff};
    const int64_t rest = m - kb;
    const unsigned t128 = (unsigned)((rest + 127) / 128);
    batched_trailing_kernel<float, 128, 8><<<dim3(t128, t128, 1), kThreads>>>(bb, d, F1, 0, 1,
                                                                               dW);
    pack_update_kernel<<<dim3(t128, kPkChunks, 1), kTcThreads>>>(bb, d, F3, 0, 1, dW, dP);
    tc_packed_kernel<<<(unsigned)std::min<int>((int)tl.size(), n_sm), kOuterThreads, kPkSmem>>>(
        bb, d, F3, 0, 1, dP, dT, (int)tl.size(), err);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&tc_err, err, 4, cudaMemcpyDeviceToHost);
  }
  std::vector<float> R1(mm), R3(mm);
  if (e == cudaSuccess) e = cudaMemcpy(R1.data(), F1, mm * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(R3.data(), F3, mm * 4, cudaMemcpyDeviceToHost);
  for (void* p : allocs) cudaFree(p);
  if (e != cudaSuccess) return NLA3D_ERR_CUDA;
  if (tc_err) return NLA3D_ERR_RANGE;
  double dmax = 0.0, umax = 0.0;
  for (int j = kb; j < m; j++)
    for (int i = j; i < m; i++) {
      const size_t q = (size_t)i + (size_t)j * m;
      dmax = std::max(dmax, (double)std::fabs(R1[q] - R3[q]));
      umax = std::max(umax, (double)std::fabs(R1[q] - F0[q]));
    }
  out[0] = dmax;
  out[1] = umax;
  return NLA3D_OK;
}

int nla3d_ldlt_destroy(nla3d_ldlt* h) {
  if (!h) return NLA3D_OK;
  // a borrowed stream may already be gone: only an owned one is synchronised
  // (cudaFree waits for the device anyway)
  if (h->own_stream && h->stream) cudaStreamSynchronize(h->stream);
  if (h->factor_exec) cudaGraphExecDestroy(h->factor_exec);
  if (h->solve_exec) cudaGraphExecDestroy(h->solve_exec);
  if (h->solve_exec_acc) cudaGraphExecDestroy(h->solve_exec_acc);
  for (void* p : h->allocs) cudaFree(p);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  cudaGetLastError();   // leave no error of this teardown to the next caller
  return NLA3D_OK;
}

}  // extern "C"
