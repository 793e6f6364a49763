// The CSR pattern of K, the element -> slot maps and the fixed-order gather
// lists of one mesh, built on the device: the same arrays as the host builder
// (build_host_pattern: FEStorage::learnTopology + the sparsity part of
// initSolutionData, FEStorage.cpp:434-589 and SparseMatrix.cpp:44-154), for
// meshes whose one-time set-up would otherwise take seconds on the host.
//
//   incidence   node -> elements by counting, an exclusive scan and a sort of
//               each node's (short) list: elements ascending, as learnTopology
//   rows        one warp per node or element: the equation numbers of every
//               DoF of every incident element (and the element's own) are
//               collected in shared memory, bitonic-sorted and made unique;
//               each DoF row takes the columns >= its equation, then its MPC
//               equations, routed to block(1) / block(1,2) / block(2); a
//               counting pass, row pointers on the host, a filling pass
//   slot maps   one thread per element contribution: binary search of the
//               column in its row (SparsityInfo::getIndex)
//   gather      the slot maps inverted by counting, a scan and a per-slot
//               sort, so every slot sums in ascending contribution order
// Limits (the caller falls back to the host builder): 1024 candidate columns
// per row entity, 32-bit counts.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "host_model.hpp"
#include "pattern_gpu.hpp"

namespace nla3d_gpu {

namespace {

constexpr int kCand = 1024;        // candidate columns per row entity
constexpr int kWarpsPerBlock = 8;
constexpr uint32_t kPad = 0xFFFFFFFFu;

enum : uint32_t { kErrCandidates = 1u, kErrNoSlot = 2u };

__global__ void inc_count_kernel(uint32_t E, int npe, const uint32_t* conn, uint32_t* cnt) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const uint32_t* c = conn + (uint64_t)e * npe;
  for (int a = 0; a < npe; a++) {
    bool dup = false;
    for (int b = 0; b < a; b++) dup |= c[b] == c[a];
    if (!dup) atomicAdd(&cnt[c[a] - 1], 1u);
  }
}

__global__ void inc_fill_kernel(uint32_t E, int npe, const uint32_t* conn, uint32_t* pos,
                                uint32_t* inc_el) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const uint32_t* c = conn + (uint64_t)e * npe;
  for (int a = 0; a < npe; a++) {
    bool dup = false;
    for (int b = 0; b < a; b++) dup |= c[b] == c[a];
    if (!dup) inc_el[atomicAdd(&pos[c[a] - 1], 1u)] = e + 1;
  }
}

// per segment [ptr[i], ptr[i+1]): insertion sort (segments are short)
__global__ void sort_segments_kernel(uint64_t n, const uint32_t* ptr, uint32_t* v) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t b = ptr[i], e = ptr[i + 1];
  for (uint32_t k = b + 1; k < e; k++) {
    const uint32_t x = v[k];
    uint32_t j = k;
    while (j > b && v[j - 1] > x) {
      v[j] = v[j - 1];
      j--;
    }
    v[j] = x;
  }
}

// exclusive scan, pass 1: per-block sums of 1024 values
__global__ void block_sums_kernel(const uint32_t* in, uint64_t n, unsigned long long* sums) {
  __shared__ unsigned long long part[32];
  const uint64_t i = (uint64_t)blockIdx.x * 1024 + threadIdx.x;
  unsigned long long v = i < n ? in[i] : 0ull;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long w = part[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xFFFFFFFFu, w, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = w;
  }
}

// exclusive scan, pass 2: out[i] = offset[block] + the block's exclusive prefix
__global__ void block_scan_kernel(const uint32_t* in, uint64_t n,
                                  const unsigned long long* offsets, uint32_t* out) {
  __shared__ unsigned long long part[32];
  const uint64_t i = (uint64_t)blockIdx.x * 1024 + threadIdx.x;
  const unsigned long long v = i < n ? in[i] : 0ull;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = v;  // inclusive scan within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) part[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = part[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    part[lane] = w;
  }
  __syncthreads();
  const unsigned long long before = (warp ? part[warp - 1] : 0ull) + x - v;
  if (i < n) out[i] = (uint32_t)(offsets[blockIdx.x] + before);
}

struct RowsArgs {
  uint32_t N, E;
  int npe;
  const uint32_t* conn;
  const uint8_t* node_mask;
  const uint8_t* elem_mask;
  const uint32_t* node_eq;   // N * kDofTypes
  const uint32_t* elem_eq;   // E * kDofTypes
  const uint32_t* inc_ptr;   // N + 1
  const uint32_t* inc_el;
  const uint32_t* mpc_ptr;   // N * kDofTypes + 1, or null
  const uint32_t* mpc_eqs;
  uint32_t nc;
  uint32_t* cnt_lo;          // count pass: per equation row r (index r)
  uint32_t* cnt_hi;
  const uint32_t* io[3];     // fill pass: iofeir of the three blocks (1-based)
  uint32_t* col[3];
  uint32_t* err;
};

// lower bound of x in the sorted c[0..n)
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* c, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (c[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <bool kFill>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) rows_kernel(const RowsArgs a) {
  __shared__ uint32_t s_cand[kWarpsPerBlock][kCand];
  __shared__ uint32_t s_n[kWarpsPerBlock];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint64_t w = (uint64_t)blockIdx.x * kWarpsPerBlock + wib;
  if (w >= (uint64_t)a.N + a.E) return;  // warp-uniform
  const bool is_node = w < a.N;
  const uint32_t id = is_node ? (uint32_t)w : (uint32_t)(w - a.N);  // 0-based
  const uint8_t own_mask = is_node ? a.node_mask[id] : a.elem_mask[id];
  if (!own_mask) return;
  uint32_t* c = s_cand[wib];
  if (lane == 0) s_n[wib] = 0;
  __syncwarp();
  // (element, entity) pairs: entity 0 = the element's own DoFs, 1..npe its nodes
  const uint32_t k0 = is_node ? a.inc_ptr[id] : 0u;
  const uint32_t k1 = is_node ? a.inc_ptr[id + 1] : 1u;
  const uint32_t pairs = (k1 - k0) * (uint32_t)(a.npe + 1);
  for (uint32_t q = lane; q < pairs; q += 32) {
    const uint32_t el = is_node ? a.inc_el[k0 + q / (a.npe + 1)] - 1 : id;  // 0-based
    const int j = (int)(q % (a.npe + 1));
    uint8_t mask;
    const uint32_t* eqs;
    if (j == 0) {
      mask = a.elem_mask[el];
      eqs = a.elem_eq + (uint64_t)el * kDofTypes;
    } else {
      const uint32_t n2 = a.conn[(uint64_t)el * a.npe + (j - 1)] - 1;
      mask = a.node_mask[n2];
      eqs = a.node_eq + (uint64_t)n2 * kDofTypes;
    }
    for (int t = 0; t < kDofTypes; t++)
      if (mask & (1u << t)) {
        const uint32_t at = atomicAdd(&s_n[wib], 1u);
        if (at < (uint32_t)kCand) c[at] = eqs[t];
      }
  }
  __syncwarp();
  const uint32_t n_c = s_n[wib];
  if (n_c > (uint32_t)kCand) {
    if (lane == 0) atomicOr(a.err, kErrCandidates);
    return;
  }
  // bitonic sort of the candidates padded to a power of two (>= 32)
  uint32_t P = 32;
  while (P < n_c) P <<= 1;
  for (uint32_t i = n_c + lane; i < P; i += 32) c[i] = kPad;
  __syncwarp();
  for (uint32_t k = 2; k <= P; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = lane; i < P; i += 32) {
        const uint32_t ixj = i ^ j;
        if (ixj > i) {
          const uint32_t x = c[i], y = c[ixj];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            c[i] = y;
            c[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
  // unique, in place (the kept values only move left)
  uint32_t n_u = 0, carry = kPad;
  for (uint32_t base = 0; base < n_c; base += 32) {
    const uint32_t i = base + lane;
    const uint32_t v = i < n_c ? c[i] : kPad;
    uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, v, 1);
    if (lane == 0) prev = carry;
    const bool keep = i < n_c && v != prev;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
    const uint32_t rank = __popc(m & ((1u << lane) - 1u));
    carry = __shfl_sync(0xFFFFFFFFu, v, 31);
    __syncwarp();
    if (keep) c[n_u + rank] = v;
    n_u += __popc(m);
    __syncwarp();
  }
  // one row per DoF of the entity
  for (int t = 0; t < kDofTypes; t++) {
    if (!(own_mask & (1u << t))) continue;
    const uint32_t r = is_node ? a.node_eq[(uint64_t)id * kDofTypes + t]
                               : a.elem_eq[(uint64_t)id * kDofTypes + t];
    const uint32_t p0 = lower_bound_u32(c, n_u, r);
    // MPC equations of this DoF (all larger than every DoF equation), unique
    uint32_t x0 = 0, x1 = 0;
    if (is_node && a.mpc_ptr) {
      const uint64_t key = (uint64_t)id * kDofTypes + t;
      x0 = a.mpc_ptr[key];
      x1 = a.mpc_ptr[key + 1];
    }
    const bool upper_rows = r > a.nc;  // row in block(2)
    const uint32_t q = upper_rows ? p0 : lower_bound_u32(c, n_u, a.nc + 1);
    const uint32_t qq = q < p0 ? p0 : q;   // first candidate column > nc, at or after p0
    uint32_t n_x = 0;
    for (uint32_t k = x0; k < x1; k++)
      if (k == x0 || a.mpc_eqs[k] != a.mpc_eqs[k - 1]) n_x++;
    const uint32_t n_lo = upper_rows ? (n_u - p0) + n_x : qq - p0;
    const uint32_t n_hi = upper_rows ? 0u : (n_u - qq) + n_x;
    if (!kFill) {
      if (lane == 0) {
        a.cnt_lo[r] = n_lo;
        a.cnt_hi[r] = n_hi;
      }
      continue;
    }
    // fill: block b of row `row` starts at io[b][row - 1] - 1
    if (upper_rows) {
      uint32_t* out = a.col[2] + (a.io[2][r - a.nc - 1] - 1);
      for (uint32_t i = p0 + lane; i < n_u; i += 32) out[i - p0] = c[i] - a.nc;
      if (lane == 0) {
        uint32_t o = n_u - p0;
        for (uint32_t k = x0; k < x1; k++)
          if (k == x0 || a.mpc_eqs[k] != a.mpc_eqs[k - 1]) out[o++] = a.mpc_eqs[k] - a.nc;
      }
    } else {
      uint32_t* lo = a.col[0] + (a.io[0][r - 1] - 1);
      uint32_t* hi = a.col[1] + (a.io[1][r - 1] - 1);
      for (uint32_t i = p0 + lane; i < qq; i += 32) lo[i - p0] = c[i];
      for (uint32_t i = qq + lane; i < n_u; i += 32) hi[i - qq] = c[i] - a.nc;
      if (lane == 0) {
        uint32_t o = n_u - qq;
        for (uint32_t k = x0; k < x1; k++)
          if (k == x0 || a.mpc_eqs[k] != a.mpc_eqs[k - 1]) hi[o++] = a.mpc_eqs[k] - a.nc;
      }
    }
  }
}

struct SlotArgs {
  uint32_t E;
  int npe, n_kc, n_fc;
  const int8_t* kl;        // n_kc * 4: (ei, ti, ej, tj), entity -1 = the element
  const int8_t* fl;        // n_fc * 4: (ei, ti, -, -)
  const uint32_t* conn;
  const uint32_t* node_eq;
  const uint32_t* elem_eq;
  uint32_t nc;
  const uint32_t* io[3];
  const uint32_t* col[3];
  uint64_t val_off[3];
  uint32_t* kslot;         // E * n_kc
  uint32_t* fslot;         // E * n_fc
  uint32_t* err;
};

__device__ __forceinline__ uint32_t eq_of(const SlotArgs& a, uint32_t e, int ent, int t) {
  if (ent < 0) return a.elem_eq[(uint64_t)e * kDofTypes + t];
  return a.node_eq[(uint64_t)(a.conn[(uint64_t)e * a.npe + ent] - 1) * kDofTypes + t];
}

__global__ void slot_map_kernel(const SlotArgs a) {
  const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nk = (uint64_t)a.E * a.n_kc;
  if (x < nk) {
    const uint32_t e = (uint32_t)(x / a.n_kc);
    const int k = (int)(x % a.n_kc);
    const int8_t* L = a.kl + 4 * k;
    uint32_t i = eq_of(a, e, L[0], L[1]), j = eq_of(a, e, L[2], L[3]);
    if (i > j) {
      const uint32_t t = i;
      i = j;
      j = t;
    }
    int b;
    if (j <= a.nc) {
      b = 0;
    } else if (i <= a.nc) {
      b = 1;
      j -= a.nc;
    } else {
      b = 2;
      i -= a.nc;
      j -= a.nc;
    }
    const uint32_t beg = a.io[b][i - 1] - 1, end = a.io[b][i] - 1;
    const uint32_t p = beg + lower_bound_u32(a.col[b] + beg, end - beg, j);
    if (p < end && a.col[b][p] == j) {
      a.kslot[x] = (uint32_t)(a.val_off[b] + p);
    } else {
      a.kslot[x] = 0;
      atomicOr(a.err, kErrNoSlot);
    }
    return;
  }
  const uint64_t y = x - nk;
  if (y < (uint64_t)a.E * a.n_fc) {
    const uint32_t e = (uint32_t)(y / a.n_fc);
    const int k = (int)(y % a.n_fc);
    a.fslot[y] = eq_of(a, e, a.fl[4 * k], a.fl[4 * k + 1]) - 1;
  }
}

__global__ void count_kernel(uint64_t n, const uint32_t* slot, uint32_t* cnt) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[slot[i]], 1u);
}

__global__ void fill_kernel(uint64_t n, const uint32_t* slot, uint32_t* pos, uint32_t* ids) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ids[atomicAdd(&pos[slot[i]], 1u)] = (uint32_t)i;
}

__global__ void inverse_kernel(uint64_t n, const uint32_t* ids, uint32_t* pos) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) pos[ids[k]] = (uint32_t)k;
}

unsigned blocks_for(uint64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Device buffers freed at scope exit (the builder's temporaries).
struct Temps {
  std::vector<void*> p;
  template <class T>
  cudaError_t get(T** out, uint64_t n) {
    *out = nullptr;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
    if (e == cudaSuccess) {
      p.push_back(q);
      *out = (T*)q;
    }
    return e;
  }
  ~Temps() {
    for (void* q : p) cudaFree(q);
  }
};

// out[0..n] = exclusive prefix sums of in[0..n), out[n] = the total
cudaError_t scan(const uint32_t* in, uint64_t n, uint32_t* out, uint64_t* total, Temps& T,
                 cudaStream_t s) {
  const uint64_t nb = (n + 1023) / 1024;
  unsigned long long* d_sums = nullptr;
  cudaError_t e = T.get(&d_sums, nb);
  if (e != cudaSuccess) return e;
  std::vector<unsigned long long> h(nb);
  if (n) {
    block_sums_kernel<<<(unsigned)nb, 1024, 0, s>>>(in, n, d_sums);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = cudaMemcpyAsync(h.data(), d_sums, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
  }
  unsigned long long run = 0;
  for (uint64_t b = 0; b < nb; b++) {
    const unsigned long long v = h[b];
    h[b] = run;
    run += v;
  }
  *total = run;
  if (run > 0xFFFFFFF0ull) return cudaErrorInvalidValue;  // caller falls back
  const uint32_t tot = (uint32_t)run;
  e = cudaMemcpyAsync(out + n, &tot, sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && n)
    e = cudaMemcpyAsync(d_sums, h.data(), sizeof(unsigned long long) * nb, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  if (n) {
    block_scan_kernel<<<(unsigned)nb, 1024, 0, s>>>(in, n, d_sums, out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // `tot` and `h` leave scope
  return e;
}

template <class T>
cudaError_t up(Temps& tmp, T** d, const std::vector<T>& h, cudaStream_t s) {
  cudaError_t e = tmp.get(d, h.size());
  if (e == cudaSuccess && !h.empty())
    e = cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
  return e;
}

}  // namespace

std::string build_pattern_gpu(HostModel& m, cudaStream_t s, const DeviceAlloc& alloc,
                              PatternDevice* out) {
  const uint32_t N = m.n_nodes, E = m.n_elems, nc = m.n_con, ntot = m.n_total();
  const int npe = m.npe;
  Temps T;
  cudaError_t e = cudaSuccess;
  std::string where;
#define GCK(x, w)                                            \
  do {                                                       \
    if ((e = (x)) != cudaSuccess) {                          \
      where = (w);                                           \
      goto cuda_error;                                       \
    }                                                        \
  } while (0)
  {
    // ---- inputs ----
    uint32_t *d_conn, *d_neq, *d_eeq, *d_mptr = nullptr, *d_meqs = nullptr, *d_err;
    uint8_t *d_nmask, *d_emask;
    GCK(up(T, &d_conn, m.conn, s), "upload");
    GCK(up(T, &d_neq, m.node_eq, s), "upload");
    GCK(up(T, &d_eeq, m.elem_eq, s), "upload");
    GCK(up(T, &d_nmask, m.node_mask, s), "upload");
    GCK(up(T, &d_emask, m.elem_mask, s), "upload");
    std::vector<uint32_t> mptr, meqs;
    mpc_extras(m, mptr, meqs);
    if (!mptr.empty()) {
      GCK(up(T, &d_mptr, mptr, s), "upload");
      GCK(up(T, &d_meqs, meqs, s), "upload");
    }
    GCK(T.get(&d_err, 1), "alloc");
    GCK(cudaMemsetAsync(d_err, 0, sizeof(uint32_t), s), "memset");

    // ---- incidence ----
    uint32_t *d_cnt, *d_iptr, *d_pos, *d_iel;
    uint64_t total = 0;
    GCK(T.get(&d_cnt, N), "alloc");
    GCK(T.get(&d_iptr, (uint64_t)N + 1), "alloc");
    GCK(cudaMemsetAsync(d_cnt, 0, sizeof(uint32_t) * (N ? N : 1), s), "memset");
    if (E) inc_count_kernel<<<blocks_for(E, 256), 256, 0, s>>>(E, npe, d_conn, d_cnt);
    GCK(cudaGetLastError(), "incidence count");
    GCK(scan(d_cnt, N, d_iptr, &total, T, s), "incidence scan");
    GCK(T.get(&d_pos, N), "alloc");
    GCK(T.get(&d_iel, total), "alloc");
    GCK(cudaMemcpyAsync(d_pos, d_iptr, sizeof(uint32_t) * N, cudaMemcpyDeviceToDevice, s), "copy");
    if (E) inc_fill_kernel<<<blocks_for(E, 256), 256, 0, s>>>(E, npe, d_conn, d_pos, d_iel);
    GCK(cudaGetLastError(), "incidence fill");
    if (N) sort_segments_kernel<<<blocks_for(N, 256), 256, 0, s>>>(N, d_iptr, d_iel);
    GCK(cudaGetLastError(), "incidence sort");

    // ---- rows: count ----
    uint32_t *d_lo, *d_hi;
    GCK(T.get(&d_lo, (uint64_t)ntot + 1), "alloc");
    GCK(T.get(&d_hi, (uint64_t)ntot + 1), "alloc");
    GCK(cudaMemsetAsync(d_lo, 0, sizeof(uint32_t) * ((uint64_t)ntot + 1), s), "memset");
    GCK(cudaMemsetAsync(d_hi, 0, sizeof(uint32_t) * ((uint64_t)ntot + 1), s), "memset");
    RowsArgs ra{};
    ra.N = N;
    ra.E = E;
    ra.npe = npe;
    ra.conn = d_conn;
    ra.node_mask = d_nmask;
    ra.elem_mask = d_emask;
    ra.node_eq = d_neq;
    ra.elem_eq = d_eeq;
    ra.inc_ptr = d_iptr;
    ra.inc_el = d_iel;
    ra.mpc_ptr = d_mptr;
    ra.mpc_eqs = d_meqs;
    ra.nc = nc;
    ra.cnt_lo = d_lo;
    ra.cnt_hi = d_hi;
    ra.err = d_err;
    const unsigned row_blocks = blocks_for((uint64_t)N + E, kWarpsPerBlock);
    rows_kernel<false><<<row_blocks, kWarpsPerBlock * 32, 0, s>>>(ra);
    GCK(cudaGetLastError(), "rows count");
    std::vector<uint32_t> lo(ntot + 1), hi(ntot + 1);
    uint32_t herr = 0;
    GCK(cudaMemcpyAsync(lo.data(), d_lo, sizeof(uint32_t) * lo.size(), cudaMemcpyDeviceToHost, s), "copy");
    GCK(cudaMemcpyAsync(hi.data(), d_hi, sizeof(uint32_t) * hi.size(), cudaMemcpyDeviceToHost, s), "copy");
    GCK(cudaMemcpyAsync(&herr, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "copy");
    GCK(cudaStreamSynchronize(s), "sync");
    if (herr & kErrCandidates) return "fallback: a row entity has more than 1024 candidate columns";
    // row pointers, as the host builder forms them
    const uint32_t ns = m.n_unk + m.n_mpc;
    m.blk[0].rows = nc; m.blk[0].cols = nc;
    m.blk[1].rows = nc; m.blk[1].cols = ns;
    m.blk[2].rows = ns; m.blk[2].cols = ns;
    for (int b = 0; b < 3; b++) m.blk[b].iofeir.assign(m.blk[b].rows + 1, 1);
    uint64_t s0 = 0, s1 = 0, s2 = 0;
    for (uint32_t r = 1; r <= ntot; r++) {
      if (r <= nc) {
        s0 += lo[r];
        s1 += hi[r];
        m.blk[0].iofeir[r] = (uint32_t)(s0 + 1);
        m.blk[1].iofeir[r] = (uint32_t)(s1 + 1);
      } else {
        s2 += lo[r];
        m.blk[2].iofeir[r - nc] = (uint32_t)(s2 + 1);
      }
      if (s0 + s1 + s2 >= 0xFFFFFFF0ull) return "fallback: K has more than 2^32 nonzeros";
    }
    std::vector<uint32_t>().swap(lo);
    std::vector<uint32_t>().swap(hi);
    m.val_off[0] = 0;
    m.val_off[1] = s0;
    m.val_off[2] = s0 + s1;
    m.nnz_total = s0 + s1 + s2;

    // ---- rows: fill ----
    uint32_t* d_io[3];
    uint32_t* d_col[3];
    for (int b = 0; b < 3; b++) {
      GCK(up(T, &d_io[b], m.blk[b].iofeir, s), "upload");
      GCK(T.get(&d_col[b], (uint64_t)m.blk[b].iofeir.back() - 1), "alloc");
      ra.io[b] = d_io[b];
      ra.col[b] = d_col[b];
    }
    rows_kernel<true><<<row_blocks, kWarpsPerBlock * 32, 0, s>>>(ra);
    GCK(cudaGetLastError(), "rows fill");
    for (int b = 0; b < 3; b++) {
      const uint64_t nnz = (uint64_t)m.blk[b].iofeir.back() - 1;
      m.blk[b].columns.resize(nnz);
      if (nnz)
        GCK(cudaMemcpyAsync(m.blk[b].columns.data(), d_col[b], sizeof(uint32_t) * nnz,
                            cudaMemcpyDeviceToHost, s), "copy");
    }

    // ---- element -> slot maps ----
    const std::vector<LocalPair> KL = element_k_layout(m.etype);
    const std::vector<LocalPair> FL = element_f_layout(m.etype);
    m.n_kc = (int)KL.size();
    m.n_fc = (int)FL.size();
    const uint64_t nk = (uint64_t)E * m.n_kc, nf = (uint64_t)E * m.n_fc;
    if (nk + nf >= 0xFFFFFFF0ull) return "fallback: too many element contributions";
    std::vector<int8_t> kl(4 * KL.size()), fl(4 * (FL.size() ? FL.size() : 1), 0);
    for (size_t k = 0; k < KL.size(); k++) std::memcpy(&kl[4 * k], &KL[k], 4);
    for (size_t k = 0; k < FL.size(); k++) std::memcpy(&fl[4 * k], &FL[k], 4);
    int8_t *d_kl, *d_fl;
    uint32_t *d_kslot, *d_fslot;
    GCK(up(T, &d_kl, kl, s), "upload");
    GCK(up(T, &d_fl, fl, s), "upload");
    GCK(T.get(&d_kslot, nk), "alloc");
    GCK(T.get(&d_fslot, nf), "alloc");
    SlotArgs sa{};
    sa.E = E;
    sa.npe = npe;
    sa.n_kc = m.n_kc;
    sa.n_fc = m.n_fc;
    sa.kl = d_kl;
    sa.fl = d_fl;
    sa.conn = d_conn;
    sa.node_eq = d_neq;
    sa.elem_eq = d_eeq;
    sa.nc = nc;
    for (int b = 0; b < 3; b++) {
      sa.io[b] = d_io[b];
      sa.col[b] = d_col[b];
      sa.val_off[b] = m.val_off[b];
    }
    sa.kslot = d_kslot;
    sa.fslot = d_fslot;
    sa.err = d_err;
    if (nk + nf) slot_map_kernel<<<blocks_for(nk + nf, 256), 256, 0, s>>>(sa);
    GCK(cudaGetLastError(), "slot maps");
    GCK(cudaMemcpyAsync(&herr, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "copy");
    GCK(cudaStreamSynchronize(s), "sync");
    if (herr & kErrNoSlot) return "an element contribution has no slot in the CSR pattern";

    // ---- gather lists (inverse slot maps), ascending within a slot ----
    const uint64_t n_slots[2] = {m.nnz_total, ntot};
    const uint64_t n_c[2] = {nk, nf};
    uint32_t* slot_of[2] = {d_kslot, d_fslot};
    uint32_t** outp[2][3] = {{&out->k_ptr, &out->k_ids, &out->k_pos},
                             {&out->f_ptr, &out->f_ids, &out->f_pos}};
    for (int w = 0; w < 2; w++) {
      uint32_t *d_c, *d_ptr, *d_ids, *d_ipos, *d_p2;
      GCK(T.get(&d_c, n_slots[w]), "alloc");
      GCK(cudaMemsetAsync(d_c, 0, sizeof(uint32_t) * (n_slots[w] ? n_slots[w] : 1), s), "memset");
      if (n_c[w]) count_kernel<<<blocks_for(n_c[w], 256), 256, 0, s>>>(n_c[w], slot_of[w], d_c);
      GCK(cudaGetLastError(), "gather count");
      GCK(alloc((void**)&d_ptr, sizeof(uint32_t) * (n_slots[w] + 1)), "alloc");
      GCK(scan(d_c, n_slots[w], d_ptr, &total, T, s), "gather scan");
      GCK(T.get(&d_p2, n_slots[w]), "alloc");
      GCK(cudaMemcpyAsync(d_p2, d_ptr, sizeof(uint32_t) * n_slots[w], cudaMemcpyDeviceToDevice, s), "copy");
      GCK(alloc((void**)&d_ids, sizeof(uint32_t) * (n_c[w] ? n_c[w] : 1)), "alloc");
      if (n_c[w]) fill_kernel<<<blocks_for(n_c[w], 256), 256, 0, s>>>(n_c[w], slot_of[w], d_p2, d_ids);
      GCK(cudaGetLastError(), "gather fill");
      if (n_slots[w])
        sort_segments_kernel<<<blocks_for(n_slots[w], 256), 256, 0, s>>>(n_slots[w], d_ptr, d_ids);
      GCK(cudaGetLastError(), "gather sort");
      GCK(alloc((void**)&d_ipos, sizeof(uint32_t) * (n_c[w] ? n_c[w] : 1)), "alloc");
      if (n_c[w]) inverse_kernel<<<blocks_for(n_c[w], 256), 256, 0, s>>>(n_c[w], d_ids, d_ipos);
      GCK(cudaGetLastError(), "gather inverse");
      *outp[w][0] = d_ptr;
      *outp[w][1] = d_ids;
      *outp[w][2] = d_ipos;
    }
    GCK(cudaStreamSynchronize(s), "sync");
  }
#undef GCK
  return host_mpc_slots(m);
cuda_error:
  return std::string("device pattern build: ") + where + ": " + cudaGetErrorString(e);
}

}  // namespace nla3d_gpu
