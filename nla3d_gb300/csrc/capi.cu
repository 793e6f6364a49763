// C ABI of the assembly path (include/nla3d_gpu.h): context, device memory
// layout and the launch sequence of one assembly.
//
// A context holds one mesh (nla3d_create) or a batch of independent meshes
// (nla3d_create_batch).  The meshes keep their own equation numbering, CSR
// pattern, K and F (each is one reference FEStorage); on the device they are
// concatenated so that one launch of each kernel assembles all of them:
//
//   Gt      24 x 8E  double  dN/dX per Gauss point, structure of arrays
//   wdet    8E       double  Gauss weight * det J
//   conn    8E       uint32  node ids, global (mesh node offset added)
//   node_eq 4N       uint32  equations of UX, UY, UZ (+ pad), global 1-based
//   p_eq    E        uint32  pressure equation per element, global 1-based
//   U, U_state       double  concatenated vecU / snapshot at updateResults()
//   contribK 325E, contribF 25E  double   element contributions, reference order
//   k_ptr nnz+1      uint32  start of each K slot's contributions in slot order
//   k_ids 325E       uint32  slot order -> element contribution id e*325+c
//                            (ascending within a slot: element order, then the
//                            reference's local order)
//   k_pos 325E       uint32  the inverse map (element contribution -> slot order)
//   f_ptr n+1, f_ids, f_pos 25E   same for F
// Two contribution layouts (nla3d_set_contrib_layout / nla3d_autotune):
//   0  element order: contribK[e*325+c]; K[s] gathers contribK[k_ids[k]]
//   1  slot order: the element kernel writes contribK[k_pos[e*325+c]]; K[s]
//      sums the contiguous contribK[k_ptr[s] .. k_ptr[s+1])
// Both sum each slot in the same order, so K is bitwise the same.
//   K (per mesh: block(1) | block(1,2) | block(2)), F   double
//   elem_mesh E, mesh_mat 8M  per-element material (only when meshes differ)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nla3d_gpu.h"
#include "host_model.hpp"
#include "kernels.cuh"
#include "pattern_gpu.hpp"

using namespace nla3d_gpu;

struct nla3d_ctx {
  std::vector<HostModel> hm;  // one per mesh
  int precision = NLA3D_PREC_FP64;
  std::string err;
  bool host_ready = false;  // nla3d_build_pattern done
  bool ready = false;       // nla3d_init_solution_data done
  int device = -1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool have_state = false;
  uint64_t launches = 0;
  // per-mesh offsets into the concatenated device arrays (n_meshes + 1 each)
  std::vector<uint64_t> elem_off, node_off, u_off, k_off, mpc_off;
  bool uniform_material = true;
  // device buffers
  double* d_xyz = nullptr;
  uint32_t* d_conn = nullptr;
  uint32_t* d_node_eq3 = nullptr;
  uint32_t* d_p_eq = nullptr;
  double* d_eparams = nullptr;
  double* d_Gt = nullptr;
  double* d_wdet = nullptr;
  double* d_U = nullptr;
  double* d_Ustate = nullptr;
  double* d_contribK = nullptr;
  double* d_contribF = nullptr;
  uint32_t* d_kptr = nullptr;
  uint32_t* d_kids = nullptr;
  uint32_t* d_kpos = nullptr;
  uint32_t* d_fptr = nullptr;
  uint32_t* d_fids = nullptr;
  uint32_t* d_fpos = nullptr;
  int layout = 0;
  double* d_K = nullptr;
  double* d_F = nullptr;
  uint32_t* d_elem_mesh = nullptr;
  double* d_mesh_mat = nullptr;
  // mixed precision: dN/dX, w det J and the materials as float pairs
  float2* d_Gdf = nullptr;
  float2* d_wdf = nullptr;
  float2* d_mesh_mat_df = nullptr;
  uint32_t* d_mpc_u32 = nullptr;  // master, slave, eq, slave_eq, master_eq6 (6), slot (5)
  int32_t* d_mpc_dof = nullptr;
  // SurfaceLINETH lines (single-mesh QUADTH contexts) and transient C / M
  uint32_t n_lines = 0;
  uint32_t* d_line_conn = nullptr;
  double* d_line_par = nullptr;
  bool transient = false;
  double* d_contribC = nullptr;
  double* d_C = nullptr;
  double* d_M = nullptr;
  // linear MPC equations of all meshes: eq, ptr (n + 1), slot (terms); b, coef
  uint64_t n_lmpc = 0;
  uint32_t* d_lmpc_eq = nullptr;
  uint32_t* d_lmpc_ptr = nullptr;
  uint32_t* d_lmpc_slot = nullptr;
  double* d_lmpc_b = nullptr;
  double* d_lmpc_coef = nullptr;
  ElementStatus* d_status = nullptr;
  std::vector<void*> allocs;
  // pattern builder: 0 host, 1 device, -1 device for single meshes of at
  // least kDevicePatternElems elements; device_pattern: the gather lists were
  // built on the device (pd)
  int pattern_mode = -1;
  bool device_pattern = false;
  PatternDevice pd;
  // walk lists of the sparse block products, built on first use:
  // per mesh, (block 1) (block 2) (block 1,2) (block 1,2 transposed)
  struct MvList {
    bool built = false;
    uint64_t n_out = 0, n_entries = 0;
    uint32_t* ptr = nullptr;
    uint32_t* slot = nullptr;
    uint32_t* xi = nullptr;
  };
  std::vector<std::vector<MvList>> mv;
  // nla3d_assemble_to_host: element ranges, and the runs of K slots summed
  // and copied after each range (range index, first slot, end slot)
  struct SlotRun {
    int k;
    uint64_t s0, s1;
  };
  // copy streams: each run of K is copied in kCopyStreams parts, one per
  // copy engine (one engine alone does not fill the host link)
  static constexpr int kCopyStreams = 2;
  cudaStream_t copy_stream[kCopyStreams] = {};
  std::vector<cudaEvent_t> chunk_ev;
  int plan_chunks = 0;
  std::vector<uint32_t> plan_eb;
  std::vector<SlotRun> plan_runs;
  // launch shape (nla3d_autotune / nla3d_set_launch_shape)
  Solid81Shape shape;
  int gather_bs = 256;
  // CUDA graph of update_results + assemble
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  // per-kernel timing ring
  bool timing = false;
  static constexpr int kRing = 256;
  std::vector<cudaEvent_t> ev;  // kRing x 5
  uint64_t timed = 0;           // assemblies recorded since the last read

  uint64_t E() const { return elem_off.empty() ? 0 : elem_off.back(); }
  uint64_t Ntot() const { return node_off.empty() ? 0 : node_off.back(); }
  uint64_t Utot() const { return u_off.empty() ? 0 : u_off.back(); }
  uint64_t Ktot() const { return k_off.empty() ? 0 : k_off.back(); }
  uint64_t Mtot() const { return mpc_off.empty() ? 0 : mpc_off.back(); }
};

namespace {

int fail(nla3d_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(nla3d_ctx* c, cudaError_t e, const char* where) {
  return fail(c, NLA3D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <class T>
cudaError_t dalloc(nla3d_ctx* c, T** p, uint64_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
  if (e == cudaSuccess) c->allocs.push_back(*p);
  return e;
}

template <class T>
cudaError_t upload(nla3d_ctx* c, T** p, const T* host, uint64_t n) {
  cudaError_t e = dalloc(c, p, n);
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpyAsync(*p, host, sizeof(T) * n, cudaMemcpyHostToDevice, c->stream);
}

// hi + lo = v to 2^-48: the mixed kernel's float-pair form of a double
float2 split_pair(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

int block_slot(int block) { return block == 1 ? 0 : (block == 2 ? 2 : (block == 12 ? 1 : -1)); }

// Walk lists of y += coef * op(B) x in the reference's order (SparseMatrix.cpp:497-558):
//   kind 0/1 (symmetric block 1/2, matBVprod(SparseSymMatrix&)): output row i
//     visits B(j,i) for j <= i ascending (column i of the stored upper
//     triangle, diagonal last), then B(i,j) for j > i ascending;
//   kind 2 (block 1,2, matBVprod(SparseMatrix&)): row i's entries in order;
//   kind 3 (block 1,2, matBTVprod): output column j visits rows i ascending.
// slot = value index within the block, xi = 0-based index into x.
void build_walk(const CsrBlock& b, int kind, std::vector<uint32_t>& ptr,
                std::vector<uint32_t>& slot, std::vector<uint32_t>& xi) {
  const bool sym = kind <= 1, trans = kind == 3;
  const uint32_t n_out = trans ? b.cols : b.rows;
  std::vector<uint32_t> cnt(n_out, 0);
  for (uint32_t r = 0; r < b.rows; r++)
    for (uint32_t k = b.iofeir[r] - 1; k < b.iofeir[r + 1] - 1; k++) {
      const uint32_t c = b.columns[k] - 1;
      if (sym) {
        cnt[c]++;
        if (c > r) cnt[r]++;
      } else {
        cnt[trans ? c : r]++;
      }
    }
  ptr.assign(n_out + 1, 0);
  for (uint32_t i = 0; i < n_out; i++) ptr[i + 1] = ptr[i] + cnt[i];
  slot.assign(ptr[n_out], 0);
  xi.assign(ptr[n_out], 0);
  std::vector<uint32_t> pos(ptr.begin(), ptr.end() - 1);
  auto put = [&](uint32_t out, uint32_t k, uint32_t x) {
    slot[pos[out]] = k;
    xi[pos[out]] = x;
    pos[out]++;
  };
  for (uint32_t r = 0; r < b.rows; r++)
    for (uint32_t k = b.iofeir[r] - 1; k < b.iofeir[r + 1] - 1; k++) {
      const uint32_t c = b.columns[k] - 1;
      if (sym) {
        // rows are visited in ascending order, so column c's lower part is
        // complete (diagonal last) before row c appends its upper part
        put(c, k, r);
        if (c > r) put(r, k, c);
      } else if (trans) {
        put(c, k, r);
      } else {
        put(r, k, c);
      }
    }
}

int check_mesh(const nla3d_mesh_desc* mesh) {
  if (!mesh || (mesh->n_elems && (!mesh->conn || !mesh->xyz))) return NLA3D_ERR_ARG;
  if (mesh->elem_type != NLA3D_SOLID81 && mesh->elem_type != NLA3D_TETRA0 &&
      mesh->elem_type != NLA3D_QUADTH && mesh->elem_type != NLA3D_PLANE41)
    return NLA3D_ERR_ARG;
  const bool hyper = mesh->elem_type == NLA3D_SOLID81 || mesh->elem_type == NLA3D_PLANE41;
  if (hyper && (mesh->mat_id < NLA3D_MAT_NEO_HOOKEAN || mesh->mat_id > NLA3D_MAT_MOONEY_RIVLIN))
    return NLA3D_ERR_ARG;
  if (!hyper && !mesh->elem_params && mesh->n_elems) return NLA3D_ERR_ARG;
  const int np = mesh->n_elem_params ? mesh->n_elem_params : 2;
  if (np != 2 && !(np == 4 && mesh->elem_type == NLA3D_QUADTH)) return NLA3D_ERR_ARG;
  return NLA3D_OK;
}

void fill_model(HostModel& m, const nla3d_mesh_desc* mesh) {
  m.etype = mesh->elem_type;
  m.npe = m.etype == NLA3D_SOLID81 ? 8 : 4;
  m.n_nodes = mesh->n_nodes;
  m.n_elems = mesh->n_elems;
  m.xyz.assign(mesh->xyz, mesh->xyz + 3 * (size_t)mesh->n_nodes);
  m.conn.assign(mesh->conn, mesh->conn + (size_t)m.npe * mesh->n_elems);
  m.mat_id = mesh->mat_id;
  for (int i = 0; i < 5; i++) m.mat_c[i] = mesh->mat_c[i];
  if (mesh->elem_params) {
    // stored kElemParams per element, missing trailing values zero
    const int np = mesh->n_elem_params ? mesh->n_elem_params : 2;
    m.eparams.assign((size_t)kElemParams * mesh->n_elems, 0.0);
    for (size_t e = 0; e < mesh->n_elems; e++)
      for (int i = 0; i < np; i++) m.eparams[kElemParams * e + i] = mesh->elem_params[np * e + i];
  }
}

double bulk_of(const HostModel& m) {
  return m.mat_id == NLA3D_MAT_NEO_HOOKEAN ? m.mat_c[1]
                                           : (m.mat_id == NLA3D_MAT_BIDERMAN ? m.mat_c[4] : m.mat_c[2]);
}

// The mixed SOLID81 kernel computes in floats and float pairs: its inputs
// must sit well inside the float exponent range.  Material constants (and
// the bulk modulus) are 0 or of magnitude 1e-20 .. 1e20; the coordinates'
// extent is 1e-6 .. 1e6.
bool mixed_range_ok(const HostModel& m) {
  auto in_range = [](double v, double lo, double hi) {
    const double a = std::fabs(v);
    return std::isfinite(v) && (a == 0.0 || (a >= lo && a <= hi));
  };
  for (int k = 0; k < 5; k++)
    if (!in_range(m.mat_c[k], 1e-20, 1e20)) return false;
  if (!in_range(bulk_of(m), 1e-20, 1e20) || bulk_of(m) == 0.0) return false;
  double ext = 0.0;
  for (int d = 0; d < 3; d++) {
    double lo = 0.0, hi = 0.0;
    for (uint64_t n = 0; n < m.n_nodes; n++) {
      const double x = m.xyz[3 * n + d];
      if (!std::isfinite(x)) return false;
      if (n == 0 || x < lo) lo = x;
      if (n == 0 || x > hi) hi = x;
    }
    ext = std::max(ext, hi - lo);
  }
  return m.n_nodes == 0 || in_range(ext, 1e-6, 1e6);
}

bool valid_mesh(const nla3d_ctx* c, uint32_t mesh) { return c && mesh < c->hm.size(); }

void graph_release(nla3d_ctx* c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
}

// The kernels of one assembly (everything nla3d_assemble enqueues).
// Element kernel over the element range [e0, e1).
cudaError_t enqueue_elements(nla3d_ctx* c, uint32_t e0, uint32_t e1) {
  const HostModel& m0 = c->hm[0];
  if (e1 <= e0) return cudaSuccess;
  cudaError_t e;
  if (m0.etype == NLA3D_SOLID81) {
    Solid81Args a{};
    a.e_begin = e0;
    a.n_elems = e1;
    a.n_total = (uint32_t)c->E();
    a.Gt = c->d_Gt;
    a.wdet = c->d_wdet;
    a.conn = c->d_conn;
    a.node_eq3 = c->d_node_eq3;
    a.p_eq = c->d_p_eq;
    a.U_state = c->d_Ustate;
    a.U_cur = c->d_U;
    a.have_state = c->have_state ? 1 : 0;
    a.mat_id = m0.mat_id;
    for (int i = 0; i < 5; i++) a.mc[i] = m0.mat_c[i];
    a.kbulk = bulk_of(m0);
    a.elem_mesh = c->uniform_material ? nullptr : c->d_elem_mesh;
    a.mesh_mat = c->uniform_material ? nullptr : c->d_mesh_mat;
    a.kpos = c->layout ? c->d_kpos : nullptr;
    a.fpos = c->layout ? c->d_fpos : nullptr;
    a.contribK = c->d_contribK;
    a.contribF = c->d_contribF;
    a.status = c->d_status;
    if (c->precision == NLA3D_PREC_MIXED) {
      a.Gdf = c->d_Gdf;
      a.wdf = c->d_wdf;
      for (int i = 0; i < 5; i++) a.mcd[i] = split_pair(m0.mat_c[i]);
      a.inv_kbd = split_pair(1.0 / a.kbulk);
      a.inv_kb = 1.0 / a.kbulk;
      a.mesh_mat_df = c->uniform_material ? nullptr : c->d_mesh_mat_df;
    }
    e = launch_solid81_shaped(a, c->precision == NLA3D_PREC_MIXED, c->shape, c->stream);
  } else if (m0.etype == NLA3D_PLANE41) {
    Plane41Args a{};
    a.e_begin = e0;
    a.n_elems = e1;
    a.xyz = c->d_xyz;
    a.conn = c->d_conn;
    a.node_eq3 = c->d_node_eq3;
    a.p_eq = c->d_p_eq;
    a.U_state = c->d_Ustate;
    a.U_cur = c->d_U;
    a.have_state = c->have_state ? 1 : 0;
    a.mat_id = m0.mat_id;
    for (int i = 0; i < 5; i++) a.mc[i] = m0.mat_c[i];
    a.kbulk = bulk_of(m0);
    a.elem_mesh = c->uniform_material ? nullptr : c->d_elem_mesh;
    a.mesh_mat = c->uniform_material ? nullptr : c->d_mesh_mat;
    a.kpos = c->layout ? c->d_kpos : nullptr;
    a.fpos = c->layout ? c->d_fpos : nullptr;
    a.contribK = c->d_contribK;
    a.contribF = c->d_contribF;
    a.status = c->d_status;
    e = launch_plane41(a, c->stream);
  } else {
    LinearArgs a{m0.etype, e1, c->d_xyz, c->d_conn, c->d_eparams, c->d_contribK,
                 c->d_contribF, c->d_status, c->layout ? c->d_kpos : nullptr,
                 c->layout ? c->d_fpos : nullptr, e0, c->transient ? c->d_contribC : nullptr};
    e = launch_linear(a, c->stream);
  }
  if (e == cudaSuccess && e1 > e0) c->launches++;
  if (e == cudaSuccess && c->n_lines && e1 == (uint32_t)c->E()) {
    // the lines are created after the elements: they go with the last range
    LineArgs la{c->n_lines, c->d_xyz, c->d_line_conn, c->d_line_par,
                (uint64_t)c->E() * m0.n_kc, (uint64_t)c->E() * m0.n_fc,
                c->layout ? c->d_kpos : nullptr, c->layout ? c->d_fpos : nullptr,
                c->d_contribK, c->d_contribF, c->d_status, (uint32_t)c->E() + 1};
    e = launch_lines(la, c->stream);
    if (e == cudaSuccess) c->launches++;
  }
  return e;
}

// K values of the slot range [s0, s1) (fixed-order sums).
cudaError_t enqueue_gather_K(nla3d_ctx* c, uint64_t s0, uint64_t s1) {
  cudaError_t e;
  if (c->layout) {
    SegSumArgs gk{s1, c->d_kptr, c->d_contribK, c->d_K, s0};
    e = launch_segsum(gk, c->gather_bs, c->stream);
  } else {
    GatherArgs gk{s1, c->d_kptr, c->d_kids, c->d_contribK, c->d_K, s0};
    e = launch_gather_bs(gk, c->gather_bs, c->stream);
  }
  if (e == cudaSuccess && s1 > s0) c->launches++;
  return e;
}

cudaError_t enqueue_gather_F(nla3d_ctx* c) {
  cudaError_t e;
  if (c->layout) {
    SegSumArgs gf{c->Utot(), c->d_fptr, c->d_contribF, c->d_F};
    e = launch_segsum(gf, c->gather_bs, c->stream);
  } else {
    GatherArgs gf{c->Utot(), c->d_fptr, c->d_fids, c->d_contribF, c->d_F};
    e = launch_gather_bs(gf, c->gather_bs, c->stream);
  }
  if (e == cudaSuccess) c->launches++;
  return e;
}

// MPC rows after the element sums (FEStorage.cpp:41-61).
cudaError_t enqueue_mpc(nla3d_ctx* c) {
  cudaError_t e = cudaSuccess;
  if (c->Mtot()) {
    const uint64_t M = c->Mtot();
    MpcArgs a{};
    a.n_mpc = (uint32_t)M;
    a.master = c->d_mpc_u32;
    a.slave = c->d_mpc_u32 + M;
    a.eq = c->d_mpc_u32 + 2 * M;
    a.slave_eq = c->d_mpc_u32 + 3 * M;
    a.master_eq6 = c->d_mpc_u32 + 4 * M;
    a.slot = c->d_mpc_u32 + 10 * M;
    a.slave_dof = c->d_mpc_dof;
    a.xyz = c->d_xyz;
    a.U = c->d_U;
    a.K = c->d_K;
    a.F = c->d_F;
    e = launch_mpc(a, c->stream);
    if (e != cudaSuccess) return e;
    c->launches++;
  }
  if (c->n_lmpc) {
    LinearMpcArgs a{(uint32_t)c->n_lmpc, c->d_lmpc_eq, c->d_lmpc_b, c->d_lmpc_ptr,
                    c->d_lmpc_slot, c->d_lmpc_coef, c->d_K, c->d_F};
    e = launch_linear_mpc(a, c->stream);
    if (e != cudaSuccess) return e;
    c->launches++;
  }
  return e;
}

// C of a transient context with the K slots' gather lists (FEStorage.cpp:63-76:
// zeroC, buildC over the elements); M stays zero (no element here builds it)
cudaError_t enqueue_gather_C(nla3d_ctx* c) {
  if (!c->transient) return cudaSuccess;
  GatherArgs gc{c->Ktot(), c->d_kptr, c->d_kids, c->d_contribC, c->d_C};
  SegSumArgs sc{c->Ktot(), c->d_kptr, c->d_contribC, c->d_C};
  cudaError_t e = c->layout ? launch_segsum(sc, c->gather_bs, c->stream)
                            : launch_gather_bs(gc, c->gather_bs, c->stream);
  if (e == cudaSuccess) c->launches++;
  return e;
}

cudaError_t reset_status(nla3d_ctx* c) {
  cudaError_t e = cudaMemsetAsync(c->d_status, 0, sizeof(ElementStatus), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(&c->d_status->first, 0xFF, sizeof(uint32_t), c->stream);
  return e;
}

cudaError_t enqueue_assembly(nla3d_ctx* c) {
  const uint64_t slot = (c->timed % nla3d_ctx::kRing) * 5;
  auto mark = [&](int i) {
    if (c->timing) cudaEventRecord(c->ev[slot + i], c->stream);
  };
  cudaError_t e = reset_status(c);
  if (e != cudaSuccess) return e;
  mark(0);
  if ((e = enqueue_elements(c, 0, (uint32_t)c->E())) != cudaSuccess) return e;
  mark(1);
  if ((e = enqueue_gather_K(c, 0, c->Ktot())) != cudaSuccess) return e;
  if ((e = enqueue_gather_C(c)) != cudaSuccess) return e;
  mark(2);
  if ((e = enqueue_gather_F(c)) != cudaSuccess) return e;
  mark(3);
  if ((e = enqueue_mpc(c)) != cudaSuccess) return e;
  mark(4);
  if (c->timing) c->timed++;
  return cudaSuccess;
}

constexpr uint32_t kDevicePatternElems = 65536;

cudaError_t enqueue_update(nla3d_ctx* c) {
  return cudaMemcpyAsync(c->d_Ustate, c->d_U, sizeof(double) * c->Utot(), cudaMemcpyDeviceToDevice,
                         c->stream);
}

}  // namespace

extern "C" {

int nla3d_create(const nla3d_mesh_desc* mesh, int precision, nla3d_ctx** out) {
  return nla3d_create_batch(mesh, 1, precision, out);
}

int nla3d_create_batch(const nla3d_mesh_desc* meshes, uint32_t n_meshes, int precision,
                       nla3d_ctx** out) {
  if (!out) return NLA3D_ERR_ARG;
  *out = nullptr;
  if (!meshes || n_meshes == 0) return NLA3D_ERR_ARG;
  if (precision != NLA3D_PREC_FP64 && precision != NLA3D_PREC_MIXED) return NLA3D_ERR_ARG;
  for (uint32_t i = 0; i < n_meshes; i++) {
    int rc = check_mesh(&meshes[i]);
    if (rc) return rc;
    if (meshes[i].elem_type != meshes[0].elem_type) return NLA3D_ERR_ARG;
  }
  nla3d_ctx* c = new (std::nothrow) nla3d_ctx();
  if (!c) return NLA3D_ERR_NOMEM;
  c->hm.resize(n_meshes);
  for (uint32_t i = 0; i < n_meshes; i++) fill_model(c->hm[i], &meshes[i]);
  c->precision = precision;
  if (precision == NLA3D_PREC_MIXED && meshes[0].elem_type == NLA3D_SOLID81) {
    for (const HostModel& m : c->hm)
      if (!mixed_range_ok(m)) {
        delete c;
        return NLA3D_ERR_RANGE;
      }
  }
  *out = c;
  return NLA3D_OK;
}

uint32_t nla3d_mesh_count(const nla3d_ctx* c) { return c ? (uint32_t)c->hm.size() : 0; }

int nla3d_destroy(nla3d_ctx* c) {
  if (!c) return NLA3D_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  graph_release(c);
  for (void* p : c->allocs) cudaFree(p);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->allocs.clear();
  for (auto& v : c->ev) cudaEventDestroy(v);
  for (auto& v : c->chunk_ev) cudaEventDestroy(v);
  for (cudaStream_t cs : c->copy_stream)
    if (cs) cudaStreamDestroy(cs);
  delete c;
  return NLA3D_OK;
}

const char* nla3d_last_error(const nla3d_ctx* c) { return c ? c->err.c_str() : "null context"; }

int nla3d_set_stream(nla3d_ctx* c, void* stream) {
  if (!c) return NLA3D_ERR_ARG;
  if (c->own_stream && c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  graph_release(c);
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return NLA3D_OK;
}

void* nla3d_get_stream(const nla3d_ctx* c) { return c ? (void*)c->stream : nullptr; }

int nla3d_mesh_add_fix(nla3d_ctx* c, uint32_t mesh, uint32_t n, const uint32_t* nodes,
                       const int32_t* dofs) {
  if (!valid_mesh(c, mesh) || c->host_ready || (n && (!nodes || !dofs)))
    return fail(c, NLA3D_ERR_ARG, "add_fix");
  for (uint32_t i = 0; i < n; i++) {
    c->hm[mesh].fix_node.push_back(nodes[i]);
    c->hm[mesh].fix_dof.push_back(dofs[i]);
  }
  return NLA3D_OK;
}

int nla3d_add_fix(nla3d_ctx* c, uint32_t n, const uint32_t* nodes, const int32_t* dofs) {
  return nla3d_mesh_add_fix(c, 0, n, nodes, dofs);
}

int nla3d_add_surface_lines(nla3d_ctx* c, uint32_t n, const uint32_t* conn, const double* htc,
                            const double* flux, const double* etemp) {
  if (!c || c->host_ready || c->hm.size() != 1 || c->hm[0].etype != NLA3D_QUADTH ||
      (n && (!conn || !htc || !flux || !etemp)))
    return fail(c, NLA3D_ERR_ARG, "add_surface_lines: single-mesh QUADTH contexts");
  HostModel& m = c->hm[0];
  for (uint32_t l = 0; l < n; l++) {
    m.line_conn.push_back(conn[2 * l]);
    m.line_conn.push_back(conn[2 * l + 1]);
    // SurfaceLINETH::pre (QUADTH.cpp:79-82): etemp[1] = etemp[0] when etemp[1] is 0
    const double t0 = etemp[2 * l], t1 = etemp[2 * l + 1] == 0.0 ? t0 : etemp[2 * l + 1];
    const double par[4] = {htc[l], flux[l], t0, t1};
    m.line_par.insert(m.line_par.end(), par, par + 4);
  }
  return NLA3D_OK;
}

int nla3d_set_transient(nla3d_ctx* c, int on) {
  if (!c || c->ready) return fail(c, NLA3D_ERR_ARG, "set_transient after init_solution_data");
  if (on)
    for (const HostModel& m : c->hm)
      if (m.etype != NLA3D_QUADTH)
        return fail(c, NLA3D_ERR_ELEMENT, "transient C, M: only QUADTH builds them "
                                          "(Element::buildC/buildM abort, element.cpp:63-70)");
  c->transient = on != 0;
  return NLA3D_OK;
}

static int get_CM(nla3d_ctx* c, const double* src, int block, double* values, const char* what) {
  const int b = block_slot(block);
  if (!c || !c->ready || b < 0 || !c->transient) return fail(c, NLA3D_ERR_ARG, what);
  const uint64_t n = c->hm[0].blk[b].nnz();
  if (!n) return NLA3D_OK;
  if (!values) return fail(c, NLA3D_ERR_ARG, what);
  cudaError_t e = cudaMemcpyAsync(values, src + c->hm[0].val_off[b], sizeof(double) * n,
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, what);
}

int nla3d_get_C(nla3d_ctx* c, int block, double* values) {
  return get_CM(c, c ? c->d_C : nullptr, block, values, "get_C");
}

int nla3d_get_M(nla3d_ctx* c, int block, double* values) {
  return get_CM(c, c ? c->d_M : nullptr, block, values, "get_M");
}

int nla3d_mesh_add_mpc(nla3d_ctx* c, uint32_t mesh, uint32_t n_terms, const uint32_t* nodes,
                       const int32_t* dofs, const double* coefs, double b) {
  if (!valid_mesh(c, mesh) || c->host_ready || n_terms == 0 || !nodes || !dofs || !coefs)
    return fail(c, NLA3D_ERR_ARG, "add_mpc");
  LinearMpc q;
  q.node.assign(nodes, nodes + n_terms);
  q.dof.assign(dofs, dofs + n_terms);
  q.coef.assign(coefs, coefs + n_terms);
  q.b = b;
  c->hm[mesh].lmpcs.push_back(std::move(q));
  return NLA3D_OK;
}

int nla3d_add_mpc(nla3d_ctx* c, uint32_t n_terms, const uint32_t* nodes, const int32_t* dofs,
                  const double* coefs, double b) {
  return nla3d_mesh_add_mpc(c, 0, n_terms, nodes, dofs, coefs, b);
}

int nla3d_mesh_add_rigid_body(nla3d_ctx* c, uint32_t mesh, uint32_t master, uint32_t n_slaves,
                              const uint32_t* slaves, uint32_t n_dofs, const int32_t* dofs) {
  if (!valid_mesh(c, mesh) || c->host_ready || n_dofs > 3 || (n_slaves && !slaves) ||
      (n_dofs && !dofs))
    return fail(c, NLA3D_ERR_ARG, "add_rigid_body");
  RigidBody rb;
  rb.master = master;
  rb.slaves.assign(slaves, slaves + n_slaves);
  rb.dofs.assign(dofs, dofs + n_dofs);
  c->hm[mesh].rbs.push_back(rb);
  return NLA3D_OK;
}

int nla3d_add_rigid_body(nla3d_ctx* c, uint32_t master, uint32_t n_slaves, const uint32_t* slaves,
                         uint32_t n_dofs, const int32_t* dofs) {
  return nla3d_mesh_add_rigid_body(c, 0, master, n_slaves, slaves, n_dofs, dofs);
}

static int set_offsets(nla3d_ctx* c);

int nla3d_build_pattern(nla3d_ctx* c) {
  if (!c) return NLA3D_ERR_ARG;
  if (c->host_ready) return NLA3D_OK;
  const size_t M = c->hm.size();
  std::vector<std::string> msgs(M);
  if (M == 1) {
    msgs[0] = build_host_model(c->hm[0], 0);
  } else {
    // many meshes: one mesh per worker thread
    const unsigned nt =
        std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)M));
    std::vector<std::thread> th;
    std::mutex mu;
    size_t next = 0;
    for (unsigned t = 0; t < nt; t++)
      th.emplace_back([&] {
        for (;;) {
          size_t i;
          {
            std::lock_guard<std::mutex> l(mu);
            if (next >= M) return;
            i = next++;
          }
          msgs[i] = build_host_model(c->hm[i], 1);
        }
      });
    for (auto& t : th) t.join();
  }
  for (size_t i = 0; i < M; i++)
    if (!msgs[i].empty()) {
      std::string msg = M > 1 ? "mesh " + std::to_string(i) + ": " + msgs[i] : msgs[i];
      return fail(c, msgs[i].find("2^32") != std::string::npos ||
                             msgs[i].find("too many") != std::string::npos
                         ? NLA3D_ERR_RANGE
                         : NLA3D_ERR_PATTERN,
                  msg);
    }
  return set_offsets(c);
}

// offsets of the meshes in the concatenation; marks the host model ready
static int set_offsets(nla3d_ctx* c) {
  const size_t M = c->hm.size();
  // offsets of the concatenation
  c->elem_off.assign(M + 1, 0);
  c->node_off.assign(M + 1, 0);
  c->u_off.assign(M + 1, 0);
  c->k_off.assign(M + 1, 0);
  c->mpc_off.assign(M + 1, 0);
  for (size_t i = 0; i < M; i++) {
    const HostModel& m = c->hm[i];
    c->elem_off[i + 1] = c->elem_off[i] + m.n_elems;
    c->node_off[i + 1] = c->node_off[i] + m.n_nodes;
    c->u_off[i + 1] = c->u_off[i] + m.n_total();
    c->k_off[i + 1] = c->k_off[i] + m.nnz_total;
    c->mpc_off[i + 1] = c->mpc_off[i] + m.mpcs.size();
  }
  const uint64_t n_kc = c->hm[0].n_kc, n_fc = c->hm[0].n_fc;
  if (c->E() * (n_kc + n_fc) >= 0xFFFFFFF0ull || c->Ktot() >= 0xFFFFFFF0ull ||
      c->Utot() >= 0xFFFFFFF0ull || c->Ntot() >= 0xFFFFFFF0ull)
    return fail(c, NLA3D_ERR_RANGE, "batch exceeds 32-bit device indexing");
  c->uniform_material = true;
  for (size_t i = 1; i < M; i++) {
    const HostModel& a = c->hm[0];
    const HostModel& b = c->hm[i];
    if (a.mat_id != b.mat_id || std::memcmp(a.mat_c, b.mat_c, sizeof(a.mat_c)) != 0)
      c->uniform_material = false;
  }
  c->host_ready = true;
  return NLA3D_OK;
}

int nla3d_slot_maps(const nla3d_ctx* c, uint32_t* kslot, uint32_t* fslot) {
  if (!c || !c->host_ready || c->ready) return NLA3D_ERR_ARG;
  const HostModel& m = c->hm[0];
  if (kslot && !m.kslot.empty()) std::memcpy(kslot, m.kslot.data(), sizeof(uint32_t) * m.kslot.size());
  if (fslot && !m.fslot.empty()) std::memcpy(fslot, m.fslot.data(), sizeof(uint32_t) * m.fslot.size());
  return NLA3D_OK;
}

int nla3d_set_pattern_builder(nla3d_ctx* c, int mode) {
  if (!c || mode < -1 || mode > 1 || c->host_ready) return fail(c, NLA3D_ERR_ARG, "set_pattern_builder");
  c->pattern_mode = mode;
  return NLA3D_OK;
}

int nla3d_pattern_on_device(const nla3d_ctx* c) { return c && c->device_pattern ? 1 : 0; }

int nla3d_init_solution_data(nla3d_ctx* c) {
  if (!c || c->ready) return fail(c, NLA3D_ERR_ARG, "init_solution_data: bad call order");
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetDevice");
  if (!c->stream) {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamCreate");
    c->own_stream = true;
  }
  const bool device_build =
      !c->host_ready && c->hm.size() == 1 && c->hm[0].line_conn.empty() &&
      (c->pattern_mode == 1 || (c->pattern_mode == -1 && c->hm[0].n_elems >= kDevicePatternElems));
  if (device_build) {
    HostModel& m = c->hm[0];
    std::string msg = build_host_numbering(m);
    if (msg.empty()) {
      DeviceAlloc alloc = [c](void** p, size_t bytes) -> cudaError_t {
        cudaError_t err = cudaMalloc(p, bytes ? bytes : 1);
        if (err == cudaSuccess) c->allocs.push_back(*p);
        return err;
      };
      msg = build_pattern_gpu(m, c->stream, alloc, &c->pd);
      if (msg.rfind("fallback:", 0) == 0)
        msg = build_host_pattern(m, 0);
      else if (msg.empty())
        c->device_pattern = true;
    }
    if (!msg.empty())
      return fail(c, msg.find("2^32") != std::string::npos || msg.find("too many") != std::string::npos
                         ? NLA3D_ERR_RANGE : NLA3D_ERR_PATTERN, msg);
    int rc = set_offsets(c);
    if (rc) return rc;
  }
  int rc = nla3d_build_pattern(c);
  if (rc) return rc;
  const size_t M = c->hm.size();
  const uint64_t E = c->E(), N = c->Ntot(), ntot = c->Utot(), nnz = c->Ktot(), NM = c->Mtot();
  const int npe = c->hm[0].npe;
  const uint64_t n_kc = c->hm[0].n_kc, n_fc = c->hm[0].n_fc;
  const bool mixed_solid = c->precision == NLA3D_PREC_MIXED && c->hm[0].etype == NLA3D_SOLID81;
  // contributions: the elements', then (single-mesh QUADTH) the surface lines'
  const uint64_t LN = c->hm[0].n_lines();
  const uint64_t CK_tot = E * n_kc + LN * kLineKc, CF_tot = E * n_fc + LN * kLineFc;
  // concatenated host arrays with global offsets
  std::vector<double> xyz(3 * N);
  std::vector<uint32_t> conn(npe * E), neq3(4 * N, 0), peq(E, 0), elem_mesh;
  std::vector<double> eparams, mesh_mat;
  const bool host_lists = !c->device_pattern;
  std::vector<uint32_t> kptr(host_lists ? nnz + 1 : 0), kids(host_lists ? CK_tot : 0),
      fptr(host_lists ? ntot + 1 : 0), fids(host_lists ? CF_tot : 0);
  if (!c->uniform_material) {
    elem_mesh.resize(E);
    mesh_mat.assign(8 * M, 0.0);
  }
  if (!c->hm[0].eparams.empty()) eparams.resize((size_t)kElemParams * E);
  for (size_t i = 0; i < M; i++) {
    const HostModel& m = c->hm[i];
    const uint64_t eo = c->elem_off[i], no = c->node_off[i], uo = c->u_off[i], ko = c->k_off[i];
    std::memcpy(&xyz[3 * no], m.xyz.data(), sizeof(double) * 3 * m.n_nodes);
    for (uint64_t k = 0; k < (uint64_t)npe * m.n_elems; k++)
      conn[npe * eo + k] = m.conn[k] + (uint32_t)no;
    for (uint64_t n = 0; n < m.n_nodes; n++)
      for (int d = 0; d < 3; d++) {
        const uint32_t q = m.node_eq[n * kDofTypes + d];
        neq3[4 * (no + n) + d] = q ? q + (uint32_t)uo : 0;
      }
    for (uint64_t el = 0; el < m.n_elems; el++) {
      const uint32_t q = m.elem_eq[el * kDofTypes + HYDRO_PRESSURE];
      peq[eo + el] = q ? q + (uint32_t)uo : 0;
    }
    if (!eparams.empty())
      std::memcpy(&eparams[kElemParams * eo], m.eparams.data(),
                  sizeof(double) * kElemParams * m.n_elems);
    if (host_lists) {
      for (uint64_t s = 0; s < m.nnz_total; s++) kptr[ko + s] = m.k_ptr[s] + (uint32_t)(eo * n_kc);
      for (uint64_t k = 0; k < m.k_ids.size(); k++)
        kids[eo * n_kc + k] = m.k_ids[k] + (uint32_t)(eo * n_kc);
      for (uint64_t s = 0; s < m.n_total(); s++) fptr[uo + s] = m.f_ptr[s] + (uint32_t)(eo * n_fc);
      for (uint64_t k = 0; k < m.f_ids.size(); k++)
        fids[eo * n_fc + k] = m.f_ids[k] + (uint32_t)(eo * n_fc);
    }
    if (!c->uniform_material) {
      for (uint64_t el = 0; el < m.n_elems; el++) elem_mesh[eo + el] = (uint32_t)i;
      mesh_mat[8 * i + 0] = m.mat_id;
      for (int k = 0; k < 5; k++) mesh_mat[8 * i + 1 + k] = m.mat_c[k];
      mesh_mat[8 * i + 6] = bulk_of(m);
      mesh_mat[8 * i + 7] = 1.0 / bulk_of(m);
    }
  }
  std::vector<uint32_t> kpos, fpos;
  if (host_lists) {
    kptr[nnz] = (uint32_t)CK_tot;
    fptr[ntot] = (uint32_t)CF_tot;
    // slot-order position of every contribution: the inverse of the gather ids
    kpos.resize(CK_tot);
    fpos.resize(CF_tot);
    for (uint64_t k = 0; k < kids.size(); k++) kpos[kids[k]] = (uint32_t)k;
    for (uint64_t k = 0; k < fids.size(); k++) fpos[fids[k]] = (uint32_t)k;
  }

#define CK(x)                                           \
  do {                                                  \
    cudaError_t _e = (x);                               \
    if (_e != cudaSuccess) return cuda_fail(c, _e, #x); \
  } while (0)
  CK(upload(c, &c->d_xyz, xyz.data(), xyz.size()));
  CK(upload(c, &c->d_conn, conn.data(), conn.size()));
  CK(upload(c, &c->d_node_eq3, neq3.data(), neq3.size()));
  CK(upload(c, &c->d_p_eq, peq.data(), peq.size()));
  if (!eparams.empty()) CK(upload(c, &c->d_eparams, eparams.data(), eparams.size()));
  if (!c->uniform_material) {
    CK(upload(c, &c->d_elem_mesh, elem_mesh.data(), elem_mesh.size()));
    CK(upload(c, &c->d_mesh_mat, mesh_mat.data(), mesh_mat.size()));
  }
  std::vector<float2> mesh_mat_df;
  if (!c->uniform_material && mixed_solid) {
    mesh_mat_df.resize(mesh_mat.size());
    for (size_t i = 0; i < mesh_mat.size(); i++) mesh_mat_df[i] = split_pair(mesh_mat[i]);
    for (size_t i = 0; i < M; i++) mesh_mat_df[8 * i + 7] = split_pair(1.0 / mesh_mat[8 * i + 6]);
    CK(upload(c, &c->d_mesh_mat_df, mesh_mat_df.data(), mesh_mat_df.size()));
  }
  if (host_lists) {
    CK(upload(c, &c->d_kptr, kptr.data(), kptr.size()));
    CK(upload(c, &c->d_kids, kids.data(), kids.size()));
    CK(upload(c, &c->d_kpos, kpos.data(), kpos.size()));
    CK(upload(c, &c->d_fptr, fptr.data(), fptr.size()));
    CK(upload(c, &c->d_fids, fids.data(), fids.size()));
    CK(upload(c, &c->d_fpos, fpos.data(), fpos.size()));
  } else {
    c->d_kptr = c->pd.k_ptr;
    c->d_kids = c->pd.k_ids;
    c->d_kpos = c->pd.k_pos;
    c->d_fptr = c->pd.f_ptr;
    c->d_fids = c->pd.f_ids;
    c->d_fpos = c->pd.f_pos;
  }
  CK(dalloc(c, &c->d_U, ntot));
  CK(dalloc(c, &c->d_Ustate, ntot));
  CK(cudaMemsetAsync(c->d_U, 0, sizeof(double) * ntot, c->stream));
  CK(cudaMemsetAsync(c->d_Ustate, 0, sizeof(double) * ntot, c->stream));
  CK(dalloc(c, &c->d_contribK, CK_tot));
  CK(dalloc(c, &c->d_contribF, CF_tot ? CF_tot : 1));
  CK(dalloc(c, &c->d_K, nnz));
  CK(dalloc(c, &c->d_F, ntot));
  CK(dalloc(c, &c->d_status, 1));
  if (LN) {
    c->n_lines = (uint32_t)LN;
    CK(upload(c, &c->d_line_conn, c->hm[0].line_conn.data(), c->hm[0].line_conn.size()));
    CK(upload(c, &c->d_line_par, c->hm[0].line_par.data(), c->hm[0].line_par.size()));
  }
  if (c->transient) {
    // C and M share K's pattern (FEStorage.cpp:475-479); no element of this
    // set builds M, so M stays zero; the lines add nothing to C
    CK(dalloc(c, &c->d_contribC, CK_tot));
    CK(cudaMemsetAsync(c->d_contribC, 0, sizeof(double) * CK_tot, c->stream));
    CK(dalloc(c, &c->d_C, nnz));
    CK(dalloc(c, &c->d_M, nnz));
    CK(cudaMemsetAsync(c->d_C, 0, sizeof(double) * (nnz ? nnz : 1), c->stream));
    CK(cudaMemsetAsync(c->d_M, 0, sizeof(double) * (nnz ? nnz : 1), c->stream));
  }
  if (NM) {
    // per MPC: master, slave, eq, slave_eq, master_eq6[6], slot[5]  (15 words), global
    std::vector<uint32_t> w(15ull * NM);
    std::vector<int32_t> dof(NM);
    for (size_t i = 0; i < M; i++) {
      const HostModel& m = c->hm[i];
      const uint32_t no = (uint32_t)c->node_off[i], uo = (uint32_t)c->u_off[i],
                     ko = (uint32_t)c->k_off[i];
      // the MPC kernel adds each coefficient to its slot; slots are distinct by
      // construction (one column per MPC equation), verify before trusting it
      std::vector<uint32_t> sl(m.mpc_slot);
      std::sort(sl.begin(), sl.end());
      if (std::adjacent_find(sl.begin(), sl.end()) != sl.end())
        return fail(c, NLA3D_ERR_PATTERN, "two MPC terms share one K slot");
      for (uint64_t k = 0; k < m.mpcs.size(); k++) {
        const uint64_t g = c->mpc_off[i] + k;
        const MpcEq& q = m.mpcs[k];
        w[g] = q.node[1] + no;
        w[NM + g] = q.slave + no;
        w[2 * NM + g] = q.eq + uo;
        w[3 * NM + g] = m.neq(q.slave, q.slave_dof) + uo;
        for (int t = 0; t < 6; t++) w[4 * NM + 6 * g + t] = m.neq(q.node[1], t) + uo;
        for (int t = 0; t < 5; t++) w[10 * NM + 5 * g + t] = m.mpc_slot[5 * k + t] + ko;
        dof[g] = q.slave_dof;
      }
    }
    CK(upload(c, &c->d_mpc_u32, w.data(), w.size()));
    CK(upload(c, &c->d_mpc_dof, dof.data(), dof.size()));
  }
  {
    // linear MPC equations, global numbering (eq + u_off, slot + k_off)
    std::vector<uint32_t> leq, lptr(1, 0), lslot;
    std::vector<double> lb, lcoef;
    for (size_t i = 0; i < M; i++) {
      const HostModel& m = c->hm[i];
      const uint32_t uo = (uint32_t)c->u_off[i], ko = (uint32_t)c->k_off[i];
      size_t t0 = 0;
      for (const LinearMpc& q : m.lmpcs) {
        leq.push_back(q.eq + uo);
        lb.push_back(q.b);
        for (size_t t = 0; t < q.node.size(); t++) {
          lslot.push_back(m.lmpc_slot[t0 + t] + ko);
          lcoef.push_back(q.coef[t]);
        }
        t0 += q.node.size();
        lptr.push_back((uint32_t)lslot.size());
      }
    }
    c->n_lmpc = leq.size();
    if (c->n_lmpc) {
      CK(upload(c, &c->d_lmpc_eq, leq.data(), leq.size()));
      CK(upload(c, &c->d_lmpc_b, lb.data(), lb.size()));
      CK(upload(c, &c->d_lmpc_ptr, lptr.data(), lptr.size()));
      CK(upload(c, &c->d_lmpc_slot, lslot.data(), lslot.size()));
      CK(upload(c, &c->d_lmpc_coef, lcoef.data(), lcoef.size()));
    }
  }
  CK(cudaMemsetAsync(c->d_status, 0, sizeof(ElementStatus), c->stream));
  CK(cudaMemsetAsync(&c->d_status->first, 0xFF, sizeof(uint32_t), c->stream));
  if (c->hm[0].etype == NLA3D_SOLID81) {
    // FP64 contexts keep dN/dX as doubles, mixed ones as float pairs only
    if (mixed_solid) {
      CK(dalloc(c, &c->d_Gdf, 24 * 8 * E));
      CK(dalloc(c, &c->d_wdf, 8 * E));
    } else {
      CK(dalloc(c, &c->d_Gt, 24 * 8 * E));
    }
    CK(dalloc(c, &c->d_wdet, 8 * E));
    JacobianArgs ja{(uint32_t)E, c->d_xyz, c->d_conn, c->d_Gt, c->d_wdet, c->d_status,
                    c->d_Gdf, c->d_wdf};
    CK(launch_solid81_jacobian(ja, c->stream));
    c->launches++;
  }
  CK(prepare_device_tables());
  CK(cudaStreamSynchronize(c->stream));
  // the gather lists and slot maps now live on the device only
  for (HostModel& m : c->hm) {
    std::vector<uint32_t>().swap(m.kslot);
    std::vector<uint32_t>().swap(m.fslot);
    std::vector<uint32_t>().swap(m.k_ids);
    std::vector<uint32_t>().swap(m.f_ids);
    std::vector<uint32_t>().swap(m.k_ptr);
    std::vector<uint32_t>().swap(m.f_ptr);
  }
  c->ready = true;
  return NLA3D_OK;
}

int nla3d_mesh_info(const nla3d_ctx* c, uint32_t mesh, uint32_t out[16], uint64_t offsets[5]) {
  if (!valid_mesh(c, mesh) || !c->host_ready || !out) return NLA3D_ERR_ARG;
  const HostModel& m = c->hm[mesh];
  std::memset(out, 0, sizeof(uint32_t) * 16);
  out[0] = m.n_dofs;
  out[1] = m.n_con;
  out[2] = m.n_unk;
  out[3] = m.n_mpc;
  for (int b = 0; b < 3; b++) {
    out[4 + 3 * b] = m.blk[b].rows;
    out[5 + 3 * b] = m.blk[b].cols;
    out[6 + 3 * b] = (uint32_t)m.blk[b].nnz();
  }
  out[13] = (uint32_t)m.n_kc;
  out[14] = (uint32_t)m.n_fc;
  if (offsets) {
    offsets[0] = c->elem_off[mesh];
    offsets[1] = c->node_off[mesh];
    offsets[2] = c->u_off[mesh];
    offsets[3] = c->k_off[mesh];
    offsets[4] = c->mpc_off[mesh];
  }
  return NLA3D_OK;
}

int nla3d_info(const nla3d_ctx* c, uint32_t out[16]) { return nla3d_mesh_info(c, 0, out, nullptr); }

int nla3d_mesh_pattern(const nla3d_ctx* c, uint32_t mesh, int block, uint32_t* iofeir,
                       uint32_t* columns) {
  const int b = block_slot(block);
  if (!valid_mesh(c, mesh) || !c->host_ready || b < 0 || !iofeir) return NLA3D_ERR_ARG;
  const CsrBlock& B = c->hm[mesh].blk[b];
  std::memcpy(iofeir, B.iofeir.data(), sizeof(uint32_t) * (B.rows + 1));
  if (B.nnz()) {
    if (!columns) return NLA3D_ERR_ARG;
    std::memcpy(columns, B.columns.data(), sizeof(uint32_t) * B.nnz());
  }
  return NLA3D_OK;
}

int nla3d_pattern(const nla3d_ctx* c, int block, uint32_t* iofeir, uint32_t* columns) {
  return nla3d_mesh_pattern(c, 0, block, iofeir, columns);
}

int nla3d_mesh_eq_numbers(const nla3d_ctx* c, uint32_t mesh, uint32_t* node_eq, uint32_t* elem_eq) {
  if (!valid_mesh(c, mesh) || !c->host_ready) return NLA3D_ERR_ARG;
  const HostModel& m = c->hm[mesh];
  if (node_eq) std::memcpy(node_eq, m.node_eq.data(), sizeof(uint32_t) * m.node_eq.size());
  if (elem_eq) std::memcpy(elem_eq, m.elem_eq.data(), sizeof(uint32_t) * m.elem_eq.size());
  return NLA3D_OK;
}

int nla3d_eq_numbers(const nla3d_ctx* c, uint32_t* node_eq, uint32_t* elem_eq) {
  return nla3d_mesh_eq_numbers(c, 0, node_eq, elem_eq);
}

int nla3d_set_U(nla3d_ctx* c, const double* U, uint64_t n) {
  if (!c || !c->ready || !U || n != c->Utot()) return fail(c, NLA3D_ERR_ARG, "set_U size");
  cudaError_t e = cudaMemcpyAsync(c->d_U, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "set_U");
}

int nla3d_set_U_device(nla3d_ctx* c, const double* U, uint64_t n) {
  if (!c || !c->ready || !U || n != c->Utot()) return fail(c, NLA3D_ERR_ARG, "set_U size");
  cudaError_t e =
      cudaMemcpyAsync(c->d_U, U, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "set_U_device");
}

int nla3d_update_results(nla3d_ctx* c) {
  if (!c || !c->ready) return fail(c, NLA3D_ERR_ARG, "update_results before init");
  // SOLID81 keeps its Gauss-point state as a snapshot of vecU; the linear
  // elements have no state on the assembly path.
  cudaError_t e = enqueue_update(c);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_results");
  c->have_state = true;
  return NLA3D_OK;
}

int nla3d_assemble(nla3d_ctx* c) {
  if (!c || !c->ready) return fail(c, NLA3D_ERR_ARG, "assemble before init");
  cudaError_t e = enqueue_assembly(c);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "assemble");
}

int nla3d_get_K(nla3d_ctx* c, int block, double* values) {
  const int b = block_slot(block);
  if (!c || !c->ready || b < 0) return fail(c, NLA3D_ERR_ARG, "get_K");
  const uint64_t n = c->hm[0].blk[b].nnz();
  if (!n) return NLA3D_OK;
  if (!values) return fail(c, NLA3D_ERR_ARG, "get_K: null output");
  cudaError_t e = cudaMemcpyAsync(values, c->d_K + c->hm[0].val_off[b], sizeof(double) * n,
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "get_K");
}

int nla3d_get_K_all(nla3d_ctx* c, double* values) {
  if (!c || !c->ready || !values) return fail(c, NLA3D_ERR_ARG, "get_K_all");
  cudaError_t e = cudaMemcpyAsync(values, c->d_K, sizeof(double) * c->Ktot(),
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "get_K_all");
}

int nla3d_get_F(nla3d_ctx* c, double* F) {
  if (!c || !c->ready || !F) return fail(c, NLA3D_ERR_ARG, "get_F");
  cudaError_t e = cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->Utot(), cudaMemcpyDeviceToHost,
                                  c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "get_F");
}

namespace {

// Element ranges for n chunks and the K slots to sum and copy after each:
// slot s is complete once the last element contributing to it is done (its
// range index r(s)); MPC slots are written after every range (r = n - 1).
// After range k < n - 1, every run of not yet copied slots with r <= k of at
// least kMinRun slots is summed and copied; after the last range the rest,
// with gaps shorter than kMaxGap merged (re-summing a finished slot writes the
// same value, so copying it again is harmless).
constexpr uint64_t kMinRun = 1u << 16;
constexpr uint64_t kMaxGap = 1u << 20;

int make_chunk_plan(nla3d_ctx* c, int n) {
  const uint64_t E = c->E(), nnz = c->Ktot();
  const uint32_t align = c->hm[0].etype == NLA3D_SOLID81 ? 4u : 1u;
  // range k holds a share n - k of n (n + 1) / 2 of the elements: long
  // ranges first, while their finished slots stream to the host behind
  // them; short ranges last, so that little is left to sum and copy after
  // the last one
  std::vector<uint32_t> eb(n + 1, 0);
  const uint64_t total_w = (uint64_t)n * (n + 1) / 2;
  for (int k = 1; k < n; k++) {
    const uint64_t w = (uint64_t)k * n - (uint64_t)k * (k - 1) / 2;
    eb[k] = (uint32_t)((E * w / total_w) / align * align);
  }
  eb[n] = (uint32_t)E;
  for (int k = 1; k <= n; k++) eb[k] = std::max(eb[k], eb[k - 1]);
  std::vector<uint8_t> r(nnz, 0);
  if (nnz) {
    uint32_t* d_eb = nullptr;
    uint8_t* d_r = nullptr;
    cudaError_t e = cudaMalloc((void**)&d_eb, sizeof(uint32_t) * (n + 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_r, nnz);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_eb, eb.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice,
                          c->stream);
    if (e == cudaSuccess)
      e = launch_slot_last_range(nnz, c->d_kptr, c->d_kids, (uint32_t)c->hm[0].n_kc, d_eb, n, d_r,
                                 c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.data(), d_r, nnz, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    const cudaError_t f1 = d_eb ? cudaFree(d_eb) : cudaSuccess;
    const cudaError_t f2 = d_r ? cudaFree(d_r) : cudaSuccess;
    if (e == cudaSuccess) e = f1 != cudaSuccess ? f1 : f2;
    if (e != cudaSuccess) return cuda_fail(c, e, "assemble_to_host plan");
  }
  for (uint32_t sl : c->hm[0].mpc_slot) r[sl] = (uint8_t)(n - 1);
  for (uint32_t sl : c->hm[0].lmpc_slot) r[sl] = (uint8_t)(n - 1);
  const uint8_t kCopied = 0xFF;  // r values are < n <= 64
  std::vector<nla3d_ctx::SlotRun> runs;
  for (int k = 0; k + 1 < n; k++) {
    uint64_t s = 0;
    while (s < nnz) {
      if (r[s] > k) {
        s++;
        continue;
      }
      uint64_t t = s;
      while (t < nnz && r[t] <= k) t++;   // copied slots (0xFF) end a run
      if (t - s >= kMinRun) {
        runs.push_back({k, s, t});
        std::fill(r.begin() + s, r.begin() + t, kCopied);
      }
      s = t;
    }
  }
  // the rest after the last range, small gaps merged
  uint64_t s = 0;
  while (s < nnz) {
    if (r[s] == kCopied) {
      s++;
      continue;
    }
    uint64_t t = s + 1, gap = 0;
    for (uint64_t q = s + 1; q < nnz && gap < kMaxGap; q++) {
      if (r[q] == kCopied) {
        gap++;
      } else {
        gap = 0;
        t = q + 1;
      }
    }
    runs.push_back({n - 1, s, t});
    s = t;
  }
  c->plan_eb.swap(eb);
  c->plan_runs.swap(runs);
  c->plan_chunks = n;
  return NLA3D_OK;
}

}  // namespace

int nla3d_assemble_to_host(nla3d_ctx* c, int n_chunks, double* K1, double* K12, double* K2,
                           double* F) {
  if (!c || !c->ready || c->hm.size() != 1 || n_chunks < 1 || n_chunks > 64)
    return fail(c, NLA3D_ERR_ARG, "assemble_to_host");
  const HostModel& m = c->hm[0];
  double* host[3] = {K1, K12, K2};
  for (int b = 0; b < 3; b++)
    if (m.blk[b].nnz() && !host[b]) return fail(c, NLA3D_ERR_ARG, "assemble_to_host: null K");
  if (!F) return fail(c, NLA3D_ERR_ARG, "assemble_to_host: null F");
  cudaError_t e = cudaGetLastError();  // an error left by an earlier call is reported here
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble_to_host: pending error");
  if (c->plan_chunks != n_chunks) {
    int rc = make_chunk_plan(c, n_chunks);
    if (rc) return rc;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble_to_host: after the plan");
  for (cudaStream_t& cs : c->copy_stream)
    if (!cs) {
      e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
      if (e != cudaSuccess) return cuda_fail(c, e, "assemble_to_host: stream");
    }
  while (c->chunk_ev.size() < 64) {
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(c, e, "assemble_to_host: event");
    c->chunk_ev.push_back(ev);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble_to_host: after stream/events");
  // copy K values [s0, s1) of the concatenated blocks into the block arrays,
  // each piece in equal parts on the copy streams
  constexpr int ncs = nla3d_ctx::kCopyStreams;
  auto copy_range = [&](uint64_t s0, uint64_t s1) -> cudaError_t {
    for (int b = 0; b < 3 && s0 < s1; b++) {
      const uint64_t lo = m.val_off[b], hi = lo + m.blk[b].nnz();
      const uint64_t a = std::max(s0, lo), z = std::min(s1, hi);
      if (a >= z) continue;
      for (int h = 0; h < ncs; h++) {
        const uint64_t p0 = a + (z - a) * h / ncs, p1 = a + (z - a) * (h + 1) / ncs;
        if (p0 >= p1) continue;
        cudaError_t err = cudaMemcpyAsync(host[b] + (p0 - lo), c->d_K + p0,
                                          sizeof(double) * (p1 - p0), cudaMemcpyDeviceToHost,
                                          c->copy_stream[h]);
        if (err != cudaSuccess) return err;
      }
    }
    return cudaSuccess;
  };
  const int n = n_chunks;
  const char* where = "status reset";
  e = reset_status(c);
  size_t ri = 0;
  const auto& runs = c->plan_runs;
  for (int k = 0; k < n && e == cudaSuccess; k++) {
    where = "element kernel";
    e = enqueue_elements(c, c->plan_eb[k], c->plan_eb[k + 1]);
    const size_t r0 = ri;
    while (ri < runs.size() && runs[ri].k == k && e == cudaSuccess) {
      where = "K gather";
      e = enqueue_gather_K(c, runs[ri].s0, runs[ri].s1);
      ri++;
    }
    if (e == cudaSuccess && k == n - 1) where = "C gather", e = enqueue_gather_C(c);
    if (e == cudaSuccess && k == n - 1) where = "F gather", e = enqueue_gather_F(c);
    if (e == cudaSuccess && k == n - 1) where = "MPC rows", e = enqueue_mpc(c);
    if (r0 == ri && k < n - 1) continue;  // nothing to copy after this range
    if (e == cudaSuccess) where = "event record", e = cudaEventRecord(c->chunk_ev[k], c->stream);
    for (int h = 0; h < ncs && e == cudaSuccess; h++)
      where = "stream wait", e = cudaStreamWaitEvent(c->copy_stream[h], c->chunk_ev[k], 0);
    for (size_t q = r0; q < ri && e == cudaSuccess; q++) {
      where = "K copy";
      e = copy_range(runs[q].s0, runs[q].s1);
    }
  }
  if (e == cudaSuccess)
    where = "F copy", e = cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->Utot(),
                                          cudaMemcpyDeviceToHost, c->copy_stream[ncs - 1]);
  for (int h = 0; h < ncs && e == cudaSuccess; h++)
    where = "copy stream sync", e = cudaStreamSynchronize(c->copy_stream[h]);
  if (e != cudaSuccess) return cuda_fail(c, e, (std::string("assemble_to_host: ") + where).c_str());
  return NLA3D_OK;
}

int nla3d_block_mv(nla3d_ctx* c, uint32_t mesh, int block, int trans, const double* x,
                   double coef, double* y) {
  const int b = block_slot(block);
  if (!c || !c->ready || !valid_mesh(c, mesh) || b < 0 || (trans != 0 && trans != 1))
    return fail(c, NLA3D_ERR_ARG, "block_mv");
  const int kind = block == 1 ? 0 : (block == 2 ? 1 : (trans ? 3 : 2));
  if (c->mv.size() != c->hm.size()) c->mv.assign(c->hm.size(), std::vector<nla3d_ctx::MvList>(4));
  nla3d_ctx::MvList& L = c->mv[mesh][kind];
  const CsrBlock& blk = c->hm[mesh].blk[b];
  if (!L.built) {
    std::vector<uint32_t> ptr, slot, xi;
    build_walk(blk, kind, ptr, slot, xi);
    cudaError_t e = upload(c, &L.ptr, ptr.data(), ptr.size());
    if (e == cudaSuccess) e = upload(c, &L.slot, slot.data(), slot.size());
    if (e == cudaSuccess) e = upload(c, &L.xi, xi.data(), xi.size());
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "block_mv lists");
    L.n_out = ptr.size() - 1;
    L.n_entries = ptr.back();
    L.built = true;
  }
  if (L.n_entries == 0) return NLA3D_OK;  // y unchanged (no stored entries)
  if (!x || !y) return fail(c, NLA3D_ERR_ARG, "block_mv: null vector");
  BlockMvArgs a{L.n_out, L.ptr, L.slot, L.xi, c->d_K + c->k_off[mesh] + c->hm[mesh].val_off[b],
                x, coef, y, kind <= 1 ? 1 : 0};
  cudaError_t e = launch_block_mv(a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "block_mv");
  c->launches++;
  return NLA3D_OK;
}

int nla3d_device_K(const nla3d_ctx* c, int block, double** values, uint64_t* n) {
  if (!c || !c->ready || !values || !n) return NLA3D_ERR_ARG;
  if (block == 0) {
    *values = c->d_K;
    *n = c->Ktot();
    return NLA3D_OK;
  }
  const int b = block_slot(block);
  if (b < 0) return NLA3D_ERR_ARG;
  *values = c->d_K + c->hm[0].val_off[b];
  *n = c->hm[0].blk[b].nnz();
  return NLA3D_OK;
}

int nla3d_device_F(const nla3d_ctx* c, double** F, uint64_t* n) {
  if (!c || !c->ready || !F || !n) return NLA3D_ERR_ARG;
  *F = c->d_F;
  *n = c->Utot();
  return NLA3D_OK;
}

int nla3d_synchronize(nla3d_ctx* c) {
  if (!c || !c->stream) return NLA3D_ERR_ARG;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "synchronize");
}

int nla3d_element_status(nla3d_ctx* c, uint32_t* count, uint32_t* first) {
  if (!c || !c->ready) return NLA3D_ERR_ARG;
  ElementStatus st{0, 0};
  cudaError_t e = cudaMemcpyAsync(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "element_status");
  if (count) *count = st.count;
  if (first) *first = st.count ? st.first : 0;
  return st.count ? NLA3D_ERR_ELEMENT : NLA3D_OK;
}

uint64_t nla3d_kernel_launches(const nla3d_ctx* c) { return c ? c->launches : 0; }

int nla3d_set_launch_shape(nla3d_ctx* c, int warps_per_block, int blocks_per_sm,
                           int gather_block) {
  if (!c) return NLA3D_ERR_ARG;
  if (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8) return NLA3D_ERR_ARG;
  if (gather_block != 128 && gather_block != 256 && gather_block != 512 && gather_block != 1024)
    return NLA3D_ERR_ARG;
  c->shape.warps_per_block = warps_per_block;
  c->shape.blocks_per_sm = blocks_per_sm < 0 ? 0 : blocks_per_sm;
  c->gather_bs = gather_block;
  graph_release(c);
  return NLA3D_OK;
}

int nla3d_set_contrib_layout(nla3d_ctx* c, int layout) {
  if (!c || (layout != 0 && layout != 1)) return NLA3D_ERR_ARG;
  c->layout = layout;
  graph_release(c);
  return NLA3D_OK;
}

int nla3d_autotune(nla3d_ctx* c, int reps, int32_t chosen[4], float* best_ms) {
  if (!c || !c->ready) return fail(c, NLA3D_ERR_ARG, "autotune before init");
  if (reps < 1) reps = 1;
  graph_release(c);
  const bool mixed = c->precision == NLA3D_PREC_MIXED;
  const bool solid = c->hm[0].etype == NLA3D_SOLID81;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess)
    return fail(c, NLA3D_ERR_CUDA, "autotune events");
  const bool was_timing = c->timing;
  c->timing = false;
  auto measure = [&](float* ms) -> cudaError_t {
    cudaError_t e = enqueue_assembly(c);  // warm
    if (e != cudaSuccess) return e;
    cudaEventRecord(t0, c->stream);
    for (int r = 0; r < reps; r++) {
      e = enqueue_assembly(c);
      if (e != cudaSuccess) return e;
    }
    cudaEventRecord(t1, c->stream);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) return e;
    cudaEventElapsedTime(ms, t0, t1);
    *ms /= reps;
    return cudaSuccess;
  };
  Solid81Shape best_shape = c->shape;
  int best_bs = c->gather_bs, best_layout = c->layout;
  float best = 3.4e38f;
  cudaError_t e = cudaSuccess;
  const int wpbs[3] = {2, 4, 8};
  for (int layout = 0; layout < 2 && e == cudaSuccess; layout++) {
    c->layout = layout;
    for (int wi = 0; wi < (solid ? 3 : 1) && e == cudaSuccess; wi++) {
      const int maxb = solid ? solid81_max_blocks_per_sm(mixed, wpbs[wi]) : 1;
      for (int b = 1; b <= maxb && e == cudaSuccess; b++) {
        c->shape.warps_per_block = wpbs[wi];
        c->shape.blocks_per_sm = b;
        float ms = 0;
        e = measure(&ms);
        if (e == cudaSuccess && ms < best) {
          best = ms;
          best_shape = c->shape;
          best_layout = layout;
        }
      }
    }
  }
  c->shape = best_shape;
  c->layout = best_layout;
  const int bss[4] = {128, 256, 512, 1024};
  best = 3.4e38f;
  for (int i = 0; i < 4 && e == cudaSuccess; i++) {
    c->gather_bs = bss[i];
    float ms = 0;
    e = measure(&ms);
    if (e == cudaSuccess && ms < best) {
      best = ms;
      best_bs = bss[i];
    }
  }
  c->gather_bs = best_bs;
  c->timing = was_timing;
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (e != cudaSuccess) return cuda_fail(c, e, "autotune");
  if (chosen) {
    chosen[0] = c->shape.warps_per_block;
    chosen[1] = c->shape.blocks_per_sm;
    chosen[2] = c->gather_bs;
    chosen[3] = c->layout;
  }
  if (best_ms) *best_ms = best;
  return NLA3D_OK;
}

int nla3d_graph_capture(nla3d_ctx* c) {
  if (!c || !c->ready) return fail(c, NLA3D_ERR_ARG, "graph_capture before init");
  graph_release(c);
  cudaError_t e = prepare_device_tables();
  if (e != cudaSuccess) return cuda_fail(c, e, "graph_capture: tables");
  const bool was_timing = c->timing;
  c->timing = false;
  e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    c->timing = was_timing;
    return cuda_fail(c, e, "graph_capture: begin");
  }
  const uint64_t launches0 = c->launches;
  cudaError_t eu = enqueue_update(c);
  cudaError_t ea = eu == cudaSuccess ? enqueue_assembly(c) : eu;
  e = cudaStreamEndCapture(c->stream, &c->graph);
  c->launches = launches0;  // nothing ran yet
  c->timing = was_timing;
  if (ea != cudaSuccess) {
    graph_release(c);
    return cuda_fail(c, ea, "graph_capture: enqueue");
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "graph_capture: end");
  e = cudaGraphInstantiate(&c->graph_exec, c->graph, 0);
  if (e != cudaSuccess) {
    graph_release(c);
    return cuda_fail(c, e, "graph_capture: instantiate");
  }
  c->have_state = true;
  return NLA3D_OK;
}

int nla3d_graph_launch(nla3d_ctx* c) {
  if (!c || !c->graph_exec) return fail(c, NLA3D_ERR_ARG, "graph_launch without a captured graph");
  cudaError_t e = cudaGraphLaunch(c->graph_exec, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "graph_launch");
  c->launches += 3 + (c->Mtot() ? 1 : 0) + (c->n_lmpc ? 1 : 0);
  return NLA3D_OK;
}

int nla3d_set_timing(nla3d_ctx* c, int on) {
  if (!c) return NLA3D_ERR_ARG;
  if (on && c->ev.empty()) {
    c->ev.resize(nla3d_ctx::kRing * 5);
    for (auto& v : c->ev) {
      cudaError_t e = cudaEventCreate(&v);
      if (e != cudaSuccess) return cuda_fail(c, e, "set_timing");
    }
  }
  c->timing = on != 0;
  c->timed = 0;
  return NLA3D_OK;
}

int nla3d_kernel_times(nla3d_ctx* c, float ms[4], uint32_t* count) {
  if (!c || !ms || c->ev.empty()) return NLA3D_ERR_ARG;
  const uint64_t n = c->timed < (uint64_t)nla3d_ctx::kRing ? c->timed : nla3d_ctx::kRing;
  double acc[4] = {0, 0, 0, 0};
  for (uint64_t k = 0; k < n; k++) {
    const uint64_t slot = ((c->timed - 1 - k) % nla3d_ctx::kRing) * 5;
    cudaError_t e = cudaEventSynchronize(c->ev[slot + 4]);
    if (e != cudaSuccess) return cuda_fail(c, e, "kernel_times");
    for (int i = 0; i < 4; i++) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, c->ev[slot + i], c->ev[slot + i + 1]);
      acc[i] += t;
    }
  }
  for (int i = 0; i < 4; i++) ms[i] = n ? (float)(acc[i] / n) : 0.0f;
  if (count) *count = (uint32_t)n;
  c->timed = 0;
  return NLA3D_OK;
}

int nla3d_probe_fma_peak(int fp64, double* flops) {
  if (!flops) return NLA3D_ERR_ARG;
  cudaError_t e = probe_fma_peak(fp64 != 0, flops);
  return e == cudaSuccess ? NLA3D_OK : NLA3D_ERR_CUDA;
}

}  // extern "C"
