// C ABI of the assembly path (include/nla3d_gpu.h): context, device memory
// layout and the launch sequence of one assembly.
//
// Device layout of one context (E elements, N nodes, nnz = K nonzeros):
//   Gt      24 x 8E  double  dN/dX per Gauss point, structure of arrays
//   wdet    8E       double  Gauss weight * det J
//   conn    8E       uint32  node ids (1-based)
//   node_eq 4N       uint32  equations of UX, UY, UZ (+ pad) per node
//   p_eq    E        uint32  equation of each element's pressure DoF
//   U, U_state       double  current vecU / vecU at the last updateResults()
//   contribK 325E, contribF 25E  double   element contributions, reference order
//   k_ptr nnz+1, k_ids 325E  uint32   fixed-order gather lists of K
//   f_ptr n+1,   f_ids 25E   uint32   same for F
//   K (block(1) | block(1,2) | block(2) values), F    double
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/nla3d_gpu.h"
#include "host_model.hpp"
#include "kernels.cuh"

using namespace nla3d_gpu;

struct nla3d_ctx {
  HostModel hm;
  int precision = NLA3D_PREC_FP64;
  std::string err;
  bool host_ready = false;  // nla3d_build_pattern done
  bool ready = false;       // nla3d_init_solution_data done
  int device = -1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool have_state = false;
  uint64_t launches = 0;
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
  uint32_t* d_fptr = nullptr;
  uint32_t* d_fids = nullptr;
  double* d_K = nullptr;
  double* d_F = nullptr;
  uint32_t* d_mpc_u32 = nullptr;  // master, slave, eq, slave_eq, master_eq6 (6), slot (5)
  int32_t* d_mpc_dof = nullptr;
  ElementStatus* d_status = nullptr;
  std::vector<void*> allocs;
  bool timing = false;
  static constexpr int kRing = 256;
  std::vector<cudaEvent_t> ev;  // kRing x 5
  uint64_t timed = 0;           // assemblies recorded since the last read
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

int block_slot(int block) { return block == 1 ? 0 : (block == 2 ? 2 : (block == 12 ? 1 : -1)); }

}  // namespace

extern "C" {

int nla3d_create(const nla3d_mesh_desc* mesh, int precision, nla3d_ctx** out) {
  if (!out) return NLA3D_ERR_ARG;
  *out = nullptr;
  if (!mesh || (mesh->n_elems && (!mesh->conn || !mesh->xyz))) return NLA3D_ERR_ARG;
  if (mesh->elem_type != NLA3D_SOLID81 && mesh->elem_type != NLA3D_TETRA0 &&
      mesh->elem_type != NLA3D_QUADTH)
    return NLA3D_ERR_ARG;
  if (precision != NLA3D_PREC_FP64 && precision != NLA3D_PREC_MIXED) return NLA3D_ERR_ARG;
  if (mesh->elem_type == NLA3D_SOLID81 &&
      (mesh->mat_id < NLA3D_MAT_NEO_HOOKEAN || mesh->mat_id > NLA3D_MAT_MOONEY_RIVLIN))
    return NLA3D_ERR_ARG;
  if (mesh->elem_type != NLA3D_SOLID81 && !mesh->elem_params && mesh->n_elems) return NLA3D_ERR_ARG;
  nla3d_ctx* c = new (std::nothrow) nla3d_ctx();
  if (!c) return NLA3D_ERR_NOMEM;
  HostModel& m = c->hm;
  m.etype = mesh->elem_type;
  m.npe = m.etype == NLA3D_SOLID81 ? 8 : 4;
  m.n_nodes = mesh->n_nodes;
  m.n_elems = mesh->n_elems;
  m.xyz.assign(mesh->xyz, mesh->xyz + 3 * (size_t)mesh->n_nodes);
  m.conn.assign(mesh->conn, mesh->conn + (size_t)m.npe * mesh->n_elems);
  m.mat_id = mesh->mat_id;
  for (int i = 0; i < 5; i++) m.mat_c[i] = mesh->mat_c[i];
  if (mesh->elem_params)
    m.eparams.assign(mesh->elem_params, mesh->elem_params + 2 * (size_t)mesh->n_elems);
  c->precision = precision;
  *out = c;
  return NLA3D_OK;
}

int nla3d_destroy(nla3d_ctx* c) {
  if (!c) return NLA3D_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void* p : c->allocs) cudaFree(p);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->allocs.clear();
  for (auto& v : c->ev) cudaEventDestroy(v);
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
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return NLA3D_OK;
}

void* nla3d_get_stream(const nla3d_ctx* c) { return c ? (void*)c->stream : nullptr; }

int nla3d_add_fix(nla3d_ctx* c, uint32_t n, const uint32_t* nodes, const int32_t* dofs) {
  if (!c || c->host_ready || (n && (!nodes || !dofs))) return fail(c, NLA3D_ERR_ARG, "add_fix");
  for (uint32_t i = 0; i < n; i++) {
    c->hm.fix_node.push_back(nodes[i]);
    c->hm.fix_dof.push_back(dofs[i]);
  }
  return NLA3D_OK;
}

int nla3d_add_rigid_body(nla3d_ctx* c, uint32_t master, uint32_t n_slaves, const uint32_t* slaves,
                         uint32_t n_dofs, const int32_t* dofs) {
  if (!c || c->host_ready || n_dofs > 3 || (n_slaves && !slaves) || (n_dofs && !dofs))
    return fail(c, NLA3D_ERR_ARG, "add_rigid_body");
  RigidBody rb;
  rb.master = master;
  rb.slaves.assign(slaves, slaves + n_slaves);
  rb.dofs.assign(dofs, dofs + n_dofs);
  c->hm.rbs.push_back(rb);
  return NLA3D_OK;
}

int nla3d_build_pattern(nla3d_ctx* c) {
  if (!c) return NLA3D_ERR_ARG;
  if (c->host_ready) return NLA3D_OK;
  std::string msg = build_host_model(c->hm, 0);
  if (!msg.empty()) return fail(c, msg.find("2^32") != std::string::npos ||
                                           msg.find("too many") != std::string::npos
                                       ? NLA3D_ERR_RANGE
                                       : NLA3D_ERR_PATTERN,
                                msg);
  c->host_ready = true;
  return NLA3D_OK;
}

int nla3d_slot_maps(const nla3d_ctx* c, uint32_t* kslot, uint32_t* fslot) {
  if (!c || !c->host_ready || c->ready) return NLA3D_ERR_ARG;
  if (kslot && !c->hm.kslot.empty())
    std::memcpy(kslot, c->hm.kslot.data(), sizeof(uint32_t) * c->hm.kslot.size());
  if (fslot && !c->hm.fslot.empty())
    std::memcpy(fslot, c->hm.fslot.data(), sizeof(uint32_t) * c->hm.fslot.size());
  return NLA3D_OK;
}

int nla3d_init_solution_data(nla3d_ctx* c) {
  if (!c || c->ready) return fail(c, NLA3D_ERR_ARG, "init_solution_data: bad call order");
  int rc = nla3d_build_pattern(c);
  if (rc) return rc;
  HostModel& m = c->hm;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetDevice");
  if (!c->stream) {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamCreate");
    c->own_stream = true;
  }
  const uint64_t E = m.n_elems, N = m.n_nodes, ntot = m.n_total();
  // node equations of UX, UY, UZ (TEMP for QUADTH is handled by the linear kernel's
  // slot maps only), padded to 4 per node for 16-byte loads
  std::vector<uint32_t> neq3(4 * N, 0);
  for (uint64_t n = 0; n < N; n++)
    for (int d = 0; d < 3; d++) neq3[4 * n + d] = m.node_eq[n * kDofTypes + d];
  std::vector<uint32_t> peq(E, 0);
  for (uint64_t el = 0; el < E; el++) peq[el] = m.elem_eq[el * kDofTypes + HYDRO_PRESSURE];

#define CK(x)                                    \
  do {                                           \
    cudaError_t _e = (x);                        \
    if (_e != cudaSuccess) return cuda_fail(c, _e, #x); \
  } while (0)
  CK(upload(c, &c->d_xyz, m.xyz.data(), m.xyz.size()));
  CK(upload(c, &c->d_conn, m.conn.data(), m.conn.size()));
  CK(upload(c, &c->d_node_eq3, neq3.data(), neq3.size()));
  CK(upload(c, &c->d_p_eq, peq.data(), peq.size()));
  if (!m.eparams.empty()) CK(upload(c, &c->d_eparams, m.eparams.data(), m.eparams.size()));
  CK(upload(c, &c->d_kptr, m.k_ptr.data(), m.k_ptr.size()));
  CK(upload(c, &c->d_kids, m.k_ids.data(), m.k_ids.size()));
  CK(upload(c, &c->d_fptr, m.f_ptr.data(), m.f_ptr.size()));
  CK(upload(c, &c->d_fids, m.f_ids.data(), m.f_ids.size()));
  CK(dalloc(c, &c->d_U, ntot));
  CK(dalloc(c, &c->d_Ustate, ntot));
  CK(cudaMemsetAsync(c->d_U, 0, sizeof(double) * ntot, c->stream));
  CK(cudaMemsetAsync(c->d_Ustate, 0, sizeof(double) * ntot, c->stream));
  CK(dalloc(c, &c->d_contribK, E * m.n_kc));
  CK(dalloc(c, &c->d_contribF, E * (m.n_fc ? m.n_fc : 1)));
  CK(dalloc(c, &c->d_K, m.nnz_total));
  CK(dalloc(c, &c->d_F, ntot));
  CK(dalloc(c, &c->d_status, 1));
  if (m.n_mpc) {
    // per MPC: master, slave, eq, slave_eq, master_eq6[6], slot[5]  (15 words)
    std::vector<uint32_t> w(15ull * m.n_mpc);
    std::vector<int32_t> dof(m.n_mpc);
    const uint64_t M = m.n_mpc;
    for (uint64_t k = 0; k < M; k++) {
      const MpcEq& q = m.mpcs[k];
      w[k] = q.node[1];
      w[M + k] = q.slave;
      w[2 * M + k] = q.eq;
      w[3 * M + k] = m.neq(q.slave, q.slave_dof);
      for (int t = 0; t < 6; t++) w[4 * M + 6 * k + t] = m.neq(q.node[1], t);
      for (int t = 0; t < 5; t++) w[10 * M + 5 * k + t] = m.mpc_slot[5 * k + t];
      dof[k] = q.slave_dof;
    }
    // the MPC kernel adds each coefficient to its slot; slots are distinct by
    // construction (one column per MPC equation), verify before trusting it
    std::vector<uint32_t> sl(m.mpc_slot);
    std::sort(sl.begin(), sl.end());
    if (std::adjacent_find(sl.begin(), sl.end()) != sl.end())
      return fail(c, NLA3D_ERR_PATTERN, "two MPC terms share one K slot");
    CK(upload(c, &c->d_mpc_u32, w.data(), w.size()));
    CK(upload(c, &c->d_mpc_dof, dof.data(), dof.size()));
  }
  if (m.etype == NLA3D_SOLID81) {
    CK(dalloc(c, &c->d_Gt, 24 * 8 * E));
    CK(dalloc(c, &c->d_wdet, 8 * E));
    CK(cudaMemsetAsync(c->d_status, 0, sizeof(ElementStatus), c->stream));
    CK(cudaMemsetAsync(&c->d_status->first, 0xFF, sizeof(uint32_t), c->stream));
    JacobianArgs ja{(uint32_t)E, c->d_xyz, c->d_conn, c->d_Gt, c->d_wdet, c->d_status};
    CK(launch_solid81_jacobian(ja, c->stream));
    c->launches++;
  }
  CK(cudaStreamSynchronize(c->stream));
  // the gather lists now live on the device only
  std::vector<uint32_t>().swap(m.kslot);
  std::vector<uint32_t>().swap(m.fslot);
  std::vector<uint32_t>().swap(m.k_ids);
  std::vector<uint32_t>().swap(m.f_ids);
  std::vector<uint32_t>().swap(m.k_ptr);
  std::vector<uint32_t>().swap(m.f_ptr);
  c->ready = true;
  return NLA3D_OK;
}

int nla3d_info(const nla3d_ctx* c, uint32_t out[16]) {
  if (!c || !out || !c->host_ready) return NLA3D_ERR_ARG;
  const HostModel& m = c->hm;
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
  return NLA3D_OK;
}

int nla3d_pattern(const nla3d_ctx* c, int block, uint32_t* iofeir, uint32_t* columns) {
  const int b = block_slot(block);
  if (!c || !c->host_ready || b < 0 || !iofeir) return NLA3D_ERR_ARG;
  const CsrBlock& B = c->hm.blk[b];
  std::memcpy(iofeir, B.iofeir.data(), sizeof(uint32_t) * (B.rows + 1));
  if (B.nnz()) {
    if (!columns) return NLA3D_ERR_ARG;
    std::memcpy(columns, B.columns.data(), sizeof(uint32_t) * B.nnz());
  }
  return NLA3D_OK;
}

int nla3d_eq_numbers(const nla3d_ctx* c, uint32_t* node_eq, uint32_t* elem_eq) {
  if (!c || !c->host_ready) return NLA3D_ERR_ARG;
  if (node_eq) std::memcpy(node_eq, c->hm.node_eq.data(), sizeof(uint32_t) * c->hm.node_eq.size());
  if (elem_eq) std::memcpy(elem_eq, c->hm.elem_eq.data(), sizeof(uint32_t) * c->hm.elem_eq.size());
  return NLA3D_OK;
}

int nla3d_set_U(nla3d_ctx* c, const double* U, uint64_t n) {
  if (!c || !c->ready || !U || n != c->hm.n_total()) return fail(c, NLA3D_ERR_ARG, "set_U size");
  cudaError_t e = cudaMemcpyAsync(c->d_U, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "set_U");
}

int nla3d_set_U_device(nla3d_ctx* c, const double* U, uint64_t n) {
  if (!c || !c->ready || !U || n != c->hm.n_total()) return fail(c, NLA3D_ERR_ARG, "set_U size");
  cudaError_t e =
      cudaMemcpyAsync(c->d_U, U, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "set_U_device");
}

int nla3d_update_results(nla3d_ctx* c) {
  if (!c || !c->ready) return fail(c, NLA3D_ERR_ARG, "update_results before init");
  // SOLID81 keeps its Gauss-point state as a snapshot of vecU; the linear
  // elements have no state on the assembly path.
  cudaError_t e = cudaMemcpyAsync(c->d_Ustate, c->d_U, sizeof(double) * c->hm.n_total(),
                                  cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "update_results");
  c->have_state = true;
  return NLA3D_OK;
}

int nla3d_assemble(nla3d_ctx* c) {
  if (!c || !c->ready) return fail(c, NLA3D_ERR_ARG, "assemble before init");
  HostModel& m = c->hm;
  cudaError_t e;
  e = cudaMemsetAsync(c->d_status, 0, sizeof(ElementStatus), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(&c->d_status->first, 0xFF, sizeof(uint32_t), c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble: status reset");
  const uint64_t slot = (c->timed % nla3d_ctx::kRing) * 5;
  auto mark = [&](int i) {
    if (c->timing) cudaEventRecord(c->ev[slot + i], c->stream);
  };
  mark(0);
  if (m.etype == NLA3D_SOLID81) {
    Solid81Args a{};
    a.n_elems = m.n_elems;
    a.Gt = c->d_Gt;
    a.wdet = c->d_wdet;
    a.conn = c->d_conn;
    a.node_eq3 = c->d_node_eq3;
    a.p_eq = c->d_p_eq;
    a.U_state = c->d_Ustate;
    a.U_cur = c->d_U;
    a.have_state = c->have_state ? 1 : 0;
    a.mat_id = m.mat_id;
    for (int i = 0; i < 5; i++) a.mc[i] = m.mat_c[i];
    a.kbulk = m.mat_id == NLA3D_MAT_NEO_HOOKEAN ? m.mat_c[1]
                                                : (m.mat_id == NLA3D_MAT_BIDERMAN ? m.mat_c[4]
                                                                                  : m.mat_c[2]);
    a.contribK = c->d_contribK;
    a.contribF = c->d_contribF;
    a.status = c->d_status;
    e = launch_solid81(a, c->precision == NLA3D_PREC_MIXED, 0, c->stream);
  } else {
    LinearArgs a{m.etype, m.n_elems, c->d_xyz, c->d_conn, c->d_eparams, c->d_contribK,
                 c->d_contribF, c->d_status};
    e = launch_linear(a, c->stream);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble: element kernel");
  c->launches++;
  mark(1);
  GatherArgs gk{m.nnz_total, c->d_kptr, c->d_kids, c->d_contribK, c->d_K};
  e = launch_gather(gk, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble: K gather");
  c->launches += m.nnz_total ? 1 : 0;
  mark(2);
  GatherArgs gf{m.n_total(), c->d_fptr, c->d_fids, c->d_contribF, c->d_F};
  e = launch_gather(gf, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "assemble: F gather");
  c->launches++;
  mark(3);
  if (m.n_mpc) {
    const uint64_t M = m.n_mpc;
    MpcArgs a{};
    a.n_mpc = m.n_mpc;
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
    if (e != cudaSuccess) return cuda_fail(c, e, "assemble: MPC rows");
    c->launches++;
  }
  mark(4);
  if (c->timing) c->timed++;
  return NLA3D_OK;
}

int nla3d_get_K(nla3d_ctx* c, int block, double* values) {
  const int b = block_slot(block);
  if (!c || !c->ready || b < 0) return fail(c, NLA3D_ERR_ARG, "get_K");
  const uint64_t n = c->hm.blk[b].nnz();
  if (!n) return NLA3D_OK;
  if (!values) return fail(c, NLA3D_ERR_ARG, "get_K: null output");
  cudaError_t e = cudaMemcpyAsync(values, c->d_K + c->hm.val_off[b], sizeof(double) * n,
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "get_K");
}

int nla3d_get_F(nla3d_ctx* c, double* F) {
  if (!c || !c->ready || !F) return fail(c, NLA3D_ERR_ARG, "get_F");
  cudaError_t e = cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->hm.n_total(),
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? NLA3D_OK : cuda_fail(c, e, "get_F");
}

int nla3d_device_K(const nla3d_ctx* c, int block, double** values, uint64_t* n) {
  const int b = block_slot(block);
  if (!c || !c->ready || b < 0 || !values || !n) return NLA3D_ERR_ARG;
  *values = c->d_K + c->hm.val_off[b];
  *n = c->hm.blk[b].nnz();
  return NLA3D_OK;
}

int nla3d_device_F(const nla3d_ctx* c, double** F, uint64_t* n) {
  if (!c || !c->ready || !F || !n) return NLA3D_ERR_ARG;
  *F = c->d_F;
  *n = c->hm.n_total();
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
