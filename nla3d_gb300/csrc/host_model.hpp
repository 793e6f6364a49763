// Host-side model of the assembly path: DoF tables, equation numbering, the
// block CSR pattern of K, and the element -> CSR slot maps with their
// fixed-order gather lists.  Everything here is integer work done once per
// mesh (the reference's FEStorage::initDofs / assignEquationNumbers /
// initSolutionData, FEStorage.cpp:338-550).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace nla3d_gpu {

constexpr int kDofTypes = 8;  // Dof::numberOfDofTypes (Dof.h:15-25)
constexpr int kElemParams = 4;  // per-element parameters stored per element
constexpr int kLineKc = 3;      // K contributions of a SurfaceLINETH line
constexpr int kLineFc = 2;      // F contributions of a SurfaceLINETH line
enum DofType { UX = 0, UY, UZ, ROTX, ROTY, ROTZ, HYDRO_PRESSURE, TEMP };
enum ElemType { PLANE41 = 1, SOLID81 = 2, TETRA0 = 3, QUADTH = 5 };

struct RigidBody {
  uint32_t master = 0;
  std::vector<uint32_t> slaves;
  std::vector<int> dofs;
  uint32_t first_mpc = 0;
};

// One MPC equation of a rigid body (Mpc.cpp:52-68): 5 terms.
struct MpcEq {
  uint32_t eq = 0;
  uint32_t node[5];
  int dof[5];
  uint32_t rb = 0;       // owning rigid body
  uint32_t slave = 0;    // slave node
  int slave_dof = 0;     // UX/UY/UZ of this equation
};

// A linear MPC equation added by the caller (Mpc, Mpc.h:31-36, through
// FEStorage::addMpc, FEStorage.cpp:175-179): sum_t coef_t u(node_t, dof_t) = b.
// Its equation is numbered after the DoFs and before the rigid-body MPCs
// (those are registered later, in initDofs, FEStorage.cpp:351-354).
struct LinearMpc {
  std::vector<uint32_t> node;
  std::vector<int> dof;
  std::vector<double> coef;
  double b = 0.0;
  uint32_t eq = 0;
};

// 1-based 3-array CSR block (SparseMatrix.h:53-69).
struct CsrBlock {
  uint32_t rows = 0, cols = 0;
  std::vector<uint32_t> iofeir;   // rows + 1, iofeir[0] = 1
  std::vector<uint32_t> columns;  // nnz, 1-based, sorted per row
  uint64_t nnz() const { return columns.size(); }
};

struct HostModel {
  // mesh
  int etype = SOLID81;
  int npe = 8;        // nodes per element
  int nodal_dofs = 3; // DoFs per node used by the element (3 solids, 2 PLANE41, 1 QUADTH)
  uint32_t n_nodes = 0, n_elems = 0;
  std::vector<double> xyz;
  std::vector<uint32_t> conn;
  int mat_id = 0;
  double mat_c[5] = {0, 0, 0, 0, 0};
  std::vector<double> eparams;  // kElemParams per element: TETRA0 (E, my, 0, 0),
                                // QUADTH (k, volFlux, rho, c)
  // SurfaceLINETH line elements of a QUADTH mesh (QUADTH.cpp:70-125), created
  // after the quads: 2 node ids and (htc, flux, etemp0, etemp1) per line
  std::vector<uint32_t> line_conn;
  std::vector<double> line_par;
  // constraints and MPC
  std::vector<uint32_t> fix_node;
  std::vector<int> fix_dof;
  std::vector<RigidBody> rbs;
  std::vector<MpcEq> mpcs;        // rigid-body MPC equations
  std::vector<LinearMpc> lmpcs;   // linear MPC equations (numbered first)
  // DoF tables
  std::vector<uint8_t> node_mask, elem_mask, node_fix;
  std::vector<uint32_t> node_eq, elem_eq;  // (entity, type) -> eq, 0 = unused
  uint32_t n_dofs = 0, n_con = 0, n_unk = 0, n_mpc = 0;
  // K pattern: blk[0] = block(1), blk[1] = block(1,2), blk[2] = block(2)
  CsrBlock blk[3];
  uint64_t val_off[3] = {0, 0, 0};  // offsets of each block in the concatenated values
  uint64_t nnz_total = 0;
  // element contributions: per element n_kc K values then n_fc F values
  int n_kc = 0, n_fc = 0;
  // gather lists: slot s of the concatenated K values sums contributions
  // k_ids[k_ptr[s] .. k_ptr[s+1]) (element-ascending, local order within an
  // element: the reference's own summation order, FEStorage.cpp:36 +
  // SOLID81.h:62-93); F row r likewise with f_ptr / f_ids.
  std::vector<uint32_t> kslot, fslot;  // element -> slot maps (freed after upload)
  std::vector<uint32_t> k_ptr, k_ids;
  std::vector<uint32_t> f_ptr, f_ids;
  // rigid-body MPC term slots (mpcs.size() * 5) and linear MPC term slots
  // (all terms, equation by equation) in the concatenated K values
  std::vector<uint32_t> mpc_slot;
  std::vector<uint32_t> lmpc_slot;

  uint32_t n_total() const { return n_dofs + n_mpc; }
  uint32_t n_lines() const { return (uint32_t)(line_conn.size() / 2); }
  uint32_t neq(uint32_t node, int t) const { return node_eq[(size_t)(node - 1) * kDofTypes + t]; }
  uint32_t eeq(uint32_t el, int t) const { return elem_eq[(size_t)(el - 1) * kDofTypes + t]; }
};

// Build DoF tables, numbering, pattern, slot maps.  Returns "" on success,
// else a message.  n_threads <= 0 means "use the hardware concurrency".
std::string build_host_model(HostModel& m, int n_threads);
// The two halves of build_host_model: DoF registration, constraints and
// equation numbers; then incidence, CSR pattern, slot maps and gather lists
// (and the MPC term slots).
std::string build_host_numbering(HostModel& m);
std::string build_host_pattern(HostModel& m, int n_threads);
// MPC equations per (node, dof): mpc_eqs[mpc_ptr[k] .. mpc_ptr[k+1]) for
// k = (node - 1) * kDofTypes + dof, ascending (may repeat).
void mpc_extras(const HostModel& m, std::vector<uint32_t>& mpc_ptr,
                std::vector<uint32_t>& mpc_eqs);
// (eq_i, eq_j) -> index in the concatenated K values of this mesh.
bool host_slot_of(const HostModel& m, uint32_t i, uint32_t j, uint32_t* out);
// MPC term slots from the pattern in m.blk.
std::string host_mpc_slots(HostModel& m);

// Local contribution layout of one element in the reference's assembly order:
// for contribution c < n_kc, the (row entity dof, col entity dof) pair.
// entity >= 0 is the element-local node index; entity == -1 the element's own
// DoF (HYDRO_PRESSURE).
struct LocalPair {
  int8_t ei, ti, ej, tj;
};
std::vector<LocalPair> element_k_layout(int etype);
std::vector<LocalPair> element_f_layout(int etype);

}  // namespace nla3d_gpu
