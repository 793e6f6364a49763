// C++ host side of the GB300 assembly: the reference's FEStorage interface
// (FEStorage.h:38-378) over the C ABI of nla3d_gpu.h, header-only.
//
// A program written against nla3d's FEStorage builds its model the same way
// (createNodes / createElements, node positions, element node numbers, the
// material, constrained DoFs, Mpc equations and RigidBodyMpc collections),
// then calls initSolutionData(), and per iteration writes vecU (getU()),
// updateResults() and assembleGlobalEqMatrices(); getK()->block(1) /
// block(1, 2) / block(2) and getF() hold the reference's arrays afterwards
// (1-based upper CSR per block, values in the reference's order).
//
// Differences, by design: the reference's initDofs / assignEquationNumbers /
// initSolutionData sequence is the single initSolutionData() here (the
// numbering is the reference's); a failing call throws nla3d_gb300::Error
// carrying the library's message where the reference aborts (LOG(FATAL),
// assert); the element types are the four of the assembly path.
#pragma once

#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <algorithm>
#include <vector>

#include "nla3d_gpu.h"

namespace nla3d_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
  int code;
};

// ElementType codes of the reference (sys.h:151-163)
enum class ElementType : int32_t {
  PLANE41 = NLA3D_PLANE41,
  SOLID81 = NLA3D_SOLID81,
  TETRA0 = NLA3D_TETRA0,
  QUADTH = NLA3D_QUADTH
};

// Dof::dofType (Dof.h:15-25)
struct Dof {
  enum dofType : int32_t {
    UX = NLA3D_UX, UY = NLA3D_UY, UZ = NLA3D_UZ, ROTX = NLA3D_ROTX, ROTY = NLA3D_ROTY,
    ROTZ = NLA3D_ROTZ, HYDRO_PRESSURE = NLA3D_HYDRO_PRESSURE, TEMP = NLA3D_TEMP
  };
};

struct Node {
  double pos[3] = {0.0, 0.0, 0.0};
};

// one element: its node numbers (1-based) and, for TETRA0 / QUADTH, the
// element constants the reference keeps as members (TETRA0: E, my; QUADTH:
// k, volFlux, rho, c)
struct Element {
  std::vector<uint32_t> nodes;
  double params[4] = {0.0, 0.0, 0.0, 0.0};
  uint32_t& getNodeNumber(uint16_t i) { return nodes.at(i); }
  uint16_t getNNodes() const { return (uint16_t)nodes.size(); }
};

// Mpc / MpcTerm (Mpc.h:17-36): sum coef * u(node, node_dof) = b
struct MpcTerm {
  uint32_t node;
  Dof::dofType node_dof;
  double coef;
};
struct Mpc {
  std::vector<MpcTerm> eq;
  double b = 0.0;
};

// RigidBodyMpc (Mpc.h:51-61): the slaves follow the master's displacement and rotation
struct RigidBodyMpc {
  uint32_t masterNode = 0;
  std::vector<uint32_t> slaveNodes;
  std::vector<Dof::dofType> dofs;
};

// one CSR block (SparseMatrix.h:206-221 accessors)
class SparseBlock {
 public:
  uint32_t nRows() const { return rows_; }
  uint32_t nColumns() const { return cols_; }
  uint32_t nValues() const { return (uint32_t)columns_.size(); }
  double* getValuesArray() { return values_.data(); }
  uint32_t* getColumnsArray() { return columns_.data(); }
  uint32_t* getIofeirArray() { return iofeir_.data(); }
  // value at the 1-based (i, j); 0 for a structural zero
  double value(uint32_t i, uint32_t j) const {
    for (uint32_t q = iofeir_[i - 1] - 1; q < iofeir_[i] - 1; q++)
      if (columns_[q] == j) return values_[q];
    return 0.0;
  }

 private:
  friend class FEStorage;
  uint32_t rows_ = 0, cols_ = 0;
  std::vector<uint32_t> iofeir_, columns_;
  std::vector<double> values_;
};

// BlockSparseSymMatrix<2> (BlockSparseMatrix.h:39-69): block(1), block(1, 2), block(2)
class BlockSparseSymMatrix {
 public:
  SparseBlock* block(int i) { return i == 1 ? &b_[0] : &b_[2]; }
  SparseBlock* block(int i, int j) { return (i == 1 && j == 2) ? &b_[1] : block(i); }

 private:
  friend class FEStorage;
  SparseBlock b_[3];
};

class FEStorage {
 public:
  explicit FEStorage(int precision = NLA3D_PREC_FP64) : precision_(precision) {}
  ~FEStorage() {
    if (ctx_) nla3d_destroy(ctx_);
  }
  FEStorage(const FEStorage&) = delete;
  FEStorage& operator=(const FEStorage&) = delete;

  // ---- model (before initSolutionData) ----
  std::vector<uint32_t> createNodes(uint32_t n) {
    std::vector<uint32_t> ids(n);
    for (uint32_t i = 0; i < n; i++) {
      nodes_.emplace_back();
      ids[i] = (uint32_t)nodes_.size();
    }
    return ids;
  }
  std::vector<uint32_t> createElements(uint32_t n, ElementType type) {
    if (!elements_.empty() && type != type_) throw Error(NLA3D_ERR_ARG, "one element type per storage");
    type_ = type;
    const uint16_t npe = type == ElementType::SOLID81 ? 8 : 4;
    std::vector<uint32_t> ids(n);
    for (uint32_t i = 0; i < n; i++) {
      elements_.emplace_back();
      elements_.back().nodes.assign(npe, 0);
      ids[i] = (uint32_t)elements_.size();
    }
    return ids;
  }
  Node& getNode(uint32_t n) { return nodes_.at(n - 1); }
  Element& getElement(uint32_t e) { return elements_.at(e - 1); }
  uint32_t nNodes() const { return (uint32_t)nodes_.size(); }
  uint32_t nElements() const { return (uint32_t)elements_.size(); }
  // the material (MaterialFactory ids; constants in the reference's order)
  void setMaterial(int32_t mat_id, std::initializer_list<double> constants) {
    mat_id_ = mat_id;
    mat_c_.assign(constants.begin(), constants.end());
  }
  void setConstrainedNodeDof(uint32_t node, Dof::dofType dof) {
    fix_nodes_.push_back(node);
    fix_dofs_.push_back(dof);
  }
  void addMpc(const Mpc& mpc) { mpcs_.push_back(mpc); }
  void addMpcCollection(const RigidBodyMpc& rb) { rigid_.push_back(rb); }

  // ---- set-up: initDofs + assignEquationNumbers + initSolutionData ----
  void initSolutionData() { setup(true); }
  // the host half only (numbering and pattern; needs no GPU): getK() has the
  // pattern, values are zero
  void buildPattern() { setup(false); }

  uint32_t nDofs() const { return info_[0]; }
  uint32_t nConstrainedDofs() const { return info_[1]; }
  uint32_t nUnknownDofs() const { return info_[2]; }
  uint32_t nMpc() const { return info_[3]; }
  uint32_t getNodeDofEqNumber(uint32_t node, Dof::dofType dof) const {
    return node_eq_.at((size_t)(node - 1) * 8 + dof);
  }
  uint32_t getElementDofEqNumber(uint32_t el, Dof::dofType dof) const {
    return elem_eq_.at((size_t)(el - 1) * 8 + dof);
  }

  // ---- per iteration ----
  std::vector<double>& getU() { return U_; }
  std::vector<double>& getF() { return F_; }
  BlockSparseSymMatrix* getK() { return &K_; }
  double getNodeDofSolution(uint32_t node, Dof::dofType dof) const {
    return U_.at(getNodeDofEqNumber(node, dof) - 1);
  }
  void updateResults() {
    check(nla3d_set_U(ctx_, U_.data(), U_.size()));
    check(nla3d_update_results(ctx_));
  }
  // K and F into getK() / getF() (the element ranges' copies overlap the assembly)
  void assembleGlobalEqMatrices(int n_chunks = 8) {
    check(nla3d_set_U(ctx_, U_.data(), U_.size()));
    check(nla3d_assemble_to_host(ctx_, n_chunks, K_.b_[0].values_.data(), K_.b_[1].values_.data(),
                                 K_.b_[2].values_.data(), F_.data()));
  }
  // elements flagged by the last assembly (J <= 0 or non-finite): count, first
  std::pair<uint32_t, uint32_t> elementStatus() {
    uint32_t count = 0, first = 0;
    const int rc = nla3d_element_status(ctx_, &count, &first);
    if (rc != NLA3D_OK && rc != NLA3D_ERR_ELEMENT) check(rc);
    return {count, first};
  }
  nla3d_ctx* ctx() { return ctx_; }
  const std::vector<Mpc>& mpcs() const { return mpcs_; }
  const std::vector<RigidBodyMpc>& rigidBodies() const { return rigid_; }

 private:
  void check(int rc) const {
    if (rc != NLA3D_OK) {
      const char* msg = ctx_ ? nla3d_last_error(ctx_) : "";
      throw Error(rc, std::string("nla3d_gb300: ") + (msg && *msg ? msg : "call failed"));
    }
  }
  void setup(bool device) {
    if (!ctx_) create();
    check(device ? nla3d_init_solution_data(ctx_) : nla3d_build_pattern(ctx_));
    check(nla3d_info(ctx_, info_));
    const int ids[3] = {1, 12, 2};
    for (int b = 0; b < 3; b++) {
      SparseBlock& blk = K_.b_[b];
      blk.rows_ = info_[4 + 3 * b];
      blk.cols_ = info_[5 + 3 * b];
      blk.iofeir_.assign(blk.rows_ + 1, 1);
      blk.columns_.assign(info_[6 + 3 * b], 0);
      blk.values_.assign(info_[6 + 3 * b], 0.0);
      if (blk.rows_ || !blk.columns_.empty())
        check(nla3d_pattern(ctx_, ids[b], blk.iofeir_.data(), blk.columns_.data()));
    }
    node_eq_.assign((size_t)nodes_.size() * 8, 0);
    elem_eq_.assign((size_t)elements_.size() * 8, 0);
    check(nla3d_eq_numbers(ctx_, node_eq_.data(), elem_eq_.data()));
    U_.assign((size_t)info_[0] + info_[3], 0.0);
    F_.assign(U_.size(), 0.0);
  }
  void create() {
    std::vector<double> xyz(3 * nodes_.size());
    for (size_t i = 0; i < nodes_.size(); i++)
      for (int d = 0; d < 3; d++) xyz[3 * i + d] = nodes_[i].pos[d];
    std::vector<uint32_t> conn;
    std::vector<double> par;
    for (const Element& e : elements_) {
      conn.insert(conn.end(), e.nodes.begin(), e.nodes.end());
      par.insert(par.end(), e.params, e.params + 4);
    }
    nla3d_mesh_desc d{};
    d.elem_type = (int32_t)type_;
    d.n_nodes = (uint32_t)nodes_.size();
    d.n_elems = (uint32_t)elements_.size();
    d.xyz = xyz.data();
    d.conn = conn.data();
    d.mat_id = mat_id_;
    for (size_t i = 0; i < mat_c_.size() && i < 5; i++) d.mat_c[i] = mat_c_[i];
    const bool linear = type_ == ElementType::TETRA0 || type_ == ElementType::QUADTH;
    d.elem_params = linear ? par.data() : nullptr;
    d.n_elem_params = linear ? 4 : 0;
    if (type_ == ElementType::TETRA0) {   // TETRA0 takes (E, my)
      par2_.clear();
      for (const Element& e : elements_) par2_.insert(par2_.end(), e.params, e.params + 2);
      d.elem_params = par2_.data();
      d.n_elem_params = 2;
    }
    check(nla3d_create(&d, precision_, &ctx_));
    if (!fix_nodes_.empty())
      check(nla3d_add_fix(ctx_, (uint32_t)fix_nodes_.size(), fix_nodes_.data(), fix_dofs_.data()));
    for (const Mpc& m : mpcs_) {
      std::vector<uint32_t> n;
      std::vector<int32_t> dof;
      std::vector<double> c;
      for (const MpcTerm& t : m.eq) {
        n.push_back(t.node);
        dof.push_back(t.node_dof);
        c.push_back(t.coef);
      }
      check(nla3d_add_mpc(ctx_, (uint32_t)n.size(), n.data(), dof.data(), c.data(), m.b));
    }
    for (const RigidBodyMpc& rb : rigid_) {
      std::vector<int32_t> dofs(rb.dofs.begin(), rb.dofs.end());
      check(nla3d_add_rigid_body(ctx_, rb.masterNode, (uint32_t)rb.slaveNodes.size(),
                                 rb.slaveNodes.data(), (uint32_t)dofs.size(), dofs.data()));
    }
  }

  int precision_;
  nla3d_ctx* ctx_ = nullptr;
  ElementType type_ = ElementType::SOLID81;
  std::vector<Node> nodes_;
  std::vector<Element> elements_;
  int32_t mat_id_ = 0;
  std::vector<double> mat_c_;
  std::vector<uint32_t> fix_nodes_;
  std::vector<int32_t> fix_dofs_;
  std::vector<Mpc> mpcs_;
  std::vector<RigidBodyMpc> rigid_;
  std::vector<double> par2_;
  uint32_t info_[16] = {};
  std::vector<uint32_t> node_eq_, elem_eq_;
  std::vector<double> U_, F_;
  BlockSparseSymMatrix K_;
};

// ---- the equation solver on the device (EquationSolver.h:19-34) ----

// A fill-reducing order of K(2) for DeviceEquationSolver (order[new] = K(2)
// row, 0-based): a point per row (the node of a nodal DoF, the element's
// centroid for an element DoF, the first node of an MPC equation), then
// nla3d_ldlt_order: geometric nested dissection, the DoFs with a stored
// diagonal first, the MPC equations next, the DoFs without a diagonal (a
// rigid-body master) last, so that the factorisation needs no pivoting.
inline std::vector<int32_t> fillReducingOrder(FEStorage& s) {
  SparseBlock* K2 = s.getK()->block(2);
  const uint32_t n = K2->nRows();
  const uint32_t nc = s.nConstrainedDofs(), nu = s.nUnknownDofs();
  const uint32_t* io = K2->getIofeirArray();
  const uint32_t* co = K2->getColumnsArray();
  std::vector<double> pts(3 * (size_t)n, 0.0);
  auto place = [&](uint32_t eq, const double* p) {
    if (eq > nc && eq - nc - 1 < n)
      for (int d = 0; d < 3; d++) pts[3 * (size_t)(eq - nc - 1) + d] = p[d];
  };
  for (uint32_t v = 1; v <= s.nNodes(); v++)
    for (int32_t d = 0; d < 8; d++) place(s.getNodeDofEqNumber(v, (Dof::dofType)d), s.getNode(v).pos);
  for (uint32_t e = 1; e <= s.nElements(); e++) {
    Element& el = s.getElement(e);
    double c[3] = {0.0, 0.0, 0.0};
    for (uint32_t v : el.nodes)
      for (int d = 0; d < 3; d++) c[d] += s.getNode(v).pos[d] / (double)el.nodes.size();
    for (int32_t d = 0; d < 8; d++) place(s.getElementDofEqNumber(e, (Dof::dofType)d), c);
  }
  uint32_t k = 0;
  auto place_row = [&](uint32_t node) {
    if (nu + k < n)
      for (int d = 0; d < 3; d++) pts[3 * (size_t)(nu + k) + d] = s.getNode(node).pos[d];
    k++;
  };
  for (const Mpc& m : s.mpcs()) place_row(m.eq.at(0).node);
  for (const RigidBodyMpc& rb : s.rigidBodies())
    for (uint32_t v : rb.slaveNodes)
      for (size_t q = 0; q < rb.dofs.size(); q++) place_row(v);
  std::vector<int32_t> order(n);
  const int rc = nla3d_ldlt_order(n, io, co, pts.data(), nu, order.data());
  if (rc != NLA3D_OK) throw Error(rc, "nla3d_ldlt_order rejected the pattern");
  return order;
}

// EquationSolver (EquationSolver.h:19-34) on the device: the sparse LDL^T of
// K(2) (nla3d_ldlt_*) factored from the K values the last assembly left in
// HBM, solved with host vectors and refined in FP64.
class DeviceEquationSolver {
 public:
  enum Precision : int { FP64 = 0, FP32 = 1, FP32_TENSOR_CORES = 2 };
  // after s.initSolutionData(); order: K(2) rows in factor order (default
  // fillReducingOrder(s))
  explicit DeviceEquationSolver(FEStorage& s, int precision = FP64,
                                std::vector<int32_t> order = {})
      : s_(s) {
    SparseBlock* K2 = s.getK()->block(2);
    n_ = K2->nRows();
    if (order.empty()) order = fillReducingOrder(s);
    const int rc = nla3d_ldlt_create(n_, K2->getIofeirArray(), K2->getColumnsArray(), order.data(),
                                     precision, nullptr, &h_);
    if (rc != NLA3D_OK) {
      const std::string msg = h_ ? nla3d_ldlt_last_error(h_) : "";
      if (h_) nla3d_ldlt_destroy(h_);
      h_ = nullptr;
      throw Error(rc, "nla3d_ldlt_create: " + msg);
    }
  }
  ~DeviceEquationSolver() {
    if (h_) nla3d_ldlt_destroy(h_);
  }
  DeviceEquationSolver(const DeviceEquationSolver&) = delete;
  DeviceEquationSolver& operator=(const DeviceEquationSolver&) = delete;

  // factorizeEquations: the device K(2) of the storage's last assembly
  void factorizeEquations() { check(nla3d_ldlt_factor(h_, deviceK2())); }
  // substituteEquations: x = K(2)^-1 rhs (host vectors of nRows() doubles),
  // refined until ||rhs - K x|| <= tol ||rhs||
  void substituteEquations(const double* rhs, double* x, double tol = 1e-12, int max_refine = 50) {
    check(nla3d_ldlt_solve_host(h_, deviceK2(), rhs, x, max_refine, tol, &steps_, &residual_));
  }
  // solveEquations: both
  void solveEquations(const double* rhs, double* x) {
    factorizeEquations();
    substituteEquations(rhs, x);
  }
  uint32_t nRows() const { return (uint32_t)n_; }
  int refinementSteps() const { return steps_; }
  double relativeResidual() const { return residual_; }

 private:
  const double* deviceK2() {
    double* v = nullptr;
    uint64_t cnt = 0;
    check(nla3d_device_K(s_.ctx(), 2, &v, &cnt));
    return v;
  }
  void check(int rc) const {
    if (rc != NLA3D_OK) {
      const char* msg = h_ ? nla3d_ldlt_last_error(h_) : "";
      throw Error(rc, std::string("nla3d_gb300 equation solver: ") + (msg && *msg ? msg : "call failed"));
    }
  }
  FEStorage& s_;
  nla3d_ldlt* h_ = nullptr;
  int64_t n_ = 0;
  int steps_ = 0;
  double residual_ = 0.0;
};

}  // namespace nla3d_gb300
