// A C++ program written against the reference's FEStorage interface, on the
// GB300 library (include/nla3d_fe_storage.hpp): it reads a model from a text
// file, builds it with createNodes / createElements / setConstrainedNodeDof /
// addMpc / addMpcCollection, runs initSolutionData, writes vecU, calls
// updateResults and assembleGlobalEqMatrices, and prints the numbering, the
// three CSR blocks of getK() and getF() (%.17g, so the values read back
// exactly).  With "pattern" as the third argument it stops after the host
// set-up (no GPU needed) and prints zero values; with "order" it also prints
// fillReducingOrder (host only); with "solve" it then solves K(2) x = F(2)
// with DeviceEquationSolver (EquationSolver::solveEquations) and prints x.
//
// Input (whitespace separated):
//   elem_type n_nodes n_elems mat_id c0 c1 c2 c3 c4 n_params
//   n_nodes x y z;  n_elems x (nodes..., params...)
//   n_fix (node dof)...;  n_mpc (n_terms b (node dof coef)...)...
//   n_rigid (master n_slaves n_dofs slaves... dofs...)...
//   n_U U...;  update_flag
#include <cstdio>
#include <fstream>
#include <string>

#include "nla3d_fe_storage.hpp"

using namespace nla3d_gb300;

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s model.txt out.txt [pattern]\n", argv[0]);
    return 2;
  }
  const std::string mode = argc > 3 ? argv[3] : "";
  const bool pattern_only = mode == "pattern" || mode == "order";
  std::ifstream in(argv[1]);
  int etype, mat_id, n_params;
  uint32_t n_nodes, n_elems;
  double c[5];
  in >> etype >> n_nodes >> n_elems >> mat_id >> c[0] >> c[1] >> c[2] >> c[3] >> c[4] >> n_params;
  FEStorage storage(NLA3D_PREC_FP64);
  auto nind = storage.createNodes(n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) {
    Node& nd = storage.getNode(nind[i]);
    in >> nd.pos[0] >> nd.pos[1] >> nd.pos[2];
  }
  auto eind = storage.createElements(n_elems, (ElementType)etype);
  for (uint32_t e = 0; e < n_elems; e++) {
    Element& el = storage.getElement(eind[e]);
    for (uint16_t j = 0; j < el.getNNodes(); j++) in >> el.getNodeNumber(j);
    for (int k = 0; k < n_params; k++) in >> el.params[k];
  }
  if (mat_id > 0) storage.setMaterial(mat_id, {c[0], c[1], c[2], c[3], c[4]});
  uint32_t n_fix;
  in >> n_fix;
  for (uint32_t i = 0; i < n_fix; i++) {
    uint32_t node;
    int dof;
    in >> node >> dof;
    storage.setConstrainedNodeDof(node, (Dof::dofType)dof);
  }
  uint32_t n_mpc;
  in >> n_mpc;
  for (uint32_t k = 0; k < n_mpc; k++) {
    uint32_t nt;
    Mpc mpc;
    in >> nt >> mpc.b;
    for (uint32_t t = 0; t < nt; t++) {
      MpcTerm term;
      int dof;
      in >> term.node >> dof >> term.coef;
      term.node_dof = (Dof::dofType)dof;
      mpc.eq.push_back(term);
    }
    storage.addMpc(mpc);
  }
  uint32_t n_rigid;
  in >> n_rigid;
  for (uint32_t k = 0; k < n_rigid; k++) {
    RigidBodyMpc rb;
    uint32_t ns, nd;
    in >> rb.masterNode >> ns >> nd;
    rb.slaveNodes.resize(ns);
    for (auto& s : rb.slaveNodes) in >> s;
    for (uint32_t q = 0; q < nd; q++) {
      int dof;
      in >> dof;
      rb.dofs.push_back((Dof::dofType)dof);
    }
    storage.addMpcCollection(rb);
  }
  try {
    if (pattern_only)
      storage.buildPattern();
    else
      storage.initSolutionData();
    uint64_t nU;
    int update;
    in >> nU;
    std::vector<double> U(nU);
    for (auto& v : U) in >> v;
    in >> update;
    if (!pattern_only) {
      if (U.size() != storage.getU().size()) throw Error(NLA3D_ERR_ARG, "vecU size");
      storage.getU() = U;
      if (update) storage.updateResults();
      storage.assembleGlobalEqMatrices();
    }
  } catch (const Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  FILE* out = std::fopen(argv[2], "w");
  std::fprintf(out, "%u %u %u %u\n", storage.nDofs(), storage.nConstrainedDofs(),
               storage.nUnknownDofs(), storage.nMpc());
  for (uint32_t n = 1; n <= storage.nNodes(); n++)
    for (int d = 0; d < 8; d++) std::fprintf(out, "%u ", storage.getNodeDofEqNumber(n, (Dof::dofType)d));
  std::fprintf(out, "\n");
  for (uint32_t e = 1; e <= storage.nElements(); e++)
    for (int d = 0; d < 8; d++)
      std::fprintf(out, "%u ", storage.getElementDofEqNumber(e, (Dof::dofType)d));
  std::fprintf(out, "\n");
  SparseBlock* blocks[3] = {storage.getK()->block(1), storage.getK()->block(1, 2),
                            storage.getK()->block(2)};
  for (SparseBlock* b : blocks) {
    std::fprintf(out, "%u %u %u\n", b->nRows(), b->nColumns(), b->nValues());
    for (uint32_t i = 0; i <= b->nRows(); i++) std::fprintf(out, "%u ", b->getIofeirArray()[i]);
    std::fprintf(out, "\n");
    for (uint32_t q = 0; q < b->nValues(); q++) std::fprintf(out, "%u ", b->getColumnsArray()[q]);
    std::fprintf(out, "\n");
    for (uint32_t q = 0; q < b->nValues(); q++) std::fprintf(out, "%.17g ", b->getValuesArray()[q]);
    std::fprintf(out, "\n");
  }
  std::fprintf(out, "%zu\n", storage.getF().size());
  for (double v : storage.getF()) std::fprintf(out, "%.17g ", v);
  std::fprintf(out, "\n");
  try {
    if (mode == "order") {
      const std::vector<int32_t> order = fillReducingOrder(storage);
      std::fprintf(out, "%zu\n", order.size());
      for (int32_t r : order) std::fprintf(out, "%d ", r);
      std::fprintf(out, "\n");
    } else if (mode == "solve") {
      DeviceEquationSolver solver(storage, DeviceEquationSolver::FP64);
      const uint32_t nc = storage.nConstrainedDofs();
      const std::vector<double>& F = storage.getF();
      std::vector<double> x(solver.nRows());
      solver.solveEquations(F.data() + nc, x.data());
      std::fprintf(out, "%zu %d %.3e\n", x.size(), solver.refinementSteps(),
                   solver.relativeResidual());
      for (double v : x) std::fprintf(out, "%.17g ", v);
      std::fprintf(out, "\n");
    }
  } catch (const Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    std::fclose(out);
    return 1;
  }
  std::fclose(out);
  return 0;
}
