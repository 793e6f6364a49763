// Harness around the COMPILED REFERENCE (nla3d sources built unmodified from
// the reference checkout by oracle/Makefile into oracle/_ref/).  Test
// infrastructure only: it lets the tests and the golden-fixture script drive
// the reference's own FEStorage / SOLID81 / TETRA0 / QUADTH / RigidBodyMpc code
// on synthetic meshes and read back its DoF numbering, CSR pattern, K and F,
// and have its VtkProcessor write the legacy VTK files of a state.
//
// It follows the reference's own set-up sequence:
//   createNodes / createElements        (main.cpp:189-205)
//   addMpcCollection(RigidBodyMpc)      (main.cpp:262-279)
//   initDofs, setConstrainedNodeDof,
//   assignEquationNumbers, initSolutionData   (FESolver.cpp:175, 221-226, 417)
// and the per-iteration pair updateResults() -> assembleGlobalEqMatrices()
// (FESolver.cpp:471 -> :446).
//
// Only SOLID81, TETRA0, QUADTH and PLANE41 are instantiated, so ElementFactory is
// provided here (the reference's factory also instantiates element types that
// are outside the assembly path and need the full third-party library).
#include <cstring>
#include <string>
#include <vector>

#include "FEStorage.h"
#include "Mpc.h"
#include "Node.h"
#include "VtkProcessor.h"
#include "elements/PLANE41.h"
#include "elements/QUADTH.h"
#include "elements/SOLID81.h"
#include "elements/TETRA0.h"
#include "materials/MaterialFactory.h"

using namespace nla3d;

namespace nla3d {
ElementType ElementFactory::elName2elType(std::string elName) {
  for (int i = 0; i < (int)ElementType::UNDEFINED; i++)
    if (elName == elTypeLabels[i]) return (ElementType)i;
  return ElementType::UNDEFINED;
}

void ElementFactory::createElements(ElementType elId, const uint32 n, std::vector<Element*>& ptr) {
  ptr.reserve(ptr.size() + n);
  for (uint32 i = 0; i < n; i++) {
    switch (elId) {
      case ElementType::SOLID81: ptr.push_back(new ElementSOLID81()); break;
      case ElementType::TETRA0: ptr.push_back(new ElementTETRA0()); break;
      case ElementType::QUADTH: ptr.push_back(new ElementQUADTH()); break;
      case ElementType::PLANE41: ptr.push_back(new ElementPLANE41()); break;
      case ElementType::SurfaceLINETH: ptr.push_back(new SurfaceLINETH()); break;
      default: LOG(FATAL) << "element type not built into the oracle harness";
    }
  }
}
}  // namespace nla3d

namespace {

struct RefModel {
  FEStorage storage;
  ElementType type = ElementType::UNDEFINED;
  unsigned n_model_elems = 0;  // the elements of ref_new; lines come after them
  std::vector<std::pair<uint32, int>> fixes;
  std::string err;
  double t_update = 0.0, t_assemble = 0.0;
};

template <class F>
int guarded(RefModel* m, F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    if (m) m->err = e.what();
    return 1;
  }
}

}  // namespace

extern "C" {

// elem_type: reference ElementType code (sys.h:151-163): 1 PLANE41, 2 SOLID81, 3 TETRA0,
//            5 QUADTH.
// mat_id: reference MaterialFactory::matId (MaterialFactory.h:12-18): 1 Neo-Hookean,
//         2 Biderman, 3 Mooney-Rivlin; 0 = no material (TETRA0 / QUADTH).
// elem_params: per element, n_elem_params doubles (missing ones are 0):
//              TETRA0 (E, my), QUADTH (k, volFlux, rho, c) (QUADTH.h:29-35).
void* ref_new(int elem_type, unsigned n_nodes, const double* xyz, unsigned n_elems,
              const unsigned* conn, int mat_id, const double* mat_c, int n_mat_c,
              const double* elem_params, int n_elem_params) {
  RefModel* m = new RefModel();
  int rc = guarded(m, [&] {
    m->type = (ElementType)elem_type;
    m->n_model_elems = n_elems;
    auto nind = m->storage.createNodes(n_nodes);
    for (unsigned i = 0; i < n_nodes; i++) {
      Node& nd = m->storage.getNode(nind[i]);
      nd.pos[0] = xyz[3 * i + 0];
      nd.pos[1] = xyz[3 * i + 1];
      nd.pos[2] = xyz[3 * i + 2];
    }
    auto eind = m->storage.createElements(n_elems, m->type);
    for (unsigned e = 0; e < n_elems; e++) {
      Element& el = m->storage.getElement(eind[e]);
      const unsigned nn = el.getNNodes();
      for (unsigned j = 0; j < nn; j++) el.getNodeNumber(j) = conn[e * nn + j];
      auto par = [&](int k) {
        return (elem_params && k < n_elem_params) ? elem_params[(size_t)e * n_elem_params + k]
                                                  : 0.0;
      };
      if (m->type == ElementType::TETRA0) {
        auto& t = dynamic_cast<ElementTETRA0&>(el);
        t.E = par(0);
        t.my = par(1);
      } else if (m->type == ElementType::QUADTH) {
        auto& q = dynamic_cast<ElementQUADTH&>(el);
        q.k = par(0);
        q.volFlux = par(1);
        q.rho = par(2);
        q.c = par(3);
      }
    }
    if (mat_id > 0) {
      Material* mat = MaterialFactory::createMaterial(MaterialFactory::matModelLabels[mat_id]);
      if (!mat) LOG(FATAL) << "bad material id";
      for (int i = 0; i < n_mat_c; i++) mat->Ci(i) = mat_c[i];
      m->storage.material = mat;
    }
  });
  if (rc) {
    delete m;
    return nullptr;
  }
  return m;
}

void ref_free(void* h) { delete static_cast<RefModel*>(h); }

const char* ref_error(void* h) { return static_cast<RefModel*>(h)->err.c_str(); }

int ref_add_fix(void* h, unsigned n, const unsigned* nodes, const int* dofs) {
  RefModel* m = static_cast<RefModel*>(h);
  for (unsigned i = 0; i < n; i++) m->fixes.emplace_back(nodes[i], dofs[i]);
  return 0;
}

int ref_add_rigid_body(void* h, unsigned master, unsigned n_slaves, const unsigned* slaves,
                       unsigned n_dofs, const int* dofs) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    RigidBodyMpc* mpc = new RigidBodyMpc;
    mpc->storage = &m->storage;
    mpc->masterNode = master;
    mpc->slaveNodes.assign(slaves, slaves + n_slaves);
    for (unsigned i = 0; i < n_dofs; i++) mpc->dofs.push_back((Dof::dofType)dofs[i]);
    m->storage.addMpcCollection(mpc);
  });
}

// FEStorage::addMpc with an Mpc built the way readCdbFile builds one from a
// CE record (FEReaders.cpp:549-573).
int ref_add_mpc(void* h, unsigned n_terms, const unsigned* nodes, const int* dofs,
                const double* coefs, double b) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    Mpc* mpc = new Mpc();
    mpc->b = b;
    for (unsigned t = 0; t < n_terms; t++)
      mpc->eq.push_back(MpcTerm(nodes[t], (Dof::dofType)dofs[t], coefs[t]));
    m->storage.addMpc(mpc);
  });
}

// SurfaceLINETH elements created after the model's elements (as a .cdb reader
// or a test would): conn 2 per line, htc, flux, etemp 2 per line.
int ref_add_surface_lines(void* h, unsigned n, const unsigned* conn, const double* htc,
                          const double* flux, const double* etemp) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    auto ind = m->storage.createElements(n, ElementType::SurfaceLINETH);
    for (unsigned l = 0; l < n; l++) {
      auto& el = dynamic_cast<SurfaceLINETH&>(m->storage.getElement(ind[l]));
      el.getNodeNumber(0) = conn[2 * l];
      el.getNodeNumber(1) = conn[2 * l + 1];
      el.htc = htc ? htc[l] : 0.0;
      el.flux = flux ? flux[l] : 0.0;
      el.etemp[0] = etemp ? etemp[2 * l] : 0.0;
      el.etemp[1] = etemp ? etemp[2 * l + 1] : 0.0;
    }
  });
}

int ref_set_transient(void* h, int on) {
  RefModel* m = static_cast<RefModel*>(h);
  m->storage.setTransient(on != 0);
  return 0;
}

int ref_setup(void* h) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    m->storage.initDofs();
    for (auto& f : m->fixes) m->storage.setConstrainedNodeDof(f.first, (Dof::dofType)f.second);
    m->storage.assignEquationNumbers();
    m->storage.initSolutionData();
  });
}

// out[0..3]  = nDofs, nConstrainedDofs, nUnknownDofs, nMpc
// out[4..12] = (rows, cols, nnz) of block(1), block(1,2), block(2)
void ref_info(void* h, unsigned* out) {
  RefModel* m = static_cast<RefModel*>(h);
  FEStorage& s = m->storage;
  out[0] = s.nDofs();
  out[1] = s.nConstrainedDofs();
  out[2] = s.nUnknownDofs();
  out[3] = s.nMpc();
  auto* K = s.getK();
  math::BaseSparseMatrix* blocks[3] = {K->block(1), K->block(1, 2), K->block(2)};
  for (int b = 0; b < 3; b++) {
    out[4 + 3 * b + 0] = blocks[b]->nRows();
    out[4 + 3 * b + 1] = blocks[b]->nColumns();
    out[4 + 3 * b + 2] = blocks[b]->nValues();
  }
}

static math::BaseSparseMatrix* pick_block(RefModel* m, int block) {
  auto* K = m->storage.getK();
  if (block == 1) return K->block(1);
  if (block == 2) return K->block(2);
  return K->block(1, 2);
}

// block: 1, 2, or 12 (= block(1,2)).  iofeir gets rows+1 entries, columns nnz.
int ref_pattern(void* h, int block, unsigned* iofeir, unsigned* columns) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    math::BaseSparseMatrix* B = pick_block(m, block);
    if (B->nRows() == 0 && B->nValues() == 0) return;
    std::memcpy(iofeir, B->getIofeirArray(), sizeof(unsigned) * (B->nRows() + 1));
    std::memcpy(columns, B->getColumnsArray(), sizeof(unsigned) * B->nValues());
  });
}

// Equation numbers per (entity, Dof::dofType) (Dof.h:15-25), 0 = DoF not used;
// elem_eq covers the elements of ref_new (surface lines carry no element DoF).
int ref_eq_numbers(void* h, unsigned* node_eq, unsigned* elem_eq) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    FEStorage& s = m->storage;
    for (uint32 n = 1; n <= s.nNodes(); n++)
      for (int t = 0; t < Dof::numberOfDofTypes; t++)
        node_eq[(n - 1) * 8 + t] = s.isNodeDofUsed(n, (Dof::dofType)t)
                                       ? s.getNodeDofEqNumber(n, (Dof::dofType)t) : 0;
    for (uint32 e = 1; e <= s.nElements() && e <= m->n_model_elems; e++)
      for (int t = 0; t < Dof::numberOfDofTypes; t++)
        elem_eq[(e - 1) * 8 + t] = s.isElementDofUsed(e, (Dof::dofType)t)
                                       ? s.getElementDofEqNumber(e, (Dof::dofType)t) : 0;
  });
}

int ref_set_U(void* h, const double* U, unsigned n) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    math::dVec* v = m->storage.getU();
    if (v->size() != n) LOG(FATAL) << "U size mismatch";
    for (unsigned i = 0; i < n; i++) (*v)[i] = U[i];
  });
}

int ref_update(void* h, double* seconds) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    auto& t = nla3d_shim::timers();
    t["updateSolutionResults"] = 0.0;
    m->storage.updateResults();
    if (seconds) *seconds = t["updateSolutionResults"];
  });
}

int ref_assemble(void* h, double* seconds) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    auto& t = nla3d_shim::timers();
    t["assembleGlobalEqMatrix"] = 0.0;
    m->storage.assembleGlobalEqMatrices();
    if (seconds) *seconds = t["assembleGlobalEqMatrix"];
  });
}

int ref_get_K(void* h, int block, double* values) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    math::BaseSparseMatrix* B = pick_block(m, block);
    if (B->nValues() == 0) return;
    std::memcpy(values, B->getValuesArray(), sizeof(double) * B->nValues());
  });
}

// y += coef * op(block) x with the reference's own sparse products
// (SparseMatrix.cpp:497-558): block 1 / 2 matBVprod(SparseSymMatrix&),
// block 12 trans 0 matBVprod(SparseMatrix&), trans 1 matBTVprod(SparseMatrix&).
int ref_block_mv(void* h, int block, int trans, const double* x, unsigned nx, double coef,
                 double* y, unsigned ny) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    math::dVec X(nx), Y(ny);
    for (unsigned i = 0; i < nx; i++) X[i] = x[i];
    for (unsigned i = 0; i < ny; i++) Y[i] = y[i];
    auto* K = m->storage.getK();
    if (block == 1 || block == 2)
      matBVprod(*K->block(block), X, coef, Y);  // friends: found by ADL
    else if (trans)
      matBTVprod(*K->block(1, 2), X, coef, Y);
    else
      matBVprod(*K->block(1, 2), X, coef, Y);
    for (unsigned i = 0; i < ny; i++) y[i] = Y[i];
  });
}

static int get_cm(RefModel* m, bool C, int block, double* values) {
  return guarded(m, [&] {
    if (!m->storage.isTransient()) LOG(FATAL) << "not a transient model";
    auto* X = C ? m->storage.getC() : m->storage.getM();
    math::BaseSparseMatrix* B = X->block(1, 2);
    if (block == 1) B = X->block(1);
    if (block == 2) B = X->block(2);
    if (B->nValues() == 0) return;
    std::memcpy(values, B->getValuesArray(), sizeof(double) * B->nValues());
  });
}

int ref_get_C(void* h, int block, double* values) {
  return get_cm(static_cast<RefModel*>(h), true, block, values);
}

int ref_get_M(void* h, int block, double* values) {
  return get_cm(static_cast<RefModel*>(h), false, block, values);
}

int ref_set_R(void* h, const double* R, unsigned n) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    math::dVec* v = m->storage.getR();
    if (v->size() != n) LOG(FATAL) << "R size mismatch";
    for (unsigned i = 0; i < n; i++) (*v)[i] = R[i];
  });
}

// The reference's VtkProcessor (VtkProcessor.cpp): pre() writes <prefix>0.vtk,
// process(step) writes <prefix><step>.vtk (step > 0), from the current vecU / vecR.
int ref_write_vtk(void* h, const char* prefix, int step) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    VtkProcessor vtk(&m->storage, prefix);
    vtk.pre();
    if (step > 0) vtk.process((uint16)step);
  });
}

int ref_get_F(void* h, double* F) {
  RefModel* m = static_cast<RefModel*>(h);
  return guarded(m, [&] {
    math::dVec* v = m->storage.getF();
    for (uint32 i = 0; i < v->size(); i++) F[i] = (*v)[i];
  });
}

}  // extern "C"
