/* Oracle for the nla3d assembly path: a plain-C restatement of the reference
 * algorithm (see nla3d_oracle.c).  TEST INFRASTRUCTURE ONLY -- the tests, the
 * smoke check and bench.py's CPU-baseline leg are the only callers; nothing on
 * the product path links or loads it.
 *
 * The model API mirrors the reference's FEStorage set-up sequence
 * (FEStorage.h:255-270): build the model, add constraints and rigid-body MPC
 * collections, orc_setup() (initDofs + setConstrainedNodeDof +
 * assignEquationNumbers + initSolutionData), then per iteration
 * orc_set_U() -> orc_update() -> orc_assemble().
 */
#ifndef NLA3D_ORACLE_H
#define NLA3D_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model orc_model;

/* elem_type: reference ElementType (sys.h:151-163): 2 SOLID81, 3 TETRA0, 5 QUADTH.
 * mat_id: reference MaterialFactory::matId (MaterialFactory.h:12-18):
 *   1 Neo-Hookean (G, K), 2 Biderman (C10, C20, C30, C01, K),
 *   3 Mooney-Rivlin (C10, C01, K); 0 = none.
 * elem_params: n_elem_params doubles per element (up to 4; missing ones are 0):
 *   TETRA0 (E, my), QUADTH (k, volFlux, rho, c) (TETRA0.h, QUADTH.h:29-35). */
orc_model* orc_new(int elem_type, uint32_t n_nodes, const double* xyz, uint32_t n_elems,
                   const uint32_t* conn, int mat_id, const double* mat_c, int n_mat_c,
                   const double* elem_params, int n_elem_params);
void orc_free(orc_model* m);
const char* orc_error(orc_model* m);
int orc_add_fix(orc_model* m, uint32_t n, const uint32_t* nodes, const int32_t* dofs);
int orc_add_rigid_body(orc_model* m, uint32_t master, uint32_t n_slaves, const uint32_t* slaves,
                       uint32_t n_dofs, const int32_t* dofs);
/* FEStorage::addMpc of an Mpc (Mpc.h:31-36): sum coefs[t] u(nodes[t], dofs[t]) = b */
int orc_add_mpc(orc_model* m, uint32_t n_terms, const uint32_t* nodes, const int32_t* dofs,
                const double* coefs, double b);
/* SurfaceLINETH elements of a QUADTH model (QUADTH.h:38-55), created after
 * its elements: conn 2 nodes per line, htc, flux (NULL = 0) and etemp
 * (2 per line; a zero second value takes the first, SurfaceLINETH::pre). */
int orc_add_surface_lines(orc_model* m, uint32_t n, const uint32_t* conn, const double* htc,
                          const double* flux, const double* etemp);
/* FEStorage::setTransient (FEStorage.h:127): assemble C and M too. */
int orc_set_transient(orc_model* m, int on);
/* max_in_row: the reference's pre-compress row capacity (BlockSparseMatrix.h:42,
 * default 100); overflow is reported as an error like SparseMatrix.cpp:84. */
int orc_setup(orc_model* m, uint32_t max_in_row);
/* out[0..3] = nDofs, nConstrained, nUnknown, nMpc;
 * out[4..12] = (rows, cols, nnz) of block(1), block(1,2), block(2). */
void orc_info(orc_model* m, uint32_t* out);
int orc_pattern(orc_model* m, int block, uint32_t* iofeir, uint32_t* columns);
int orc_eq_numbers(orc_model* m, uint32_t* node_eq, uint32_t* elem_eq);
int orc_set_U(orc_model* m, const double* U, uint32_t n);
int orc_update(orc_model* m);
int orc_assemble(orc_model* m);
int orc_get_K(orc_model* m, int block, double* values);
int orc_get_F(orc_model* m, double* F);
/* TETRA0 stresses from the current U (ElementTETRA0::update, TETRA0.cpp:79-108):
 * 6 per element (xx, yy, zz, xy, yz, xz). */
int orc_tetra0_stress(orc_model* m, double* out);
/* C and M of a transient model, block 1 / 12 / 2 on K's pattern. */
int orc_get_C(orc_model* m, int block, double* values);
int orc_get_M(orc_model* m, int block, double* values);
/* y += coef * op(block) x on the assembled K (SparseMatrix.cpp:497-558):
 * block 1 / 2: matBVprod(SparseSymMatrix&) (both triangles, x_j with
 * |x_j| <= 1e-20 skipped; stored entries only, in the reference's order);
 * block 12: trans 0 matBVprod(SparseMatrix&), trans 1 matBTVprod(SparseMatrix&). */
int orc_block_mv(orc_model* m, int block, int trans, const double* x, double coef, double* y);

/* Element-level pieces (for tests against the reference's own fixtures). */
void orc_hex_jacobian(const double* X /*8x3*/, int int_order, double* NiXj /*np x 8 x 3*/,
                      double* det /*np*/);
void orc_material_S(int mat_id, const double* mc, const double* C, double p, double* S);
void orc_material_D(int mat_id, const double* mc, const double* C, double p, double* Dd,
                    double* Dp);
/* The dense kernels of Mat.h:686-801 on row-major arrays. */
void orc_matBTDBprod(int M, int N, const double* B, const double* Dsym, double coef, double* Rsym);
void orc_matBTVprod(int M, int N, const double* B, const double* V, double coef, double* R);
void orc_matBVprod(int M, int N, const double* B, const double* V, double coef, double* R);
void orc_matABprod(int M1, int N1, int N2, const double* A, const double* B, double coef,
                   double* R);
void orc_matATBprod(int M1, int N1, int N2, const double* A, const double* B, double coef,
                    double* R);

#ifdef __cplusplus
}
#endif
#endif
