/* nla3d_gpu.h -- C ABI of the GB300 (sm_103a) implementation of nla3d's
 * per-iteration global assembly.
 *
 * The entry points replace the FEStorage member functions of the reference
 * (paths relative to the reference's src/lib/) for the assembly path:
 *
 *   nla3d_create                 FEStorage::createNodes / createElements  FEStorage.h:211,223
 *                                (+ node positions, the Material instance  FEStorage.h:48)
 *   nla3d_add_fix                FEStorage::setConstrainedNodeDof           FEStorage.h:159
 *   nla3d_add_rigid_body         FEStorage::addMpcCollection(RigidBodyMpc)  FEStorage.h:200, Mpc.h:51
 *   nla3d_add_mpc                FEStorage::addMpc(Mpc)                     FEStorage.h:198, Mpc.h:31
 *   nla3d_build_pattern          initDofs + assignEquationNumbers + the
 *                                sparsity part of initSolutionData (host)   FEStorage.h:259,263,265
 *   nla3d_init_solution_data     initSolutionData: the above + device
 *                                allocation and upload                      FEStorage.h:265
 *   nla3d_set_U / _device        writes of FEStorage::getU() (vecU)         FEStorage.h:109
 *   nla3d_update_results         FEStorage::updateResults                   FEStorage.h:270
 *   nla3d_assemble               FEStorage::assembleGlobalEqMatrices        FEStorage.h:115
 *   nla3d_get_K / nla3d_pattern  FEStorage::getK() -> BlockSparseSymMatrix<2>::block(..)
 *                                getValuesArray / getColumnsArray /
 *                                getIofeirArray                             FEStorage.h:100,
 *                                                                           SparseMatrix.h:206-221
 *   nla3d_get_F                  FEStorage::getF()                          FEStorage.h:105
 *   nla3d_eq_numbers             FEStorage::getNodeDofEqNumber /
 *                                getElementDofEqNumber                      FEStorage.h:148-149
 *
 * Conventions kept from the reference: node, element and equation numbers
 * start at 1; constrained equations are numbered first; K is split into
 * block(1) (constrained x constrained, symmetric upper), block(1,2)
 * (constrained x unknown+MPC, general) and block(2) (unknown+MPC, symmetric
 * upper), each a 1-based 3-array CSR with sorted columns.
 *
 * Errors: every function returns an int status (NLA3D_OK == 0).  Nothing
 * aborts the process; nla3d_last_error() describes the last failure.
 * Threading: one context = one CUDA stream; calls on a context must be
 * serialised by the caller (the reference is single-threaded too).
 */
#ifndef NLA3D_GPU_H
#define NLA3D_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NLA3D_OK 0
#define NLA3D_ERR_ARG 1      /* bad argument or call order                       */
#define NLA3D_ERR_CUDA 2     /* a CUDA runtime call failed                        */
#define NLA3D_ERR_PATTERN 3  /* a contribution has no CSR slot (SparseMatrix.cpp:400) */
#define NLA3D_ERR_NOMEM 4    /* host or device allocation failed                  */
#define NLA3D_ERR_RANGE 5    /* a size exceeds an index type or a fixed limit     */
#define NLA3D_ERR_ELEMENT 6  /* an element reported J <= 0 or a non-finite value  */

/* Element types: the reference's ElementType codes (sys.h:151-163). */
#define NLA3D_PLANE41 1
#define NLA3D_SOLID81 2
#define NLA3D_TETRA0 3
#define NLA3D_QUADTH 5

/* Materials: the reference's MaterialFactory::matId (MaterialFactory.h:12-18).
 * Constants in the reference's order (materials_hyperelastic.h:45-105). */
#define NLA3D_MAT_NEO_HOOKEAN 1   /* G, K                 */
#define NLA3D_MAT_BIDERMAN 2      /* C10, C20, C30, C01, K */
#define NLA3D_MAT_MOONEY_RIVLIN 3 /* C10, C01, K           */

/* DoF types: Dof::dofType (Dof.h:15-25). */
#define NLA3D_UX 0
#define NLA3D_UY 1
#define NLA3D_UZ 2
#define NLA3D_ROTX 3
#define NLA3D_ROTY 4
#define NLA3D_ROTZ 5
#define NLA3D_HYDRO_PRESSURE 6
#define NLA3D_TEMP 7

/* Arithmetic of the SOLID81 element kernel. */
#define NLA3D_PREC_FP64 0  /* everything in FP64 (parity path, <=1e-12 vs the reference) */
#define NLA3D_PREC_MIXED 1 /* FP32 tangent K_uu (B^T.D.B and the geometric term); FP64
                              volumetric terms (J = det F, J-1, p/K, the pressure
                              coupling K_up = w J C^-1 B, K_pp, F_p) and MPC rows; the
                              rest of the residual chain (gradient, C, S, F_u) in
                              float-pair arithmetic (~2^-48 per operation); FP64 CSR
                              sums.  SOLID81
                              meshes whose material constants are outside 1e-20 .. 1e20 in
                              magnitude, or whose extent is outside 1e-6 .. 1e6, are
                              rejected by nla3d_create(_batch) with NLA3D_ERR_RANGE */

typedef struct nla3d_ctx nla3d_ctx;

typedef struct {
  int32_t elem_type;          /* NLA3D_SOLID81 / NLA3D_PLANE41 / NLA3D_TETRA0 / QUADTH */
  uint32_t n_nodes;
  uint32_t n_elems;
  const double* xyz;          /* 3 * n_nodes, host                                    */
  const uint32_t* conn;       /* nodes_per_elem * n_elems, 1-based node ids, host     */
  int32_t mat_id;             /* NLA3D_MAT_* (SOLID81, PLANE41), 0 otherwise          */
  double mat_c[5];
  const double* elem_params;  /* n_elem_params * n_elems: TETRA0 (E, my), QUADTH (k,
                                 volFlux[, rho, c]); or NULL                          */
  int32_t n_elem_params;      /* 2 (also when 0) or 4 (QUADTH with rho, c)            */
} nla3d_mesh_desc;

/* Create a model (FEStorage with nodes, elements and material).  `precision`
 * selects the SOLID81 arithmetic (NLA3D_PREC_*).  Makes no CUDA call. */
int nla3d_create(const nla3d_mesh_desc* mesh, int precision, nla3d_ctx** out);

/* A batch of independent meshes in one context (each one a separate reference
 * FEStorage with its own numbering, pattern, K and F; same element type, any
 * material constants).  Every kernel of an assembly then runs once over all
 * meshes.  vecU, F and K of the batch are the concatenation of the meshes'
 * arrays; nla3d_mesh_info gives each mesh's offsets.  The single-mesh calls
 * (nla3d_info, nla3d_pattern, nla3d_eq_numbers, nla3d_slot_maps, nla3d_get_K,
 * nla3d_add_fix, nla3d_add_rigid_body) refer to mesh 0; nla3d_set_U,
 * nla3d_get_F and nla3d_device_F take the whole concatenation. */
int nla3d_create_batch(const nla3d_mesh_desc* meshes, uint32_t n_meshes, int precision,
                       nla3d_ctx** out);
uint32_t nla3d_mesh_count(const nla3d_ctx* ctx);
int nla3d_mesh_add_fix(nla3d_ctx* ctx, uint32_t mesh, uint32_t n, const uint32_t* nodes,
                       const int32_t* dofs);
int nla3d_mesh_add_rigid_body(nla3d_ctx* ctx, uint32_t mesh, uint32_t master, uint32_t n_slaves,
                              const uint32_t* slaves, uint32_t n_dofs, const int32_t* dofs);
int nla3d_mesh_add_mpc(nla3d_ctx* ctx, uint32_t mesh, uint32_t n_terms, const uint32_t* nodes,
                       const int32_t* dofs, const double* coefs, double b);
/* out as nla3d_info; offsets[0..4] = the mesh's first element, node, equation
 * (index into vecU / F), K value and MPC equation in the concatenation. */
int nla3d_mesh_info(const nla3d_ctx* ctx, uint32_t mesh, uint32_t out[16], uint64_t offsets[5]);
int nla3d_mesh_pattern(const nla3d_ctx* ctx, uint32_t mesh, int block, uint32_t* iofeir,
                       uint32_t* columns);
int nla3d_mesh_eq_numbers(const nla3d_ctx* ctx, uint32_t mesh, uint32_t* node_eq,
                          uint32_t* elem_eq);
int nla3d_destroy(nla3d_ctx* ctx);
const char* nla3d_last_error(const nla3d_ctx* ctx);

/* Run on this CUDA stream (cudaStream_t passed as void*); default: the
 * context's own non-blocking stream. */
int nla3d_set_stream(nla3d_ctx* ctx, void* stream);
void* nla3d_get_stream(const nla3d_ctx* ctx);

int nla3d_add_fix(nla3d_ctx* ctx, uint32_t n, const uint32_t* nodes, const int32_t* dofs);
int nla3d_add_rigid_body(nla3d_ctx* ctx, uint32_t master, uint32_t n_slaves,
                         const uint32_t* slaves, uint32_t n_dofs, const int32_t* dofs);
/* SurfaceLINETH elements (QUADTH.cpp:70-125) of a single-mesh QUADTH
 * context: n lines of 2 nodes (conn, 1-based) with convection coefficient
 * htc, flux and environment temperatures etemp (2 per line; a zero second
 * value takes the first, as SurfaceLINETH::pre does).  They are numbered
 * after the QUADTH elements, as when created after them.  Before
 * nla3d_init_solution_data. */
int nla3d_add_surface_lines(nla3d_ctx* ctx, uint32_t n, const uint32_t* conn, const double* htc,
                            const double* flux, const double* etemp);
/* FEStorage::setTransient (FEStorage.h:127): each assembly also builds the
 * capacity matrix C and the mass matrix M on K's pattern (FEStorage.cpp:63-76).
 * Of the element types here only QUADTH builds C (QUADTH.cpp:51-67) and none
 * builds M, so M is zero; other types abort in the reference and are refused
 * here (NLA3D_ERR_ELEMENT).  Before nla3d_init_solution_data. */
int nla3d_set_transient(nla3d_ctx* ctx, int on);
/* Values of C or M, block 1 / 12 / 2 (as nla3d_get_K), after an assembly of
 * a transient context. */
int nla3d_get_C(nla3d_ctx* ctx, int block, double* values);
int nla3d_get_M(nla3d_ctx* ctx, int block, double* values);

/* A linear MPC equation sum_t coefs[t] * u(nodes[t], dofs[t]) = b (an Mpc
 * with these terms passed to FEStorage::addMpc, as readCdbFile builds it from
 * a CE record, FEReaders.cpp:549-573).  Its equation comes after the DoFs, in
 * the order of the calls and before the rigid-body MPC equations; each
 * assembly writes F[eq] = b and adds every coefficient to K(DoF, eq)
 * (FEStorage.cpp:49-60).  Every term's DoF must be used by an element or a
 * rigid body. */
int nla3d_add_mpc(nla3d_ctx* ctx, uint32_t n_terms, const uint32_t* nodes, const int32_t* dofs,
                  const double* coefs, double b);

/* Host-only set-up: DoF registration, equation numbering, the CSR pattern
 * (bit-exact with the reference) and the element -> CSR slot maps with their
 * fixed-order gather lists.  Makes no CUDA call.  Idempotent. */
int nla3d_build_pattern(nla3d_ctx* ctx);
/* nla3d_build_pattern (if not done yet), device allocation and upload, and
 * the once-per-mesh Jacobian precompute.  Synchronous.  Selects the device
 * that is current at this call.  For a single mesh, the CSR pattern, slot
 * maps and gather lists may be built on the device instead (the numbering
 * stays on the host; same arrays, bit for bit): see nla3d_set_pattern_builder. */
int nla3d_init_solution_data(nla3d_ctx* ctx);
/* Where nla3d_init_solution_data builds the pattern of a single-mesh context:
 * 0 host, 1 device, -1 (default) device for meshes of 65,536 elements or
 * more.  A mesh beyond the device builder's limits (more than 1024 distinct
 * columns around one node) is built on the host.  Call before
 * nla3d_build_pattern / nla3d_init_solution_data.  No counterpart in the
 * reference (its initSolutionData is host code, FEStorage.cpp:434-550). */
int nla3d_set_pattern_builder(nla3d_ctx* ctx, int mode);
/* 1 if this context's pattern was built on the device. */
int nla3d_pattern_on_device(const nla3d_ctx* ctx);
/* Element -> slot maps (valid after nla3d_build_pattern and until
 * nla3d_init_solution_data releases them): kslot[e * nk + c] is the index
 * into the concatenated K values (block(1) | block(1,2) | block(2)) of K
 * contribution c of element e (reference assembly order); fslot[e * nf + c]
 * is the 0-based F row.  nk, nf: out[13], out[14] of nla3d_info. */
int nla3d_slot_maps(const nla3d_ctx* ctx, uint32_t* kslot, uint32_t* fslot);

/* out[0..3] = nDofs, nConstrainedDofs, nUnknownDofs, nMpc;
 * out[4..12] = (rows, cols, nnz) of block(1), block(1,2), block(2);
 * out[13], out[14] = K and F contributions per element; out[15] reserved.
 * Valid after nla3d_build_pattern. */
int nla3d_info(const nla3d_ctx* ctx, uint32_t out[16]);
/* block: 1, 2 or 12 (= block(1,2)).  iofeir: rows+1 entries; columns: nnz. */
int nla3d_pattern(const nla3d_ctx* ctx, int block, uint32_t* iofeir, uint32_t* columns);
/* Equation number per (node, Dof type) and (element, Dof type), 8 types each,
 * 0 = unused. */
int nla3d_eq_numbers(const nla3d_ctx* ctx, uint32_t* node_eq, uint32_t* elem_eq);

/* vecU (nDofs + nMpc doubles) from host memory (copied on the context
 * stream) or from device memory. */
int nla3d_set_U(nla3d_ctx* ctx, const double* U, uint64_t n);
int nla3d_set_U_device(nla3d_ctx* ctx, const double* U_dev, uint64_t n);

/* FEStorage::updateResults: the per-Gauss-point state of the next assembly is
 * taken from the current U (asynchronous). */
int nla3d_update_results(nla3d_ctx* ctx);
/* FEStorage::assembleGlobalEqMatrices: element tangents and residuals,
 * fixed-order CSR sums, MPC rows (asynchronous; K and F stay on the device). */
int nla3d_assemble(nla3d_ctx* ctx);

/* Results.  Host copies synchronise the stream. */
int nla3d_get_K(nla3d_ctx* ctx, int block, double* values);
int nla3d_get_F(nla3d_ctx* ctx, double* F);
/* All K values of the context (every mesh: block(1) | block(1,2) | block(2)). */
int nla3d_get_K_all(nla3d_ctx* ctx, double* values);
/* nla3d_assemble, then the K blocks and F copied into host arrays (what
 * nla3d_get_K for blocks 1, 12, 2 and nla3d_get_F return), with the copies
 * overlapping the assembly: the element kernel runs over n_chunks element
 * ranges (1..64; range k holds n_chunks - k parts of n_chunks (n_chunks + 1)
 * / 2, the shortest last), and after each range the runs of K slots whose last
 * contributing element is done (and that are at least 65,536 slots long)
 * are summed and copied while the next range computes; the rest, MPC terms
 * included, comes after the last range.  Same values as the unchunked path,
 * bit for bit.  The plan is built on the first call per n_chunks.  Single-mesh
 * contexts; host arrays should be page-locked for the copies to overlap.
 * Synchronous.  Replaces FEStorage::assembleGlobalEqMatrices + reading
 * matK / vecF on the host (FEStorage.cpp:26-78, FEStorage.h:100-105). */
int nla3d_assemble_to_host(nla3d_ctx* ctx, int n_chunks, double* K1, double* K12, double* K2,
                           double* F);

/* y += coef * op(K block) x on the device, with the values of the last
 * nla3d_assemble of mesh `mesh` (0 for a single-mesh context), on the
 * context's stream (asynchronous, like nla3d_assemble).  Replaces the
 * reference's sparse products of the Newton iteration (FESolver.cpp:454-466):
 *   block 1 or 2: matBVprod(SparseSymMatrix&, dVec, coef, dVec&)
 *       (SparseMatrix.cpp:497-519): both triangles of the symmetric block,
 *       entries x_j with |x_j| <= 1e-20 skipped as there; trans is ignored;
 *   block 12, trans 0: matBVprod(SparseMatrix&, ...)  (SparseMatrix.cpp:522-540);
 *   block 12, trans 1: matBTVprod(SparseMatrix&, ...) (SparseMatrix.cpp:542-558).
 * Each y entry is accumulated in the reference's order with (K x) coef
 * rounded before the add, so y is the reference's result bit for bit (the
 * reference's symmetric product also adds +-0 for structural zeros, which
 * can only change the sign of a zero result).  x, y: device arrays of the
 * block's column / row count (transposed for trans 1); a block without stored
 * entries leaves y unchanged and reads neither pointer.  The first call per
 * (mesh, block, trans) builds its walk list (about 8 bytes per stored entry,
 * twice that for a symmetric block) and synchronises the stream once. */
int nla3d_block_mv(nla3d_ctx* ctx, uint32_t mesh, int block, int trans, const double* x,
                   double coef, double* y);

/* Device pointers (valid until nla3d_destroy): K values of one block (block 0
 * = all K values of the context), F. */
int nla3d_device_K(const nla3d_ctx* ctx, int block, double** values, uint64_t* n);
int nla3d_device_F(const nla3d_ctx* ctx, double** F, uint64_t* n);
int nla3d_synchronize(nla3d_ctx* ctx);

/* Elements flagged by the last assembly (J <= 0, det J <= 0 or a non-finite
 * value): count and smallest 1-based element number (0 if none).
 * Synchronises.  Returns NLA3D_ERR_ELEMENT when count > 0. */
int nla3d_element_status(nla3d_ctx* ctx, uint32_t* count, uint32_t* first);

/* Number of kernels launched by the library on this context so far. */
uint64_t nla3d_kernel_launches(const nla3d_ctx* ctx);

/* Launch shape of the element kernel (warps per block 2/4/8, resident blocks
 * per SM, 0 = as many as fit), the gather block size (128..1024), and the
 * layout of the element contributions (0: element order, K gathered through
 * an index list; 1: the element kernel writes each contribution at its slot
 * position and K is a contiguous sum).  Every choice sums each K slot in the
 * same order, so the results do not depend on them.  nla3d_autotune times the
 * candidates on this context's own mesh(es) with `reps` assemblies, keeps the
 * fastest and reports it in chosen[4] = (warps per block, blocks per SM,
 * gather block, layout) and *best_ms (one assembly).  No counterpart in the
 * reference. */
int nla3d_set_launch_shape(nla3d_ctx* ctx, int warps_per_block, int blocks_per_sm,
                           int gather_block);
int nla3d_set_contrib_layout(nla3d_ctx* ctx, int layout);
int nla3d_autotune(nla3d_ctx* ctx, int reps, int32_t chosen[4], float* best_ms);

/* Record updateResults + assembleGlobalEqMatrices (on the current vecU buffer)
 * as a CUDA graph on the context stream, and replay it.  A new launch shape
 * or stream releases the graph.  No counterpart in the reference. */
int nla3d_graph_capture(nla3d_ctx* ctx);
int nla3d_graph_launch(nla3d_ctx* ctx);

/* Measurement helpers (no counterpart in the reference, which has no GPU).
 * nla3d_set_timing(ctx, 1) records CUDA events on the context stream around
 * each kernel of every nla3d_assemble (a ring of the last 256 assemblies);
 * nla3d_kernel_times() returns the mean time in ms per assembly over the
 * assemblies recorded since the previous call (or since timing was switched
 * on): [0] element kernel, [1] K gather, [2] F gather, [3] MPC rows, and in
 * *count how many assemblies the mean covers (synchronises). */
int nla3d_set_timing(nla3d_ctx* ctx, int on);
int nla3d_kernel_times(nla3d_ctx* ctx, float ms[4], uint32_t* count);
/* Throughput probe of dependent-chain-free FMA on the current device:
 * fp64 != 0 -> DFMA, else FFMA.  Returns FLOP/s (2 per FMA) in *flops. */
int nla3d_probe_fma_peak(int fp64, double* flops);

/* ---------------------------------------------------------------------------
 * Learned Newton start: kernels of a small MLP (BF16 weights, FP32
 * accumulation) trained on converged increments.  No counterpart in the
 * reference (it always restarts Newton from the previous converged state).
 * All pointers are device memory; calls are asynchronous on `stream`.
 *   nla3d_mlp_gemm    C[m,n] = act(sum_k A[m,k] B[k,n] + bias[n]); A[m,k] is at
 *                     A + m*lda_m + k*lda_k (B likewise), a_bf16 / b_bf16 select
 *                     BF16 inputs; act 0 = identity, 1 = tanh; bias may be NULL
 *                     (A and B too when K = 0: C = act(bias)).
 *                     Runs on the tensor cores (tcgen05.mma, BF16 operands,
 *                     FP32 accumulation in TMEM); an FP32 operand enters as a
 *                     BF16 pair hi + lo (|x - hi - lo| <= 2^-16 |x|).  A bounded
 *                     wait that runs out sets the tile to NaN and is counted.
 *   nla3d_mlp_status  *timeouts = GEMM tiles whose MMA wait ran out since the
 *                     last call (then reset; synchronous)
 *   nla3d_mlp_tanh_backward   dY *= 1 - Y*Y (in place)
 *   nla3d_mlp_column_sum      out[c] = sum_r X[r, c] (row-major rows x cols)
 *   nla3d_mlp_adam    Adam step on FP32 master weights (step >= 1), refreshing
 *                     the BF16 copy w_bf16 when non-NULL
 *   nla3d_mlp_mse_grad dY = scale * (Y - T)
 *   nla3d_mlp_to_bf16 round-to-nearest-even FP32 -> BF16 */
int nla3d_mlp_gemm(int M, int N, int K, const void* A, int a_bf16, int64_t lda_m, int64_t lda_k,
                   const void* B, int b_bf16, int64_t ldb_k, int64_t ldb_n, float* C, int64_t ldc,
                   const float* bias, int act, void* stream);
int nla3d_mlp_tanh_backward(const float* Y, float* dY, int64_t n, void* stream);
int nla3d_mlp_column_sum(const float* X, int64_t rows, int64_t cols, float* out, void* stream);
int nla3d_mlp_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float beta1,
                   float beta2, float eps, int step, uint16_t* w_bf16, void* stream);
int nla3d_mlp_mse_grad(const float* Y, const float* T, float* dY, int64_t n, float scale,
                       void* stream);
int nla3d_mlp_to_bf16(const float* x, uint16_t* y, int64_t n, void* stream);
int nla3d_mlp_status(uint32_t* timeouts);

/* ---------------------------------------------------------------------------
 * SOLID81 assembly without device allocation.  No counterpart in the
 * reference (which has no GPU code); it is an extra entry point for callers
 * that may not allocate device memory: host frameworks that own all device
 * memory through their own pool and forbid a plugin from calling cudaMalloc,
 * and time-critical loops that cannot afford cudaMalloc's implicit device
 * synchronisation.
 *
 * The caller passes every input and output as device memory it owns; the
 * library keeps its intermediate data (shape-function gradients and element
 * contributions, 4400 bytes per element) in a fixed array of
 * NLA3D_NOALLOC_SCRATCH_BYTES compiled into the library, which every GPU that
 * loads the library holds until exit.  Hence at most NLA3D_NOALLOC_MAX_ELEMS
 * elements per call; larger meshes are rejected with NLA3D_ERR_RANGE before
 * anything runs.  The call makes no cudaMalloc / cudaFree and uses no
 * allocating library routine.
 *
 * All calls share that array: calls whose kernels overlap on the GPU (other
 * streams or threads without ordering) race and corrupt each other.  The
 * first call on a device looks up the array's device address with that
 * device current, and uploads a constant table; make that first call before
 * any stream capture.  The looked-up address is cached per device ordinal
 * for the device's primary context: after cudaDeviceReset(), or under
 * another driver-API context on that device, it no longer applies.
 *
 * Preconditions, checked on the device by the first kernel of every call:
 * conn in 1..n_nodes; node_eq[4 (node - 1) + 0..2] of every node that conn
 * names, and p_eq, in 1..n_eq; k_ptr non-decreasing with
 * k_ptr[nnz] <= 325 n_elems and every k_ids < 325 n_elems; f_ptr
 * non-decreasing with f_ptr[n_eq] <= 25 n_elems and every f_ids <
 * 25 n_elems.  If any fails, nothing is assembled (K and F keep their
 * contents, no out-of-bounds access) and, when `flagged` is non-NULL, the
 * call returns NLA3D_ERR_ARG.
 *
 * Semantics: updateResults() followed by assembleGlobalEqMatrices() on the
 * same U, SOLID81 elements only (no MPC rows), FP64.  Inputs:
 *   node_eq  4 per node: equations of UX, UY, UZ (nla3d_eq_numbers) and a pad
 *            word; 16-byte aligned;
 *   p_eq     the HYDRO_PRESSURE equation of each element;
 *   k_ptr / k_ids, f_ptr / f_ids: the inverse of nla3d_slot_maps -- for each
 *            K slot (F row) the ids e * 325 + c (e * 25 + c) of its
 *            contributions in ascending order, as CSR (nnz + 1 / n_eq + 1
 *            offsets).
 * Asynchronous on `stream` unless `flagged` is non-NULL, in which case it
 * synchronises and stores the number of flagged elements there
 * (NLA3D_ERR_ELEMENT if any). */
#define NLA3D_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define NLA3D_NOALLOC_MAX_ELEMS 15252u

typedef struct {
  uint32_t n_elems;        /* 1 .. NLA3D_NOALLOC_MAX_ELEMS                */
  uint32_t n_nodes;
  uint32_t n_eq;           /* vecU and F length (nDofs + nMpc)            */
  uint64_t nnz;            /* K values, block(1) | block(1,2) | block(2)  */
  const double* xyz;       /* 3 * n_nodes                                 */
  const uint32_t* conn;    /* 8 * n_elems, 1-based node ids               */
  const uint32_t* node_eq; /* 4 * n_nodes                                 */
  const uint32_t* p_eq;    /* n_elems                                     */
  const double* U;         /* n_eq                                        */
  const uint32_t* k_ptr;   /* nnz + 1                                     */
  const uint32_t* k_ids;   /* 325 * n_elems                               */
  const uint32_t* f_ptr;   /* n_eq + 1                                    */
  const uint32_t* f_ids;   /* 25 * n_elems                                */
  int32_t mat_id;          /* NLA3D_MAT_*                                 */
  double mat_c[5];
  double* K;               /* out: nnz                                    */
  double* F;               /* out: n_eq                                   */
} nla3d_solid81_noalloc_args;

int nla3d_assemble_solid81_noalloc(const nla3d_solid81_noalloc_args* args, void* stream,
                                   uint32_t* flagged);

/* ---- sparse LDL^T of K(2) on the device --------------------------------
 * Replaces the reference's EquationSolver (EquationSolver.h:19-34:
 * factorizeEquations / substituteEquations / solveEquations on the
 * SparseSymMatrix K(2), upper CSR, 1-based) with a supernodal multifrontal
 * LDL^T whose factor stays on the device next to the assembled K.
 * iofeir / columns: the upper CSR pattern (nla3d_pattern of block 2); perm:
 * a fill-reducing order (perm[new] = equation - 1) or NULL; rows with a zero
 * diagonal (MPC / CE equations) must come after the DoFs they couple to.
 * There is no pivoting: a pivot below pivot_rel * max|K| (1e-13 FP64, 1e-7
 * FP32) is replaced by +-that value and counted; the solve refines in FP64. */
typedef struct nla3d_ldlt nla3d_ldlt;
/* A fill-reducing order for nla3d_ldlt_create (host; no GPU needed): points
 * holds a point per row (n x 3: the node of a nodal DoF, an element's
 * centroid, an MPC equation's first node); geometric nested dissection (split
 * at the median of the longest extent, the lower half's rows that couple to
 * the upper half as separator after both halves, leaves of 64 rows), then the
 * rows below n_dofs with a stored diagonal, the rows from n_dofs on (MPC / CE
 * equations), the rows below n_dofs without a diagonal.  order: n entries
 * (order[new] = row, 0-based). */
int nla3d_ldlt_order(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                     const double* points, int64_t n_dofs, int32_t* order);
/* Symbolic analysis only (host; no GPU needed).  stats[8] = supernodes,
 * levels, largest front, entries of L (incl. D), factorisation flops, front
 * buffer entries, most children of a supernode, total supernode rows; each
 * other output may be NULL: perm_out (n, factor order -> equation - 1),
 * sn_first_out (supernodes + 1), row_ptr_out (supernodes + 1), rows_out
 * (stats[7]; each supernode's rows in factor order, its pivots first). */
int nla3d_ldlt_analyze(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                       const int32_t* perm, double* stats, int32_t* perm_out, int32_t* sn_first_out,
                       int64_t* row_ptr_out, int32_t* rows_out);
/* precision 0: FP64 fronts; 1: FP32 fronts (half the memory, FP64 refinement);
 * 2: FP32 fronts whose trailing updates run on the tensor cores (tcgen05,
 * TF32 split in high and low parts: hi.hi + hi.lo + lo.hi, FP32 accumulation).
 * stream: the stream the values are produced on (NULL: a stream of its own);
 * a borrowed stream must outlive the handle.
 * On an error after the handle exists, *out is set: read nla3d_ldlt_last_error
 * and call nla3d_ldlt_destroy. */
int nla3d_ldlt_create(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                      const int32_t* perm, int precision, void* stream, nla3d_ldlt** out);
/* EquationSolver::factorizeEquations: values = the device K(2) values
 * (nla3d_device_K block 2).  NLA3D_ERR_ELEMENT on a non-finite pivot. */
int nla3d_ldlt_factor(nla3d_ldlt* h, const double* values);
/* EquationSolver::substituteEquations: x = K(2)^-1 b on device vectors, then
 * refinement until ||b - K x|| <= tol ||b|| with at most max_refine further
 * applications of the factor: steps x += K^-1 (b - K x) while each cuts the
 * residual tenfold, then restarted GMRES(30) preconditioned by the factor
 * (values: the same K as factored, or a nearby one).  NLA3D_ERR_RANGE when
 * tol is not reached; steps and rel_residual may be NULL. */
int nla3d_ldlt_solve(nla3d_ldlt* h, const double* values, const double* b, double* x,
                     int max_refine, double tol, int* steps, double* rel_residual);
/* EquationSolver::solveEquations(K(2), rhs, x) with host vectors: b_host and
 * x_host hold n doubles (pageable or pinned); they go through device buffers
 * the handle owns, then as nla3d_ldlt_solve.  x_host is written also on
 * NLA3D_ERR_RANGE (the refined x, tol not reached).  Synchronises the
 * handle's stream. */
int nla3d_ldlt_solve_host(nla3d_ldlt* h, const double* values, const double* b_host,
                          double* x_host, int max_refine, double tol, int* steps,
                          double* rel_residual);
/* out[8]: supernodes, levels, largest front, entries of L, flops, front bytes,
 * perturbed pivots and non-finite pivots of the last factorisation. */
int nla3d_ldlt_info(const nla3d_ldlt* h, double* out);
const char* nla3d_ldlt_last_error(const nla3d_ldlt* h);
/* Self-check of the tensor-core updates (precision 2): one front of m rows
 * (65 .. 4096) after its first outer block (256 columns when m > 512, else
 * 64), updated from the same random data by the FMA kernel and by the
 * tcgen05 path (operands packed once, then bulk-copied by the persistent
 * kernel); out[0] = max |difference|, out[1] = max |update|.
 * NLA3D_ERR_RANGE if an MMA or copy wait timed out.  Synchronises the
 * device. */
int nla3d_ldlt_tc_check(int m, double* out);
int nla3d_ldlt_destroy(nla3d_ldlt* h);

#ifdef __cplusplus
}
#endif
#endif /* NLA3D_GPU_H */
