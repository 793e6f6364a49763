// Device-side argument blocks and launchers of the assembly kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nla3d_gpu {

constexpr int kSolidKc = 325;  // SOLID81 K contributions per element (300 Kuu + 24 Kup + 1 Kpp)
constexpr int kSolidFc = 25;   // SOLID81 F contributions per element (24 Fu + 1 Fp)

struct ElementStatus {
  uint32_t count;  // elements flagged (J <= 0, det J <= 0, non-finite)
  uint32_t first;  // smallest flagged 1-based element number, 0xFFFFFFFF if none
};

struct Solid81Args {
  uint32_t n_elems;
  const double* Gt;         // dN/dX, structure of arrays: Gt[c * E8 + e*8 + g], c = 3*node + dim
  const double* wdet;       // Gauss weight * det J, [e*8 + g]
  const uint32_t* conn;     // 8 node ids per element, 1-based
  const uint32_t* node_eq3; // per node: equation numbers of UX, UY, UZ (1-based), 4 per node
  const uint32_t* p_eq;     // per element: equation number of HYDRO_PRESSURE
  const double* U_state;    // vecU captured by the last updateResults()
  const double* U_cur;      // current vecU
  int have_state;           // 0: state of Element::pre() (C = I, S = 0, O = 0)
  int mat_id;
  double mc[5];
  double kbulk;
  // optional per-element material (several meshes in one launch): when
  // elem_mesh != nullptr, element e uses mesh_mat[8 * elem_mesh[e] + ...] =
  // (mat_id, c0..c4, K, 1/K) instead of mat_id / mc / kbulk
  const uint32_t* elem_mesh;
  const double* mesh_mat;
  // optional slot-ordered output: contribution c of element e goes to
  // contribK[kpos[e * 325 + c]] (contribF[fpos[e * 25 + c]]); nullptr = e * 325 + c
  const uint32_t* kpos;
  const uint32_t* fpos;
  double* contribK;         // [E * 325]
  double* contribF;         // [E * 25]
  ElementStatus* status;
  // element range [e_begin, n_elems) of a mesh of n_total elements (the
  // structure-of-arrays stride of Gt); e_begin a multiple of 4; n_total 0
  // means n_elems
  uint32_t e_begin;
  uint32_t n_total;
  // mixed precision only: inputs of the residual as float pairs (hi, lo)
  // with hi + lo = the double to 2^-48 (Gdf replaces Gt, same layout); the
  // residual is computed in float-pair arithmetic
  const float2* Gdf;
  const float2* wdf;        // w det J
  float2 mcd[5];            // material constants
  float2 inv_kbd;           // 1 / K
  double inv_kb;            // 1 / K in FP64 (the mixed kernel's volumetric terms)
  const float2* mesh_mat_df;  // per mesh: 8 pairs (-, c0..c4, K, 1/K) when elem_mesh != nullptr
  // optional: a device word; when non-null and non-zero the launch does
  // nothing (set by a kernel that found invalid indices in the inputs)
  const uint32_t* skip;
};

struct JacobianArgs {
  uint32_t n_elems;
  const double* xyz;
  const uint32_t* conn;
  double* Gt;               // FP64 dN/dX, or nullptr
  double* wdet;
  ElementStatus* status;
  float2* Gdf;              // the same as float pairs (mixed precision), or nullptr
  float2* wdf;
  // optional: a device word; when non-null and non-zero the launch does
  // nothing (set by a kernel that found invalid indices in the inputs)
  const uint32_t* skip;
};

struct GatherArgs {
  uint64_t n_slots;
  const uint32_t* ptr;   // n_slots + 1
  const uint32_t* ids;   // contribution ids
  const double* contrib;
  double* out;
  uint64_t s_begin;      // slot range [s_begin, n_slots)
  // optional: a device word; when non-null and non-zero the launch does
  // nothing (set by a kernel that found invalid indices in the inputs)
  const uint32_t* skip;
};

struct MpcArgs {
  uint32_t n_mpc;
  const uint32_t* master;     // per MPC: master node
  const uint32_t* slave;      // per MPC: slave node
  const int32_t* slave_dof;   // per MPC: UX/UY/UZ
  const uint32_t* eq;         // per MPC: its equation number
  const uint32_t* master_eq6; // per MPC: eqs of master UX,UY,UZ,ROTX,ROTY,ROTZ (6 each)
  const uint32_t* slave_eq;   // per MPC: eq of the slave DoF
  const uint32_t* slot;       // per MPC: 5 K slots
  const double* xyz;
  const double* U;
  double* K;                  // concatenated K values
  double* F;
};

constexpr int kEparamStride = 4;  // per-element parameters: TETRA0 (E, my, -, -),
                                  // QUADTH (k, volFlux, rho, c)

struct LinearArgs {
  int etype;
  uint32_t n_elems;
  const double* xyz;
  const uint32_t* conn;
  const double* eparams;           // kEparamStride per element
  double* contribK;
  double* contribF;
  ElementStatus* status;
  const uint32_t* kpos;  // optional slot-ordered output (as Solid81Args)
  const uint32_t* fpos;
  uint32_t e_begin;      // element range [e_begin, n_elems)
  double* contribC;      // QUADTH capacity contributions [E * 10] (transient), or null
};

// SurfaceLINETH (QUADTH.cpp:86-121): convection and flux on 2-node lines,
// one thread per line; K contributions (0,0), (0,1), (1,1) at contribK[k_off
// + 3 l + c], F contributions at contribF[f_off + 2 l + c].
struct LineArgs {
  uint32_t n_lines;
  const double* xyz;
  const uint32_t* conn;    // 2 node ids per line
  const double* par;       // (htc, flux, etemp0, etemp1) per line
  uint64_t k_off, f_off;
  const uint32_t* kpos;
  const uint32_t* fpos;
  double* contribK;
  double* contribF;
  ElementStatus* status;
  uint32_t first_elem;     // element number of line 0 (for the status word)
};

// PLANE41 (PLANE41.cpp:29-146): 4-node plane-strain u/p quad, one thread per
// element, FP64; Gauss-point state (O, C, S) recomputed from U_state as
// updateResults() leaves it, tangent and residual with the current pressure.
struct Plane41Args {
  uint32_t e_begin, n_elems;  // element range [e_begin, n_elems)
  const double* xyz;
  const uint32_t* conn;       // 4 node ids per element, 1-based
  const uint32_t* node_eq3;   // per node: equations of UX, UY, UZ (4 per node)
  const uint32_t* p_eq;
  const double* U_state;
  const double* U_cur;
  int have_state;
  int mat_id;
  double mc[5];
  double kbulk;
  const uint32_t* elem_mesh;  // optional per-element material, as Solid81Args
  const double* mesh_mat;
  const uint32_t* kpos;       // optional slot-ordered output, as Solid81Args
  const uint32_t* fpos;
  double* contribK;           // [E * 45]
  double* contribF;           // [E * 9]
  ElementStatus* status;
};

// Contiguous segmented sums: out[s] = sum of contrib[ptr[s] .. ptr[s+1]) in
// ascending order, starting from 0.
struct SegSumArgs {
  uint64_t n_slots;
  const uint32_t* ptr;
  const double* contrib;
  double* out;
  uint64_t s_begin;      // slot range [s_begin, n_slots)
  // optional: a device word; when non-null and non-zero the launch does
  // nothing (set by a kernel that found invalid indices in the inputs)
  const uint32_t* skip;
};

// Linear MPC rows (FEStorage.cpp:49-60 for an Mpc added with addMpc): one
// thread per equation: F[eq] = b, then K[slot_t] += coef_t in term order.
struct LinearMpcArgs {
  uint32_t n;
  const uint32_t* eq;     // per equation (1-based global equation)
  const double* b;        // per equation
  const uint32_t* ptr;    // n + 1: its terms
  const uint32_t* slot;   // per term: K slot
  const double* coef;     // per term
  double* K;
  double* F;
};

// y[r] += sum over the walk list of r of (K[slot] * x[xi]) * coef, in list
// order (the reference's matBVprod / matBTVprod order, SparseMatrix.cpp:497-558);
// sym: skip |x| <= 1e-20 as the symmetric product does.
struct BlockMvArgs {
  uint64_t n_out;
  const uint32_t* ptr;   // n_out + 1
  const uint32_t* slot;  // value index within the block
  const uint32_t* xi;    // index into x
  const double* K;       // the block's values
  const double* x;
  double coef;
  double* y;
  int sym;
};

// Launchers (return cudaError_t of the launch).
cudaError_t launch_solid81_jacobian(const JacobianArgs& a, cudaStream_t s);
cudaError_t launch_solid81(const Solid81Args& a, bool mixed, int blocks_per_sm_hint,
                           cudaStream_t s);
// Launch shape of the SOLID81 element kernel: warps per block (2, 4 or 8) and
// resident blocks per SM (0 = as many as fit).
struct Solid81Shape {
  int warps_per_block = 4;
  int blocks_per_sm = 0;
};
cudaError_t launch_solid81_shaped(const Solid81Args& a, bool mixed, Solid81Shape shape,
                                  cudaStream_t s);
int solid81_max_blocks_per_sm(bool mixed, int warps_per_block);
cudaError_t launch_gather_bs(const GatherArgs& a, int block_size, cudaStream_t s);
cudaError_t launch_segsum(const SegSumArgs& a, int block_size, cudaStream_t s);
// kernel tables (constant memory) for the current device; call before any
// stream capture
cudaError_t prepare_device_tables();
cudaError_t launch_gather(const GatherArgs& a, cudaStream_t s);
cudaError_t launch_mpc(const MpcArgs& a, cudaStream_t s);
cudaError_t launch_block_mv(const BlockMvArgs& a, cudaStream_t s);
// per K slot: the index of the element range (bounds eb[0..n], n <= 255) that
// holds the last element contributing to it (contribution ids e * n_kc + c,
// ascending within a slot)
cudaError_t launch_slot_last_range(uint64_t n_slots, const uint32_t* ptr, const uint32_t* ids,
                                   uint32_t n_kc, const uint32_t* eb, int n, uint8_t* out,
                                   cudaStream_t s);
cudaError_t launch_linear_mpc(const LinearMpcArgs& a, cudaStream_t s);
cudaError_t launch_linear(const LinearArgs& a, cudaStream_t s);
cudaError_t launch_plane41(const Plane41Args& a, cudaStream_t s);
cudaError_t launch_lines(const LineArgs& a, cudaStream_t s);
size_t solid81_smem_bytes(bool mixed);
cudaError_t probe_fma_peak(bool fp64, double* flops);

}  // namespace nla3d_gpu
