// SOLID81 assembly that performs no device allocation.
//
// Some programs that embed this assembly cannot let it call cudaMalloc: a host
// framework that hands out all device memory from its own pool and does not
// allow a plugin to allocate behind its back, or a time-critical solve loop
// where cudaMalloc's implicit device synchronisation and unpredictable cost
// are not acceptable.  For them nla3d_assemble_solid81_noalloc() takes every
// input and output as a device pointer owned by the caller and keeps its
// intermediate data (per-Gauss-point shape-function gradients and the element
// contributions) in a fixed array compiled into this library.
//
// The array, g_noalloc_scratch, is NLA3D_NOALLOC_SCRATCH_BYTES (64 MiB) of
// device memory that every GPU which loads the library holds until the
// process exits.  It is shared by all calls: a call leaves its data behind,
// and two calls whose kernels overlap on the GPU (different streams, or
// different host threads, without ordering between them) corrupt each
// other's results.  The element-status counter that must start at zero is
// cleared by every call; the rest of the scratch is fully rewritten before it
// is read.
//
// Device set-up: the host cannot use the array's name as a device address, so
// the first call on each device, with that device current, asks the runtime
// for the address (cudaGetSymbolAddress) and caches it, and uploads the
// element kernel's constant table.  That first call should therefore come
// before any stream capture on that device.  The cache is keyed by device
// ordinal and assumes the device's primary context for the life of the
// process: after cudaDeviceReset(), or under another driver-API context on
// the same device, the cached addresses no longer apply.
//
// Input check: the caller's index arrays are device memory, so they are
// checked on the device, by the first kernel of each call: node ids in
// 1..n_nodes, equation numbers in 1..n_eq, gather offsets non-decreasing and
// at most 325 (25) per element, contribution ids below 325 * n_elems
// (25 * n_elems).  If any is out of range, the kernels that follow do
// nothing (no out-of-bounds access; K and F are left as they were) and, when
// the caller asks for the flagged count, the call returns NLA3D_ERR_ARG.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/nla3d_gpu.h"
#include "kernels.cuh"

using namespace nla3d_gpu;

namespace {

constexpr uint64_t kScratchDoubles = NLA3D_NOALLOC_SCRATCH_BYTES / sizeof(double);
// per element: Gt (24 x 8) + w det J (8) + K contributions (325) + F contributions (25)
constexpr uint64_t kDoublesPerElem = 24 * 8 + 8 + kSolidKc + kSolidFc;
static_assert(NLA3D_NOALLOC_MAX_ELEMS * kDoublesPerElem <= kScratchDoubles,
              "NLA3D_NOALLOC_MAX_ELEMS does not fit the scratch array");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];
static __device__ __align__(256) ElementStatus g_noalloc_status;
static __device__ __align__(256) uint32_t g_noalloc_bad;  // invalid input entries found

// One pass over the caller's index arrays (grid-stride over the longest).
__global__ void check_inputs_kernel(const nla3d_solid81_noalloc_args a, uint32_t* bad) {
  const uint64_t E = a.n_elems, nK = (uint64_t)kSolidKc * E, nF = (uint64_t)kSolidFc * E;
  uint64_t n = nK > a.nnz + 1 ? nK : a.nnz + 1;
  if ((uint64_t)a.n_eq + 1 > n) n = (uint64_t)a.n_eq + 1;
  uint32_t found = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (i < 8 * E) {
      const uint32_t nid = a.conn[i];
      if (nid == 0 || nid > a.n_nodes) {
        found++;
      } else {
        for (int c = 0; c < 3; c++) {
          const uint32_t eq = a.node_eq[4 * (uint64_t)(nid - 1) + c];
          if (eq == 0 || eq > a.n_eq) found++;
        }
      }
    }
    if (i < E && (a.p_eq[i] == 0 || a.p_eq[i] > a.n_eq)) found++;
    if (i < nK && a.k_ids[i] >= nK) found++;
    if (i < nF && a.f_ids[i] >= nF) found++;
    if (i <= a.nnz) {
      const uint32_t v = a.k_ptr[i];
      if (v > nK || (i < a.nnz && v > a.k_ptr[i + 1])) found++;
    }
    if (i <= a.n_eq) {
      const uint32_t v = a.f_ptr[i];
      if (v > nF || (i < a.n_eq && v > a.f_ptr[i + 1])) found++;
    }
  }
  if (found) atomicAdd(bad, found);
}

constexpr int kMaxDevices = 64;
struct DeviceScratch {
  bool ready = false;
  double* scratch = nullptr;
  ElementStatus* status = nullptr;
  uint32_t* bad = nullptr;
};
DeviceScratch g_dev[kMaxDevices];
std::mutex g_mutex;

int device_scratch(DeviceScratch** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return NLA3D_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return NLA3D_ERR_RANGE;
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceScratch& d = g_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return NLA3D_ERR_CUDA;
    d.scratch = static_cast<double*>(p);
    p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_status) != cudaSuccess || !p) return NLA3D_ERR_CUDA;
    d.status = static_cast<ElementStatus*>(p);
    p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_bad) != cudaSuccess || !p) return NLA3D_ERR_CUDA;
    d.bad = static_cast<uint32_t*>(p);
    // the element kernel's constant table (a synchronous upload, done here so
    // that later calls enqueue work only)
    if (prepare_device_tables() != cudaSuccess) return NLA3D_ERR_CUDA;
    d.ready = true;
  }
  *out = &d;
  return NLA3D_OK;
}

}  // namespace

extern "C" int nla3d_assemble_solid81_noalloc(const nla3d_solid81_noalloc_args* a, void* stream,
                                              uint32_t* flagged) {
  if (!a) return NLA3D_ERR_ARG;
  if (a->n_elems > NLA3D_NOALLOC_MAX_ELEMS) return NLA3D_ERR_RANGE;
  if (a->n_elems == 0 || a->n_nodes == 0 || a->n_eq == 0 || !a->xyz || !a->conn ||
      !a->node_eq || !a->p_eq || !a->U ||
      !a->k_ptr || !a->k_ids || !a->f_ptr || !a->f_ids || !a->K || !a->F)
    return NLA3D_ERR_ARG;
  if (a->mat_id < NLA3D_MAT_NEO_HOOKEAN || a->mat_id > NLA3D_MAT_MOONEY_RIVLIN) return NLA3D_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(a->node_eq) & 15u) != 0) return NLA3D_ERR_ARG;  // 16-byte loads
  DeviceScratch* d = nullptr;
  int rc = device_scratch(&d);
  if (rc != NLA3D_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t E = a->n_elems;
  double* Gt = d->scratch;
  double* wdet = Gt + 24 * 8 * E;
  double* contribK = wdet + 8 * E;
  double* contribF = contribK + kSolidKc * E;

  // the only scratch that must start from a known value: the status word and
  // the invalid-input count
  if (cudaMemsetAsync(d->status, 0, sizeof(ElementStatus), s) != cudaSuccess ||
      cudaMemsetAsync(&d->status->first, 0xFF, sizeof(uint32_t), s) != cudaSuccess ||
      cudaMemsetAsync(d->bad, 0, sizeof(uint32_t), s) != cudaSuccess)
    return NLA3D_ERR_CUDA;

  check_inputs_kernel<<<304, 256, 0, s>>>(*a, d->bad);
  if (cudaGetLastError() != cudaSuccess) return NLA3D_ERR_CUDA;

  JacobianArgs ja{a->n_elems, a->xyz, a->conn, Gt, wdet, d->status};
  ja.skip = d->bad;
  if (launch_solid81_jacobian(ja, s) != cudaSuccess) return NLA3D_ERR_CUDA;

  Solid81Args ea{};
  ea.n_elems = a->n_elems;
  ea.Gt = Gt;
  ea.wdet = wdet;
  ea.conn = a->conn;
  ea.node_eq3 = a->node_eq;
  ea.p_eq = a->p_eq;
  ea.U_state = a->U;  // updateResults() and assembleGlobalEqMatrices() on the same U
  ea.U_cur = a->U;
  ea.have_state = 1;
  ea.mat_id = a->mat_id;
  for (int i = 0; i < 5; i++) ea.mc[i] = a->mat_c[i];
  ea.kbulk = a->mat_id == NLA3D_MAT_NEO_HOOKEAN ? a->mat_c[1]
                                                : (a->mat_id == NLA3D_MAT_BIDERMAN ? a->mat_c[4]
                                                                                   : a->mat_c[2]);
  ea.contribK = contribK;
  ea.contribF = contribF;
  ea.status = d->status;
  ea.skip = d->bad;
  if (launch_solid81(ea, false, 0, s) != cudaSuccess) return NLA3D_ERR_CUDA;

  GatherArgs gk{a->nnz, a->k_ptr, a->k_ids, contribK, a->K};
  gk.skip = d->bad;
  if (launch_gather(gk, s) != cudaSuccess) return NLA3D_ERR_CUDA;
  GatherArgs gf{a->n_eq, a->f_ptr, a->f_ids, contribF, a->F};
  gf.skip = d->bad;
  if (launch_gather(gf, s) != cudaSuccess) return NLA3D_ERR_CUDA;

  if (flagged) {
    ElementStatus st{0, 0};
    uint32_t bad = 0;
    if (cudaMemcpyAsync(&st, d->status, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&bad, d->bad, sizeof(bad), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return NLA3D_ERR_CUDA;
    *flagged = st.count;
    if (bad) return NLA3D_ERR_ARG;
    if (st.count) return NLA3D_ERR_ELEMENT;
  }
  return NLA3D_OK;
}
