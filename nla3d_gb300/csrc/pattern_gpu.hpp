// Device build of one mesh's CSR pattern, slot maps and gather lists
// (pattern_gpu.cu); the host builder's results, computed on the GPU.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>

#include "host_model.hpp"

namespace nla3d_gpu {

// gather lists left on the device: K slot s sums contributions
// k_ids[k_ptr[s] .. k_ptr[s+1]) (ids e * n_kc + c, ascending); k_pos is the
// inverse (contribution -> position); the same for F rows
struct PatternDevice {
  uint32_t* k_ptr = nullptr;
  uint32_t* k_ids = nullptr;
  uint32_t* k_pos = nullptr;
  uint32_t* f_ptr = nullptr;
  uint32_t* f_ids = nullptr;
  uint32_t* f_pos = nullptr;
};

// device allocation owned by the caller (freed with the context)
using DeviceAlloc = std::function<cudaError_t(void**, size_t)>;

// m must hold the numbering (build_host_numbering).  On success ("") m holds
// the pattern (blk, val_off, nnz_total, n_kc, n_fc) and the MPC term slots,
// and *out the device gather lists.  A message starting with "fallback:"
// means the mesh is outside the device builder's limits.
std::string build_pattern_gpu(HostModel& m, cudaStream_t s, const DeviceAlloc& alloc,
                              PatternDevice* out);

}  // namespace nla3d_gpu
