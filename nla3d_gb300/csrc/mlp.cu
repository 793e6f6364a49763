// Kernels of the learned Newton start: a small multilayer perceptron whose
// weights are stored in BF16 and whose products accumulate in FP32.  No
// counterpart in the reference (which always starts Newton from the previous
// converged state).
//
//   gemm:        C[m,n] = act( sum_k A[m,k] B[k,n] + bias[n] )  (A, B FP32 or BF16,
//                arbitrary strides so that X W^T, dZ^T X and dZ W use one kernel),
//                on the tensor cores (tcgen05, BF16 operands, FP32 accumulation)
//   tanh_bwd:    dZ = dY * (1 - Y^2)
//   column_sum:  s[n] = sum_m X[m,n]            (bias gradient)
//   mse_grad:    dY = scale * (Y - T)
//   adam:        FP32 master weights, moments, BF16 copy refreshed in place
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nla3d_gpu.h"

namespace {

// ---- C = act(A B + bias) on the tensor cores (tcgen05.mma kind::f16, BF16) ----
//
// One CTA (256 threads) per 128 x 128 tile of C, K in chunks of 32.  Both
// operands are staged in shared memory as BF16 in the canonical K-major
// layout without swizzle (8-row x 16-byte core matrices; K-adjacent cores
// 128 B apart, 8-row groups 512 B apart): A as its 128 rows m, B as its 128
// columns n (the MMA computes D[m][n] = sum_k A[m][k] B'[n][k]).  An FP32
// operand (activations, gradients) is split into a BF16 high part and the
// BF16 rounding of the remainder, x = hi + lo + O(2^-16 |x|); a BF16 operand
// (the weights) is exact as it is.  One thread issues, per 16-wide K step,
// hi.hi, then hi.lo and lo.hi where an operand has a low part (BF16 x BF16
// products are exact in FP32), accumulating in FP32 in 128 TMEM columns, and
// commits them to an mbarrier; the next chunk is staged once they have
// released the buffers.  The epilogue reads TMEM (warp w: lanes 32 (w % 4)
// .. +31 = rows, columns 64 (w / 4) .. +63), adds the bias, applies the
// activation and stores FP32.  Every wait is bounded: on a timeout the
// tile's outputs are set to NaN and g_mlp_timeouts is incremented.
constexpr int kTcM = 128, kTcN = 128, kTcK = 32;
constexpr int kThreads = 256;
constexpr uint32_t kTileElems = kTcM * kTcK;                      // one 128 x 32 operand
constexpr size_t kTcSmem = 4 * kTileElems * sizeof(__nv_bfloat16) + 64;
// instruction descriptor: D F32 (bit 4), A and B BF16 (bits 7, 10), both
// K-major, N / 8 at bit 17, M / 16 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                            ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
constexpr long long kSpinLimit = 1ll << 26;

__device__ unsigned int g_mlp_timeouts;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, leading (K) and stride (8-row) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t mat_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (long long it = 0; it < kSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ float load_elem(const void* p, int bf16, long i) {
  if (bf16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(p)[i]);
  return reinterpret_cast<const float*>(p)[i];
}

// 16 consecutive K values of one operand row into the hi / lo tiles
// (8 bf16 = one 16-byte core-matrix row per store)
__device__ __forceinline__ void stage_row(__nv_bfloat16* hi, __nv_bfloat16* lo, bool split,
                                          int r, int kq, const float v[16]) {
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int k = kq * 16 + half * 8;
    const uint32_t off = (uint32_t)(((r >> 3) * (kTcK / 8) + (k >> 3)) * 64 + (r & 7) * 8);
    __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float x = v[half * 8 + q];
      h[q] = __float2bfloat16_rn(x);
      l[q] = __float2bfloat16_rn(x - __bfloat162float(h[q]));
    }
    *reinterpret_cast<uint4*>(hi + off) = *reinterpret_cast<const uint4*>(h);
    if (split) *reinterpret_cast<uint4*>(lo + off) = *reinterpret_cast<const uint4*>(l);
  }
}

__global__ void __launch_bounds__(kThreads)
    tc_gemm_kernel(int M, int N, int K, const void* __restrict__ A, int a_bf16, long lda_m,
                   long lda_k, const void* __restrict__ B, int b_bf16, long ldb_k, long ldb_n,
                   float* __restrict__ C, long ldc, const float* __restrict__ bias, int act) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __nv_bfloat16* Ahi = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* Alo = Ahi + kTileElems;
  __nv_bfloat16* Bhi = Alo + kTileElems;
  __nv_bfloat16* Blo = Bhi + kTileElems;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(Blo + kTileElems);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
  const bool a_split = !a_bf16, b_split = !b_bf16;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(kTcN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int r = threadIdx.x % kTcM, kq = threadIdx.x / kTcM;  // operand row, which 16 of 32
  const int ma = m0 + r, nb = n0 + r;
  const uint32_t lbo = 128, sbo = (kTcK / 8) * 128;
  const int n_chunks = (K + kTcK - 1) / kTcK;
  bool ok = true;
  for (int c = 0; c < n_chunks && ok; c++) {
    if (c > 0) ok = mbar_wait(smem_addr(mbar), (uint32_t)(c - 1) & 1u);  // buffers released
    if (ok) {
      float av[16], bv[16];
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int k = c * kTcK + kq * 16 + q;
        av[q] = (ma < M && k < K) ? load_elem(A, a_bf16, (long)ma * lda_m + (long)k * lda_k) : 0.f;
        bv[q] = (nb < N && k < K) ? load_elem(B, b_bf16, (long)k * ldb_k + (long)nb * ldb_n) : 0.f;
      }
      stage_row(Ahi, Alo, a_split, r, kq, av);
      stage_row(Bhi, Blo, b_split, r, kq, bv);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (ok && threadIdx.x == 0) {
      const uint32_t ahi = smem_addr(Ahi), alo = smem_addr(Alo);
      const uint32_t bhi = smem_addr(Bhi), blo = smem_addr(Blo);
#pragma unroll
      for (int st = 0; st < kTcK / 16; st++) {
        const uint32_t koff = st * 256;   // 16 K values = two core matrices
        const uint64_t dah = mat_desc(ahi + koff, lbo, sbo), dbh = mat_desc(bhi + koff, lbo, sbo);
        mma_bf16(tmem, dah, dbh, (c > 0 || st > 0) ? 1u : 0u);
        if (b_split) mma_bf16(tmem, dah, mat_desc(blo + koff, lbo, sbo), 1u);
        if (a_split) mma_bf16(tmem, mat_desc(alo + koff, lbo, sbo), dbh, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr(mbar))
          : "memory");
    }
  }
  if (ok && n_chunks > 0) ok = mbar_wait(smem_addr(mbar), (uint32_t)(n_chunks - 1) & 1u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  const int row = (warp & 3) * 32 + lane;
  const int m = m0 + row;
  for (int c0 = (warp >> 2) * 64; c0 < (warp >> 2) * 64 + 64; c0 += 16) {
    uint32_t v[16];
    if (ok && n_chunks > 0) {
      const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
          "%11, %12, %13, %14, %15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    } else {
#pragma unroll
      for (int q = 0; q < 16; q++) v[q] = ok ? 0u : 0x7FC00000u;   // K = 0: zero; timeout: NaN
    }
    if (m < M)
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int n = n0 + c0 + q;
        if (n < N) {
          float y = __uint_as_float(v[q]) + (bias ? bias[n] : 0.f);
          if (act == 1) y = tanhf(y);
          C[(long)m * ldc + n] = y;
        }
      }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    if (!ok) {
      // after a timeout the MMAs may still run: one more bounded wait on each phase
      if (lane == 0) atomicAdd(&g_mlp_timeouts, 1u);
      mbar_wait(smem_addr(mbar), 0);
      mbar_wait(smem_addr(mbar), 1);
    }
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcN));
  }
}

__global__ void tanh_bwd_kernel(const float* Y, float* dY, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dY[i] *= 1.0f - Y[i] * Y[i];
}

// one block per 32 columns; threads stride over the rows, fixed order
__global__ void column_sum_kernel(const float* X, long rows, long cols, float* out) {
  __shared__ float part[8][33];
  const int c = blockIdx.x * 32 + (threadIdx.x % 32);
  const int r0 = threadIdx.x / 32;  // 0..7
  float s = 0.f;
  if (c < cols)
    for (long r = r0; r < rows; r += 8) s += X[r * cols + c];
  part[r0][threadIdx.x % 32] = s;
  __syncthreads();
  if (r0 == 0 && c < cols) {
    float t = 0.f;
    for (int k = 0; k < 8; k++) t += part[k][threadIdx.x % 32];
    out[c] = t;
  }
}

__global__ void adam_kernel(float* w, const float* g, float* m, float* v, long n, float lr,
                            float b1, float b2, float eps, float c1, float c2,
                            __nv_bfloat16* w_bf16) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (w_bf16) w_bf16[i] = __float2bfloat16_rn(wi);
}

__global__ void mse_grad_kernel(const float* Y, const float* T, float* dY, long n, float scale) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dY[i] = scale * (Y[i] - T[i]);
}

__global__ void to_bf16_kernel(const float* x, __nv_bfloat16* y, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

int status(cudaError_t e) { return e == cudaSuccess ? NLA3D_OK : NLA3D_ERR_CUDA; }

}  // namespace

extern "C" {

int nla3d_mlp_gemm(int M, int N, int K, const void* A, int a_bf16, int64_t lda_m, int64_t lda_k,
                   const void* B, int b_bf16, int64_t ldb_k, int64_t ldb_n, float* C, int64_t ldc,
                   const float* bias, int act, void* stream) {
  if (M < 0 || N < 0 || K < 0 || (K > 0 && (!A || !B)) || !C || (act != 0 && act != 1))
    return NLA3D_ERR_ARG;
  if (M == 0 || N == 0) return NLA3D_OK;
  const dim3 grid((N + kTcN - 1) / kTcN, (M + kTcM - 1) / kTcM);
  tc_gemm_kernel<<<grid, kThreads, kTcSmem, (cudaStream_t)stream>>>(
      M, N, K, A, a_bf16, lda_m, lda_k, B, b_bf16, ldb_k, ldb_n, C, ldc, bias, act);
  return status(cudaGetLastError());
}

int nla3d_mlp_status(uint32_t* timeouts) {
  if (!timeouts) return NLA3D_ERR_ARG;
  unsigned int v = 0, zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_mlp_timeouts, sizeof(v));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_mlp_timeouts, &zero, sizeof(zero));
  *timeouts = v;
  return status(e);
}

int nla3d_mlp_tanh_backward(const float* Y, float* dY, int64_t n, void* stream) {
  if (!Y || !dY || n < 0) return NLA3D_ERR_ARG;
  if (n == 0) return NLA3D_OK;
  tanh_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(Y, dY, n);
  return status(cudaGetLastError());
}

int nla3d_mlp_column_sum(const float* X, int64_t rows, int64_t cols, float* out, void* stream) {
  if (!X || !out || rows < 0 || cols < 0) return NLA3D_ERR_ARG;
  if (cols == 0) return NLA3D_OK;
  column_sum_kernel<<<(unsigned)((cols + 31) / 32), 256, 0, (cudaStream_t)stream>>>(X, rows, cols,
                                                                                     out);
  return status(cudaGetLastError());
}

int nla3d_mlp_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float beta1,
                   float beta2, float eps, int step, uint16_t* w_bf16, void* stream) {
  if (!w || !g || !m || !v || n < 0 || step < 1) return NLA3D_ERR_ARG;
  if (n == 0) return NLA3D_OK;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      w, g, m, v, n, lr, beta1, beta2, eps, c1, c2, reinterpret_cast<__nv_bfloat16*>(w_bf16));
  return status(cudaGetLastError());
}

int nla3d_mlp_mse_grad(const float* Y, const float* T, float* dY, int64_t n, float scale,
                       void* stream) {
  if (!Y || !T || !dY || n < 0) return NLA3D_ERR_ARG;
  if (n == 0) return NLA3D_OK;
  mse_grad_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(Y, T, dY, n,
                                                                                  scale);
  return status(cudaGetLastError());
}

int nla3d_mlp_to_bf16(const float* x, uint16_t* y, int64_t n, void* stream) {
  if (!x || !y || n < 0) return NLA3D_ERR_ARG;
  if (n == 0) return NLA3D_OK;
  to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      x, reinterpret_cast<__nv_bfloat16*>(y), n);
  return status(cudaGetLastError());
}

}  // extern "C"
