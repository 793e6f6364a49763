// Kernels of the learned Newton start: a small multilayer perceptron whose
// weights are stored in BF16 and whose products accumulate in FP32.  No
// counterpart in the reference (which always starts Newton from the previous
// converged state).
//
//   gemm:        C[m,n] = act( sum_k A[m,k] B[k,n] + bias[n] )  (A, B FP32 or BF16,
//                arbitrary strides so that X W^T, dZ^T X and dZ W use one kernel)
//   tanh_bwd:    dZ = dY * (1 - Y^2)
//   column_sum:  s[n] = sum_m X[m,n]            (bias gradient)
//   mse_grad:    dY = scale * (Y - T)
//   adam:        FP32 master weights, moments, BF16 copy refreshed in place
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nla3d_gpu.h"

namespace {

constexpr int kTile = 64;   // C tile per block
constexpr int kTileK = 16;  // K slice per shared-memory stage
constexpr int kThreads = 256;

__device__ __forceinline__ float load_elem(const void* p, int bf16, long i) {
  if (bf16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(p)[i]);
  return reinterpret_cast<const float*>(p)[i];
}

// 64x64 tile of C per block, 4x4 outputs per thread, FP32 accumulation.
__global__ void __launch_bounds__(kThreads)
    gemm_kernel(int M, int N, int K, const void* A, int a_bf16, long lda_m, long lda_k,
                const void* B, int b_bf16, long ldb_k, long ldb_n, float* C, long ldc,
                const float* bias, int act) {
  __shared__ float As[kTileK][kTile + 1];
  __shared__ float Bs[kTileK][kTile + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTileK) {
    for (int i = threadIdx.x; i < kTileK * kTile; i += kThreads) {
      const int kk = i / kTile, mm = i % kTile;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? load_elem(A, a_bf16, (long)m * lda_m + (long)k * lda_k) : 0.f;
      const int n = n0 + mm;
      Bs[kk][mm] = (n < N && k < K) ? load_elem(B, b_bf16, (long)k * ldb_k + (long)n * ldb_n) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTileK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j] + (bias ? bias[n] : 0.f);
      if (act == 1) v = tanhf(v);
      C[(long)m * ldc + n] = v;
    }
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
  if (M < 0 || N < 0 || K < 0 || !A || !B || !C || (act != 0 && act != 1)) return NLA3D_ERR_ARG;
  if (M == 0 || N == 0) return NLA3D_OK;
  const dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  gemm_kernel<<<grid, kThreads, 0, (cudaStream_t)stream>>>(M, N, K, A, a_bf16, lda_m, lda_k, B,
                                                          b_bf16, ldb_k, ldb_n, C, ldc, bias, act);
  return status(cudaGetLastError());
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
