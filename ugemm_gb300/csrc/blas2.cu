// blas2.cu -- SAXPY and SGEMV on the GPU (the reference's saxpy_cpu and
// sgemv_cpu, ugemm.h:86-160).  Both are HBM-bound: every element of x / A is
// read once with coalesced loads; reductions are done in a fixed order, so
// results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"

namespace ugemm {
namespace {

// y[i*incy] += alpha * x[i*incx]  (ugemm.h:86-97)
__global__ void saxpy_kernel(int n, float alpha, const float* __restrict__ x, int incx,
                             float* __restrict__ y, int incy) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (incx == 1 && incy == 1 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0) {
    const long long n4 = n / 4;
    for (long long v = i; v < n4; v += stride) {
      const float4 a = reinterpret_cast<const float4*>(x)[v];
      float4 b = reinterpret_cast<float4*>(y)[v];
      b.x += alpha * a.x; b.y += alpha * a.y; b.z += alpha * a.z; b.w += alpha * a.w;
      reinterpret_cast<float4*>(y)[v] = b;
    }
    for (long long t = n4 * 4 + i; t < n; t += stride) y[t] += alpha * x[t];
    return;
  }
  for (; i < n; i += stride) y[i * incy] += alpha * x[i * incx];
}

// 'N': A is column-major M x N (A[m + n*lda]); y[m] = alpha * sum_n A[m,n] x[n]
// + beta * y[m].  A block owns 32 rows; its 8 warps take every 8th column and
// the 8 partial sums are added in a fixed order.
__global__ void __launch_bounds__(256) sgemv_n_kernel(int M, int N, float alpha,
                                                      const float* __restrict__ A, int lda,
                                                      const float* __restrict__ x, int incx,
                                                      float beta, float* __restrict__ y, int incy) {
  __shared__ float part[8][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int m = blockIdx.x * 32 + lane;
  float s = 0.f;
  if (m < M)
    for (int n = w; n < N; n += 8) s += A[m + static_cast<long long>(n) * lda] * x[static_cast<long long>(n) * incx];
  part[w][lane] = s;
  __syncthreads();
  if (w == 0 && m < M) {
    float t = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) t += part[j][lane];
    float* yp = y + static_cast<long long>(m) * incy;
    *yp = (beta == 0.f) ? alpha * t : alpha * t + beta * *yp;
  }
}

// 'T': A is column-major N x M (A[n + m*lda]); y[m] = alpha * sum_n A[n,m] x[n]
// + beta * y[m].  One warp per output, coalesced along the column, reduced by
// a fixed shuffle tree.
__global__ void __launch_bounds__(256) sgemv_t_kernel(int M, int N, float alpha,
                                                      const float* __restrict__ A, int lda,
                                                      const float* __restrict__ x, int incx,
                                                      float beta, float* __restrict__ y, int incy) {
  const int lane = threadIdx.x & 31;
  const int m = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (m >= M) return;
  const float* col = A + static_cast<long long>(m) * lda;
  float s = 0.f;
  for (int n = lane; n < N; n += 32) s += col[n] * x[static_cast<long long>(n) * incx];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    float* yp = y + static_cast<long long>(m) * incy;
    *yp = (beta == 0.f) ? alpha * s : alpha * s + beta * *yp;
  }
}

}  // namespace
}  // namespace ugemm

using namespace ugemm;

extern "C" {

UGEMM_API int ugemm_saxpy(int N, float alpha, const float* x, int incx, float* y, int incy,
                          void* stream) {
  if (N < 0 || incx <= 0 || incy <= 0) return UGEMM_ERR_ARG;
  if (N == 0) return UGEMM_OK;
  if (!x || !y) return UGEMM_ERR_ARG;
  const int grid = static_cast<int>(std::min<long long>((N + 1023) / 1024, 152LL * 16));
  prof_begin(static_cast<cudaStream_t>(stream));
  saxpy_kernel<<<std::max(grid, 1), 256, 0, static_cast<cudaStream_t>(stream)>>>(N, alpha, x, incx,
                                                                                y, incy);
  prof_end(static_cast<cudaStream_t>(stream), kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

UGEMM_API int ugemm_sgemv(char trans, int M, int N, float alpha, const float* A, int lda,
                          const float* x, int incx, float beta, float* y, int incy,
                          void* stream) {
  const bool t = (trans == 'T' || trans == 't');
  if (!t && trans != 'N' && trans != 'n') return UGEMM_ERR_ARG;
  if (M < 0 || N < 0 || incx <= 0 || incy <= 0) return UGEMM_ERR_ARG;
  if (lda < std::max(1, t ? N : M)) return UGEMM_ERR_ARG;
  if (M == 0) return UGEMM_OK;
  if (!y || (N > 0 && (!A || !x))) return UGEMM_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_begin(st);
  if (t) sgemv_t_kernel<<<(M + 7) / 8, 256, 0, st>>>(M, N, alpha, A, lda, x, incx, beta, y, incy);
  else sgemv_n_kernel<<<(M + 31) / 32, 256, 0, st>>>(M, N, alpha, A, lda, x, incx, beta, y, incy);
  prof_end(st, kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // extern "C"
