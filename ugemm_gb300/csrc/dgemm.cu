// dgemm.cu -- FP64 GEMM on the GPU, the accuracy oracle of the FP32 forms.
//
// The reference checks its GEMMs against FP64 CPU GEMMs (dgemm_cpu,
// ugemm.h:162-286; _dgemm_c, gemm_cpu.h:238-363; dgemm_avx, dgemm_avx.h:844),
// which take minutes at the 8192^3 shapes the GPU forms are measured on.
// This kernel computes the same C = alpha*op(A)*op(B) + beta*C in FP64 on
// the GPU: every element is one fused multiply-add chain over k in FP64, so
// its error is at most about K * 2^-53 relative to sum_k |a_ik b_kj| -- some
// 10^8 times below the FP32 forms' -- and it does not depend on a library
// whose FP64 arithmetic may be emulated.  It is test and measurement
// infrastructure (the tests and the benchmark compare every FP32 form with
// it); the FP32 product path never calls it.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, so the kernel is
// plain: 64 x 64 tiles of C, 16-deep k slices staged in shared memory with
// coalesced loads for either transpose, 4 x 4 outputs per thread.
#include <cuda_runtime.h>

#include <utility>

#include "internal.h"

namespace ugemm {
namespace {

constexpr int kDT = 64;   // tile of C
constexpr int kDK = 16;   // k depth of a shared-memory slice

// op(A)[m][k] = A[m*lda + k] ('N') or A[k*lda + m] ('T');
// op(B)[k][n] = B[k*ldb + n] ('N') or B[n*ldb + k] ('T').
__global__ void __launch_bounds__(256) dgemm_oracle_kernel(bool ta, bool tb, int M, int N, int K,
                                                           double alpha, const double* __restrict__ A,
                                                           int lda, const double* __restrict__ B,
                                                           int ldb, double beta, double* C, int ldc) {
  __shared__ double as[kDK][kDT + 1];
  __shared__ double bs[kDK][kDT + 1];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int m0 = blockIdx.y * kDT, n0 = blockIdx.x * kDT;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kDK) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = t + 256 * i;
      // the contiguous dimension varies fastest across the threads
      const int am = ta ? idx % kDT : idx / kDK, ak = ta ? idx / kDT : idx % kDK;
      const int m = m0 + am, k = k0 + ak;
      as[ak][am] = (m < M && k < K) ? A[ta ? size_t(k) * lda + m : size_t(m) * lda + k] : 0.0;
      const int bn = tb ? idx / kDK : idx % kDT, bk = tb ? idx % kDK : idx / kDT;
      const int n = n0 + bn, kb = k0 + bk;
      bs[bk][bn] = (n < N && kb < K) ? B[tb ? size_t(n) * ldb + kb : size_t(kb) * ldb + n] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kDK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = as[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      double* cp = C + size_t(m) * ldc + n;
      *cp = beta != 0.0 ? alpha * acc[i][j] + beta * *cp : alpha * acc[i][j];
    }
  }
}

int trans_flag(char t) {
  if (t == 'N' || t == 'n') return 0;
  if (t == 'T' || t == 't' || t == 'C' || t == 'c') return 1;
  return -1;
}

}  // namespace
}  // namespace ugemm

using namespace ugemm;

extern "C" UGEMM_API int ugemm_dgemm_oracle_dev(char major, char transa, char transb, int M, int N,
                                                int K, double alpha, const double* A, int lda,
                                                const double* B, int ldb, double beta, double* C,
                                                int ldc, void* stream) {
  int ta = trans_flag(transa), tb = trans_flag(transb);
  if (ta < 0 || tb < 0) {
    set_last_error(UGEMM_ERR_ARG, "transpose flags must be 'N', 'T' or 'C'");
    return UGEMM_ERR_ARG;
  }
  const bool row = major == 'R' || major == 'r';
  if (!row && major != 'C' && major != 'c') {
    set_last_error(UGEMM_ERR_ARG, "major must be 'R' or 'C'");
    return UGEMM_ERR_ARG;
  }
  if (M < 0 || N < 0 || K < 0) {
    set_last_error(UGEMM_ERR_ARG, "negative dimension");
    return UGEMM_ERR_ARG;
  }
  if (!row) {  // column-major C = op(A) op(B)  <=>  row-major C^T = op(B)^T op(A)^T
    std::swap(M, N);
    std::swap(A, B);
    std::swap(lda, ldb);
    std::swap(ta, tb);
  }
  if (M == 0 || N == 0) return UGEMM_OK;
  const int a_cols = ta ? M : K, b_cols = tb ? K : N;
  if (lda < (a_cols > 0 ? a_cols : 1) || ldb < (b_cols > 0 ? b_cols : 1) || ldc < N) {
    set_last_error(UGEMM_ERR_ARG, "leading dimension smaller than the matrix width");
    return UGEMM_ERR_ARG;
  }
  if (!C || (K > 0 && (!A || !B))) {
    set_last_error(UGEMM_ERR_ARG, "NULL matrix pointer");
    return UGEMM_ERR_ARG;
  }
  const dim3 grid(cdiv(N, kDT), cdiv(M, kDT));
  if (grid.y > 65535u) {
    set_last_error(UGEMM_ERR_ARG, "M too large for the FP64 oracle's grid");
    return UGEMM_ERR_ARG;
  }
  dgemm_oracle_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      ta != 0, tb != 0, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(UGEMM_ERR_CUDA, cudaGetErrorString(e));
    return UGEMM_ERR_CUDA;
  }
  return UGEMM_OK;
}
