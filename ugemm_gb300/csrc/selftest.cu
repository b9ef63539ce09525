// selftest.cu -- failure detection without a GPU fault.
//
// Every pipeline wait in the library's kernels is a bounded mbarrier wait
// (ptx.cuh mbar_wait): after its time limit it records an error code in a
// device word and returns, and the kernel winds down.  This self-test runs
// that same wait, with a short limit, on an mbarrier that nothing ever
// arrives on: the waiters must give up, the first one must record its code,
// the others must see the recorded error and stop early, and the kernel must
// return, leaving the CUDA context usable.  Nothing here faults, traps or
// hangs: the only failure is a wait that runs out.
#include <cuda_runtime.h>

#include <chrono>

#include "internal.h"
#include "ptx.cuh"

namespace ugemm {
namespace {

constexpr uint64_t kSelfTestLimitNs = 100000000ull;  // 100 ms

// Two warps wait on a barrier expecting one arrival that never comes; lane 0
// of warp 0 records the timeout, warp 1 stops when it sees the error word.
__global__ void wait_timeout_kernel(int* err, int* returned) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  const bool ok = mbar_wait<kSelfTestLimitNs>(&bar, 0, err, kDevTimeoutFull);
  if (!ok) atomicAdd(returned, 1);  // each thread that gave up reports back
}

}  // namespace
}  // namespace ugemm

using namespace ugemm;

extern "C" UGEMM_API int ugemm_selftest_wait_timeout(int* code, int* threads_returned,
                                                     double* seconds) {
  int* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) return UGEMM_ERR_ALLOC;
  int host[2] = {0, 0};
  cudaError_t e = cudaMemset(d, 0, 2 * sizeof(int));
  const auto t0 = std::chrono::steady_clock::now();
  if (e == cudaSuccess) {
    wait_timeout_kernel<<<1, 64>>>(d, d + 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  const auto t1 = std::chrono::steady_clock::now();
  if (e == cudaSuccess) e = cudaMemcpy(host, d, sizeof host, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return UGEMM_ERR_CUDA;
  if (code) *code = host[0];
  if (threads_returned) *threads_returned = host[1];
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  return host[0] != 0 ? UGEMM_ERR_TIMEOUT : UGEMM_OK;
}
