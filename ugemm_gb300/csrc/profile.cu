// profile.cu -- optional per-kernel CUDA-event timing.  When enabled, every
// kernel launch of the library is bracketed by a pair of events recorded on
// its own stream; ugemm_profile_collect synchronises and sums the elapsed
// time per kernel kind.  Disabled (the default) it costs one branch.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "internal.h"

namespace ugemm {
namespace {
struct Span { cudaEvent_t a, b; int kind; };
std::mutex g_pmu;
bool g_on = false;
std::vector<Span> g_spans;
cudaEvent_t g_open = nullptr;
}  // namespace

void prof_begin(cudaStream_t st) {
  if (!g_on) return;
  std::lock_guard<std::mutex> l(g_pmu);
  cudaEventCreate(&g_open);
  cudaEventRecord(g_open, st);
}

void prof_end(cudaStream_t st, int kind) {
  if (!g_on) return;
  std::lock_guard<std::mutex> l(g_pmu);
  if (!g_open) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, st);
  g_spans.push_back(Span{g_open, e, kind});
  g_open = nullptr;
}

// FP32 FMA throughput: every thread runs eight independent FMA chains (the
// FMA latency covered by eight chains times eight or more warps per
// scheduler); the result is stored only if it equals a value it cannot
// reach, so the chains are not removed.
__global__ void __launch_bounds__(256) fp32_fma_peak_kernel(long long iters, float* sink) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-3f + i;
  const float b = 0.999999f, c = 1e-7f;
  for (long long n = 0; n < iters; ++n) {
#pragma unroll
    for (int r = 0; r < 16; ++r)
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == -1.f) *sink = s;
}

}  // namespace ugemm

extern "C" {

// Measured FP32 FMA peak of the current device (no reference counterpart:
// measurement infrastructure, the roofline of the plain SIMT form): a
// warm-up launch, then one of about `ms` milliseconds timed with CUDA events.
UGEMM_API int ugemm_fp32_peak(double ms, double* tflops) {
  if (!tflops || ms <= 0) return UGEMM_ERR_ARG;
  int dev = 0, sms = 0, clk = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return UGEMM_ERR_CUDA;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);  // kHz
  const int blocks = sms * 4, threads = 256;  // 32 warps per SM
  // flops per iteration of every thread: 16 x 8 FMAs
  const double per_iter = double(blocks) * threads * 16 * 8 * 2;
  // the nominal rate (128 FMA lanes per SM) sizes the launch
  const double nominal = double(sms) * 128 * 2 * (clk > 0 ? clk * 1e3 : 2e9);
  const long long iters = static_cast<long long>(nominal * ms * 1e-3 / per_iter) + 1;
  float* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) return UGEMM_ERR_ALLOC;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  ugemm::fp32_fma_peak_kernel<<<blocks, threads>>>(iters / 4 + 1, sink);
  cudaEventRecord(e0);
  ugemm::fp32_fma_peak_kernel<<<blocks, threads>>>(iters, sink);
  cudaEventRecord(e1);
  float t = 0.f;
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess || t <= 0.f) return UGEMM_ERR_CUDA;
  *tflops = per_iter * iters / (t * 1e-3) / 1e12;
  return UGEMM_OK;
}

UGEMM_API int ugemm_profile_enable(int on) {
  std::lock_guard<std::mutex> l(ugemm::g_pmu);
  ugemm::g_on = on != 0;
  return UGEMM_OK;
}

UGEMM_API int ugemm_profile_collect(double* ms_per_kind, int* launches_per_kind, int nkinds) {
  std::lock_guard<std::mutex> l(ugemm::g_pmu);
  for (int k = 0; k < nkinds; ++k) {
    if (ms_per_kind) ms_per_kind[k] = 0;
    if (launches_per_kind) launches_per_kind[k] = 0;
  }
  int rc = UGEMM_OK;
  for (auto& s : ugemm::g_spans) {
    float ms = 0.f;
    if (cudaEventSynchronize(s.b) != cudaSuccess || cudaEventElapsedTime(&ms, s.a, s.b) != cudaSuccess)
      rc = UGEMM_ERR_CUDA;
    if (s.kind >= 0 && s.kind < nkinds) {
      if (ms_per_kind) ms_per_kind[s.kind] += ms;
      if (launches_per_kind) launches_per_kind[s.kind] += 1;
    }
    cudaEventDestroy(s.a);
    cudaEventDestroy(s.b);
  }
  ugemm::g_spans.clear();
  return rc;
}

}  // extern "C"
