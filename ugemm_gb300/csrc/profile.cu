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

}  // namespace ugemm

extern "C" {

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
