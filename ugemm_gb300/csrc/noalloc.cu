// noalloc.cu -- a split-precision SGEMM entry point that allocates nothing.
//
// ugemm_sgemm_dev takes the scratch of its split-precision form (the bf16
// pieces of A and B) from a workspace that it grows with cudaMalloc.  Some
// callers cannot allow that: a process that sets its device-memory budget at
// start-up and must not take more while it runs, a framework whose own
// allocator owns every byte of device memory and forbids allocations behind
// its back, or a latency-critical loop where an allocation could block on a
// device-wide synchronisation or fail at an unpredictable moment.  For them
// this file keeps the scratch in a fixed array in the library's own device
// memory, so ugemm_sgemm_dev_noalloc never calls cudaMalloc, cudaFree or any
// allocating routine.
//
// The array costs every GPU that loads this code kNoAllocScratchBytes of
// device memory until the process exits.  Its address is looked up once per
// device (cudaGetSymbolAddress, with that device current) on the first call
// made on the device; host code must never hand the symbol itself to a
// kernel, because on the host it names a host-side stand-in, not device
// memory.  Calls share the array: two calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on it.
//
// A kernel wait that times out writes a code into this file's error word;
// the next call moves it aside before its own kernels run (so it does not
// stop them early) and ugemm_check reports it.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "internal.h"

namespace ugemm {
namespace {

// 64 MiB: the bf16 pieces of both operands, 6 * (M + N) * Kp bytes for the
// three-piece forms (e.g. M = N = K = 2048 needs 48 MiB).
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
// [0]: written by the kernels of a call; [1]: the first code an earlier call
// left, held for ugemm_check
static __device__ __align__(16) int g_noalloc_err[2];

// Before a call's kernels: move a code an earlier call left to the held word.
__global__ void noalloc_error_fold_kernel() {
  const int code = g_noalloc_err[0];
  if (code != 0) {
    if (g_noalloc_err[1] == 0) g_noalloc_err[1] = code;
    g_noalloc_err[0] = 0;
  }
}

struct DeviceSlot {
  bool ready = false;
  void* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int* err = nullptr;       // device address of g_noalloc_err
};

constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceSlot g_slots[kMaxDevices];

ugemm_status fail(ugemm_status s, const char* msg) {
  set_last_error(s, msg);
  return s;
}

int trans_of(char t) {
  if (t == 'N' || t == 'n') return 'N';
  if (t == 'T' || t == 't' || t == 'C' || t == 'c') return 'T';
  return 0;
}

// The device addresses of this file's arrays on the current device, looked
// up on the first call made on that device.
ugemm_status slot_for_current_device(DeviceSlot** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(UGEMM_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceSlot& s = g_slots[dev];
  if (!s.ready) {
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3)
      return fail(UGEMM_ERR_UNSUPPORTED, "libugemm_cuda is built for sm_103a (GB300)");
    void* scratch = nullptr;
    e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
    void* err = nullptr;
    e = cudaGetSymbolAddress(&err, g_noalloc_err);
    if (e != cudaSuccess) return fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
    s.scratch = scratch;
    s.err = static_cast<int*>(err);
    s.ready = true;
  }
  *out = &s;
  return UGEMM_OK;
}

}  // namespace

int* noalloc_error_words() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  return g_slots[dev].ready ? g_slots[dev].err : nullptr;
}

}  // namespace ugemm

using namespace ugemm;

extern "C" UGEMM_API int ugemm_sgemm_dev_noalloc(char major, char transa, char transb, int M,
                                                 int N, int K, float alpha, const float* A,
                                                 int lda, const float* B, int ldb, float beta,
                                                 float* C, int ldc, int precision, void* stream) {
  const int ta = trans_of(transa), tb = trans_of(transb);
  if (!ta || !tb) return fail(UGEMM_ERR_ARG, "transpose flags must be 'N', 'T' or 'C'");
  const bool row = (major == 'R' || major == 'r');
  if (!row && major != 'C' && major != 'c') return fail(UGEMM_ERR_ARG, "major must be 'R' or 'C'");
  if (M < 0 || N < 0 || K < 0) return fail(UGEMM_ERR_ARG, "negative dimension");
  int form = precision == UGEMM_PREC_AUTO ? UGEMM_PREC_BF16X6 : precision;
  if (form != UGEMM_PREC_BF16X6 && form != UGEMM_PREC_BF16X9 && form != UGEMM_PREC_BF16X3)
    return fail(UGEMM_ERR_UNSUPPORTED,
                "the allocation-free entry point runs the bf16 split forms only (BF16X6, BF16X9, BF16X3)");
  // column-major C = op(A) op(B)  <=>  row-major C^T = op(B)^T op(A)^T
  Gemm g = row ? Gemm{static_cast<char>(ta), static_cast<char>(tb), M, N, K, alpha, beta, A, lda,
                      B, ldb, C, ldc}
               : Gemm{static_cast<char>(tb), static_cast<char>(ta), N, M, K, alpha, beta, B, ldb,
                      A, lda, C, ldc};
  if (g.M == 0 || g.N == 0) return UGEMM_OK;
  const int a_cols = g.ta == 'N' ? g.K : g.M, b_cols = g.tb == 'N' ? g.N : g.K;
  if (g.lda < (a_cols > 0 ? a_cols : 1) || g.ldb < (b_cols > 0 ? b_cols : 1) || g.ldc < g.N)
    return fail(UGEMM_ERR_ARG, "leading dimension smaller than the matrix width");
  if (!g.C) return fail(UGEMM_ERR_ARG, "C is NULL");
  if (g.K > 0 && alpha != 0.f && (!g.A || !g.B)) return fail(UGEMM_ERR_ARG, "A or B is NULL");

  DeviceSlot* slot = nullptr;
  ugemm_status s = slot_for_current_device(&slot);
  if (s != UGEMM_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (g.K == 0 || g.alpha == 0.f) {
    s = scale_c_launch(g, st);
    return s == UGEMM_OK ? s : fail(s, "scale launch failed");
  }
  const SplitPlan plan = split_plan_for(form, g);
  const size_t need = split_scratch_bytes(g, plan);
  if (need > kNoAllocScratchBytes) {
    char msg[160];
    std::snprintf(msg, sizeof msg,
                  "this call needs %zu bytes of scratch; the fixed array holds %zu bytes",
                  need, kNoAllocScratchBytes);
    return fail(UGEMM_ERR_ARENA_TOO_SMALL, msg);
  }
  // A pending error of earlier, unrelated work is not this call's; a code an
  // earlier call left in the error word is moved aside for ugemm_check.
  (void)cudaGetLastError();
  prof_begin(st);
  noalloc_error_fold_kernel<<<1, 1, 0, st>>>();
  prof_end(st, kProfControl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
  s = split_launch(g, plan, Scratch{slot->scratch, kNoAllocScratchBytes}, slot->err, st);
  if (s != UGEMM_OK) {
    const cudaError_t le = cudaGetLastError();
    return fail(s, le != cudaSuccess ? cudaGetErrorString(le) : "split launch failed");
  }
  return UGEMM_OK;
}
