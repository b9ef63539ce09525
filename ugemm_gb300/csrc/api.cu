// api.cu -- the C ABI of libugemm_cuda.so (include/sgemm_cuda.h).
//
// Host-side orchestration that replaces the reference's OpenCL backend glue
// (sgemm_ocl2.h:133-224 and the ocl.h runtime shim): argument checks, the
// init-time device arena of the compat API, the growable workspace of the
// device-pointer API, the choice between the SIMT and split-precision
// tensor-core forms, and error reporting (the reference reports none).
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"

namespace ugemm {

namespace {
thread_local int t_last_status = UGEMM_OK;
thread_local std::string t_last_msg;

struct DeviceState {
  bool ready = false;
  // Device-side error words: dev_err[0] is written by the bounded waits of
  // the kernels of one call (the word the kernels see); dev_err[1] holds the
  // first code that a device-pointer call left there, until ugemm_check
  // reads it (error_fold_kernel moves it before the next call's kernels).
  int* dev_err = nullptr;
  void* ws = nullptr;         // workspace of the device-pointer API
  size_t ws_bytes = 0;
  int sms = 0, cc_major = 0, cc_minor = 0;
};

constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceState g_dev[kMaxDevices];

struct Compat {
  bool init = false;
  int device = 0;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  cudaStream_t stream = nullptr;
  int precision = UGEMM_PREC_AUTO;
};
Compat g_compat;
int g_default_precision = UGEMM_PREC_AUTO;

ugemm_status fail(ugemm_status s, const char* fmt, const char* detail = "") {
  char buf[512];
  std::snprintf(buf, sizeof buf, fmt, detail);
  set_last_error(s, buf);
  return s;
}

ugemm_status cuda_fail(cudaError_t e, const char* what) {
  char buf[512];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  set_last_error(e == cudaErrorNoKernelImageForDevice ? UGEMM_ERR_UNSUPPORTED : UGEMM_ERR_CUDA,
                 buf);
  return e == cudaErrorNoKernelImageForDevice ? UGEMM_ERR_UNSUPPORTED : UGEMM_ERR_CUDA;
}

// Set up (once) the state of the current device.  Caller holds g_mu.
ugemm_status device_state(DeviceState** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(UGEMM_ERR_ARG, "device index out of range%s");
  DeviceState& d = g_dev[dev];
  if (!d.ready) {
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (d.cc_major != 10 || d.cc_minor != 3)
      return fail(UGEMM_ERR_UNSUPPORTED, "libugemm_cuda is built for sm_103a (GB300)%s");
    e = cudaMalloc(&d.dev_err, 2 * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(error word)");
    e = cudaMemset(d.dev_err, 0, 2 * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(error word)");
    d.ready = true;
  }
  *out = &d;
  return UGEMM_OK;
}

// Stream-ordered start of a call on the device path: a code left in the
// kernels' word by an earlier call moves to the held word (the first one is
// kept) and the kernels' word is cleared, so a stale timeout neither stops
// this call's waits early nor is reported as this call's; ugemm_check reports
// it.  One thread, a few instructions.
__global__ void error_fold_kernel(int* words) {
  const int code = words[0];
  if (code != 0) {
    if (words[1] == 0) words[1] = code;
    words[0] = 0;
  }
}

ugemm_status begin_call(int* words, cudaStream_t st) {
  (void)cudaGetLastError();  // a pending error of earlier, unrelated work is not this call's
  prof_begin(st);
  error_fold_kernel<<<1, 1, 0, st>>>(words);
  prof_end(st, kProfControl);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? UGEMM_OK : cuda_fail(e, "error word fold");
}

bool is_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return false;
  return cs != cudaStreamCaptureStatusNone;
}

// Grow the device workspace to `need` bytes (never during stream capture).
ugemm_status ensure_workspace(DeviceState& d, size_t need, cudaStream_t st) {
  if (need <= d.ws_bytes) return UGEMM_OK;
  if (is_capturing(st))
    return fail(UGEMM_ERR_ARENA_TOO_SMALL,
                "workspace too small during stream capture; call ugemm_reserve_workspace first%s");
  if (d.ws) {
    cudaError_t e = cudaFree(d.ws);  // synchronises the device: no kernel still uses it
    d.ws = nullptr;
    d.ws_bytes = 0;
    if (e != cudaSuccess) return cuda_fail(e, "cudaFree(workspace)");
  }
  const size_t bytes = align_up(need, size_t(1) << 21);
  cudaError_t e = cudaMalloc(&d.ws, bytes);
  if (e != cudaSuccess) {
    d.ws = nullptr;
    return cuda_fail(e, "cudaMalloc(workspace)");
  }
  d.ws_bytes = bytes;
  return UGEMM_OK;
}

int norm_trans(char t) {
  if (t == 'N' || t == 'n') return 'N';
  if (t == 'T' || t == 't' || t == 'C' || t == 'c') return 'T';
  return 0;
}

// Validate a BLAS-style call and rewrite it as a row-major Gemm.
ugemm_status make_gemm(char major, char transa, char transb, int M, int N, int K, float alpha,
                       const float* A, int lda, const float* B, int ldb, float beta, float* C,
                       int ldc, Gemm* g) {
  const int ta = norm_trans(transa), tb = norm_trans(transb);
  if (!ta || !tb) return fail(UGEMM_ERR_ARG, "transpose flags must be 'N' or 'T'%s");
  if (major != 'R' && major != 'r' && major != 'C' && major != 'c')
    return fail(UGEMM_ERR_ARG, "major must be 'R' or 'C'%s");
  if (M < 0 || N < 0 || K < 0) return fail(UGEMM_ERR_ARG, "negative dimension%s");
  const bool row = (major == 'R' || major == 'r');
  // column-major C = op(A) op(B)  <=>  row-major C^T = op(B)^T op(A)^T
  Gemm r;
  if (row) {
    r = Gemm{static_cast<char>(ta), static_cast<char>(tb), M, N, K, alpha, beta, A, lda, B, ldb, C, ldc};
  } else {
    r = Gemm{static_cast<char>(tb), static_cast<char>(ta), N, M, K, alpha, beta, B, ldb, A, lda, C, ldc};
  }
  if (r.M == 0 || r.N == 0) { *g = r; return UGEMM_OK; }
  const int a_cols = r.ta == 'N' ? r.K : r.M, b_cols = r.tb == 'N' ? r.N : r.K;
  if (r.lda < (a_cols > 0 ? a_cols : 1) || r.ldb < (b_cols > 0 ? b_cols : 1) || r.ldc < r.N)
    return fail(UGEMM_ERR_ARG, "leading dimension smaller than the matrix width%s");
  if (!r.C) return fail(UGEMM_ERR_ARG, "C is NULL%s");
  if (r.K > 0 && alpha != 0.f && (!r.A || !r.B)) return fail(UGEMM_ERR_ARG, "A or B is NULL%s");
  *g = r;
  return UGEMM_OK;
}

int resolve_form(int precision, const Gemm& g) {
  if (precision != UGEMM_PREC_AUTO) return precision;
  // Tensor-core splitting pays once the problem fills the GPU; the split
  // pre-pass and the 128-row tiles waste too much on small problems.
  if (g.M >= 256 && g.N >= 256 && g.K >= 256) return UGEMM_PREC_BF16X6;
  return UGEMM_PREC_SIMT;
}

bool is_split_form(int form) {
  return form == UGEMM_PREC_BF16X6 || form == UGEMM_PREC_BF16X9 || form == UGEMM_PREC_BF16X3 ||
         form == UGEMM_PREC_FP16X3 || form == UGEMM_PREC_TF32X3;
}

size_t scratch_for(const Gemm& g, int form) {
  if (g.M == 0 || g.N == 0 || g.K == 0 || g.alpha == 0.f) return 0;
  if (form == UGEMM_PREC_SIMT) return simt_scratch_bytes(g);
  const SplitPlan p = split_plan_for(form, g);
  // an under-filled GEMM with deep k runs as split-K slices (multi.cu)
  if (multi_wanted(g, p)) return multi_scratch_bytes(&g, 1, p);
  return split_scratch_bytes(g, p);
}

// Launch one GEMM on `st` using `ws` as scratch.
ugemm_status launch(const Gemm& g, int form, Scratch ws, int* dev_err, cudaStream_t st) {
  if (g.M == 0 || g.N == 0) return UGEMM_OK;
  if (g.K == 0 || g.alpha == 0.f) return scale_c_launch(g, st);
  ugemm_status s;
  if (form == UGEMM_PREC_SIMT) {
    s = simt_launch(g, simt_pick_tile(g), ws, dev_err, st);
  } else if (is_split_form(form)) {
    const SplitPlan p = split_plan_for(form, g);
    s = multi_wanted(g, p) ? multi_launch(&g, 1, p, ws, dev_err, st)
                           : split_launch(g, p, ws, dev_err, st);
  } else {
    return fail(UGEMM_ERR_ARG, "unknown precision%s");
  }
  if (s == UGEMM_ERR_CUDA) {
    cudaError_t e = cudaGetLastError();
    return cuda_fail(e, "kernel launch");
  }
  if (s != UGEMM_OK) return fail(s, "launch failed%s");
  return UGEMM_OK;
}

// Read and clear the device error word (synchronises `st`).
ugemm_status check_device_error(DeviceState& d, cudaStream_t st) {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  int code = 0;
  e = cudaMemcpy(&code, d.dev_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(error word)");
  if (code != 0) {
    cudaMemset(d.dev_err, 0, sizeof(int));
    char buf[128];
    std::snprintf(buf, sizeof buf, "kernel pipeline wait timed out (code %d)", code);
    set_last_error(UGEMM_ERR_TIMEOUT, buf);
    return UGEMM_ERR_TIMEOUT;
  }
  return UGEMM_OK;
}

ugemm_status dev_gemm(const Gemm& g, int precision, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceState* d = nullptr;
  ugemm_status s = device_state(&d);
  if (s != UGEMM_OK) return s;
  const int form = resolve_form(precision, g);
  s = ensure_workspace(*d, scratch_for(g, form), st);
  if (s != UGEMM_OK) return s;
  s = begin_call(d->dev_err, st);
  if (s != UGEMM_OK) return s;
  return launch(g, form, Scratch{d->ws, d->ws_bytes}, d->dev_err, st);
}

// Host-pointer GEMM in an arena too small for the 256-byte-aligned layout:
// A and B are packed into it with rows padded to 16 bytes (the host copies
// do the padding, so the SIMT form needs no scratch: its tensor maps read the
// packed rows directly), C tightly, regions 16-byte aligned, the scratch of a
// split form 256-byte aligned after them.  The reference sizes its arena at
// ten times the three matrices (sgemm_test.c:29), which this layout fits for
// every shape in the SIMT form (at most 3 padding floats per row).
ugemm_status host_gemm_tight(const Gemm& g, int form, void* arena, size_t arena_bytes,
                             DeviceState& d, cudaStream_t st) {
  const size_t a_rows = g.ta == 'N' ? g.M : g.K, b_rows = g.tb == 'N' ? g.K : g.N;
  const size_t a_cols = g.ta == 'N' ? g.K : g.M, b_cols = g.tb == 'N' ? g.N : g.K;
  const bool need_ab = g.K > 0 && g.alpha != 0.f;
  const int lda4 = static_cast<int>(align_up(std::max<size_t>(a_cols, 1), 4));
  const int ldb4 = static_cast<int>(align_up(std::max<size_t>(b_cols, 1), 4));
  const size_t a_bytes = need_ab ? align_up(a_rows * lda4 * sizeof(float), 16) : 0;
  const size_t b_bytes = need_ab ? align_up(b_rows * ldb4 * sizeof(float), 16) : 0;
  const size_t c_bytes = size_t(g.M) * g.N * sizeof(float);
  uint8_t* base = static_cast<uint8_t*>(arena);
  Gemm dg = g;
  dg.A = reinterpret_cast<const float*>(base);
  dg.B = reinterpret_cast<const float*>(base + a_bytes);
  dg.C = reinterpret_cast<float*>(base + a_bytes + b_bytes);
  dg.lda = lda4;
  dg.ldb = ldb4;
  dg.ldc = g.N;
  const size_t scratch = scratch_for(dg, form);
  const size_t s_off = scratch ? align_up(a_bytes + b_bytes + c_bytes, 256) : a_bytes + b_bytes + c_bytes;
  if (s_off + scratch > arena_bytes)
    return fail(UGEMM_ERR_ARENA_TOO_SMALL, "device arena too small for this call%s");
  cudaError_t e;
  if (need_ab) {
    e = cudaMemcpy2DAsync(const_cast<float*>(dg.A), lda4 * sizeof(float), g.A, g.lda * sizeof(float),
                          a_cols * sizeof(float), a_rows, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy A to device");
    e = cudaMemcpy2DAsync(const_cast<float*>(dg.B), ldb4 * sizeof(float), g.B, g.ldb * sizeof(float),
                          b_cols * sizeof(float), b_rows, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy B to device");
  }
  if (g.beta != 0.f) {  // beta == 0: C is not read (sgemm_ocl2.h:177)
    e = cudaMemcpy2DAsync(dg.C, g.N * sizeof(float), g.C, g.ldc * sizeof(float),
                          g.N * sizeof(float), g.M, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy C to device");
  }
  ugemm_status s = launch(dg, form, Scratch{base + s_off, arena_bytes - s_off}, d.dev_err, st);
  if (s != UGEMM_OK) return s;
  e = cudaMemcpy2DAsync(g.C, g.ldc * sizeof(float), dg.C, g.N * sizeof(float), g.N * sizeof(float),
                        g.M, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "copy C to host");
  return check_device_error(d, st);
}

// Host-pointer GEMM through a device arena [A | B | C | scratch].
ugemm_status host_gemm(const Gemm& g, int precision, void* arena, size_t arena_bytes,
                       DeviceState& d, cudaStream_t st) {
  if (g.M == 0 || g.N == 0) return UGEMM_OK;
  {
    ugemm_status bs = begin_call(d.dev_err, st);
    if (bs != UGEMM_OK) return bs;
  }
  const size_t a_rows = g.ta == 'N' ? g.M : g.K, b_rows = g.tb == 'N' ? g.K : g.N;
  const size_t a_cols = g.ta == 'N' ? g.K : g.M, b_cols = g.tb == 'N' ? g.N : g.K;
  const size_t a_bytes = align_up(a_rows * g.lda * sizeof(float), 256);
  const size_t b_bytes = align_up(b_rows * g.ldb * sizeof(float), 256);
  const size_t c_bytes = align_up(size_t(g.M) * g.ldc * sizeof(float), 256);
  const int form = resolve_form(precision, g);
  {
    ugemm_status ps = host_gemm_pipelined(g, form, arena, arena_bytes, d.dev_err, st);
    if (ps == UGEMM_OK) return check_device_error(d, st);
    if (ps != UGEMM_ERR_UNSUPPORTED) return fail(ps, "pipelined host GEMM failed%s");
  }
  const bool need_ab = g.K > 0 && g.alpha != 0.f;
  const size_t need = (need_ab ? a_bytes + b_bytes : 0) + c_bytes + scratch_for(g, form);
  if (need > arena_bytes) return host_gemm_tight(g, form, arena, arena_bytes, d, st);
  uint8_t* base = static_cast<uint8_t*>(arena);
  Gemm dg = g;
  size_t off = 0;
  cudaError_t e;
  if (need_ab) {
    dg.A = reinterpret_cast<const float*>(base);
    dg.B = reinterpret_cast<const float*>(base + a_bytes);
    off = a_bytes + b_bytes;
    // Copy up to the last element actually used, never past it.
    e = cudaMemcpyAsync(const_cast<float*>(dg.A), g.A, ((a_rows - 1) * g.lda + a_cols) * sizeof(float),
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy A to device");
    e = cudaMemcpyAsync(const_cast<float*>(dg.B), g.B, ((b_rows - 1) * g.ldb + b_cols) * sizeof(float),
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy B to device");
  }
  dg.C = reinterpret_cast<float*>(base + off);
  const size_t c_copy = (size_t(g.M) - 1) * g.ldc + g.N;
  if (g.beta != 0.f) {  // beta == 0: C is not read (sgemm_ocl2.h:177)
    e = cudaMemcpyAsync(dg.C, g.C, c_copy * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy C to device");
  }
  Scratch ws{base + off + c_bytes, arena_bytes - off - c_bytes};
  ugemm_status s = launch(dg, form, ws, d.dev_err, st);
  if (s != UGEMM_OK) return s;
  // Copy back row by row only when the host C has padding we must not touch.
  if (g.ldc == g.N) {
    e = cudaMemcpyAsync(g.C, dg.C, size_t(g.M) * g.N * sizeof(float), cudaMemcpyDeviceToHost, st);
  } else {
    e = cudaMemcpy2DAsync(g.C, g.ldc * sizeof(float), dg.C, g.ldc * sizeof(float),
                          g.N * sizeof(float), g.M, cudaMemcpyDeviceToHost, st);
  }
  if (e != cudaSuccess) return cuda_fail(e, "copy C to host");
  return check_device_error(d, st);
}

}  // namespace

void set_last_error(ugemm_status s, const std::string& msg) {
  t_last_status = s;
  t_last_msg = msg;
}

}  // namespace ugemm

using namespace ugemm;

extern "C" {

const char* ugemm_status_string(int s) {
  switch (s) {
    case UGEMM_OK: return "ok";
    case UGEMM_ERR_ARG: return "invalid argument";
    case UGEMM_ERR_ALLOC: return "allocation failed";
    case UGEMM_ERR_ARENA_TOO_SMALL: return "arena or workspace too small";
    case UGEMM_ERR_CUDA: return "CUDA error";
    case UGEMM_ERR_TIMEOUT: return "kernel wait timed out";
    case UGEMM_ERR_NOT_INIT: return "sgemm_cuda_init not called";
    case UGEMM_ERR_UNSUPPORTED: return "unsupported device or form";
    default: return "unknown status";
  }
}

int ugemm_last_error(void) { return t_last_status; }
const char* ugemm_last_error_message(void) { return t_last_msg.c_str(); }

void sgemm_cuda_init(int platform, int device, size_t size) {
  (void)platform;
  std::lock_guard<std::mutex> lock(g_mu);
  set_last_error(UGEMM_OK, "");
  if (g_compat.init) {
    set_last_error(UGEMM_ERR_ARG, "sgemm_cuda_init called twice without sgemm_cuda_finish");
    return;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { cuda_fail(e, "cudaSetDevice"); return; }
  DeviceState* d = nullptr;
  if (device_state(&d) != UGEMM_OK) return;
  e = cudaStreamCreateWithFlags(&g_compat.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { cuda_fail(e, "cudaStreamCreate"); return; }
  e = cudaMalloc(&g_compat.arena, size);
  if (e != cudaSuccess) {
    cudaStreamDestroy(g_compat.stream);
    g_compat.stream = nullptr;
    g_compat.arena = nullptr;
    set_last_error(UGEMM_ERR_ALLOC, "cudaMalloc(arena) failed");
    return;
  }
  g_compat.arena_bytes = size;
  g_compat.device = device;
  g_compat.precision = g_default_precision;
  g_compat.init = true;
}

int sgemm_cuda_set_precision(int precision) {
  if (precision < UGEMM_PREC_AUTO || precision > UGEMM_PREC_TF32X3) return UGEMM_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mu);
  g_default_precision = precision;
  g_compat.precision = precision;
  return UGEMM_OK;
}

int sgemm_cuda_status(char ta, char tb, int m, int n, int k, float alpha, const float* a,
                      const float* b, float beta, float* c) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_compat.init) return fail(UGEMM_ERR_NOT_INIT, "sgemm_cuda before sgemm_cuda_init%s");
  // sgemm_ocl2.h:180,190: 'T' transposes, anything else is 'N'; tight lds.
  const char tA = (ta == 'T') ? 'T' : 'N', tB = (tb == 'T') ? 'T' : 'N';
  Gemm g;
  ugemm_status s = make_gemm('R', tA, tB, m, n, k, alpha, a, tA == 'N' ? k : m, b,
                             tB == 'N' ? n : k, beta, c, n, &g);
  if (s != UGEMM_OK) return s;
  cudaError_t e = cudaSetDevice(g_compat.device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  DeviceState* d = nullptr;
  s = device_state(&d);
  if (s != UGEMM_OK) return s;
  s = host_gemm(g, g_compat.precision, g_compat.arena, g_compat.arena_bytes, *d, g_compat.stream);
  if (s == UGEMM_OK) set_last_error(UGEMM_OK, "");
  return s;
}

void sgemm_cuda(char ta, char tb, int m, int n, int k, float alpha, float* a, float* b, float beta,
                float* c) {
  sgemm_cuda_status(ta, tb, m, n, k, alpha, a, b, beta, c);
}

void sgemm_cuda_finish(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_compat.init) return;
  cudaSetDevice(g_compat.device);
  if (g_compat.stream) cudaStreamSynchronize(g_compat.stream);
  cudaFree(g_compat.arena);
  cudaStreamDestroy(g_compat.stream);
  g_compat = Compat{};
}

int ugemm_sgemm_host(char major, char transa, char transb, int M, int N, int K, float alpha,
                     const float* A, int lda, const float* B, int ldb, float beta, float* C,
                     int ldc, int precision) {
  Gemm g;
  ugemm_status s = make_gemm(major, transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, &g);
  if (s != UGEMM_OK) return s;
  if (g.M == 0 || g.N == 0) return UGEMM_OK;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_compat.init) {
    cudaError_t e = cudaSetDevice(g_compat.device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  }
  DeviceState* d = nullptr;
  s = device_state(&d);
  if (s != UGEMM_OK) return s;
  if (g_compat.init)
    return host_gemm(g, precision, g_compat.arena, g_compat.arena_bytes, *d, g_compat.stream);
  // Without init: a temporary arena sized for this call.
  const int form = resolve_form(precision, g);
  const size_t a_rows = g.ta == 'N' ? g.M : g.K, b_rows = g.tb == 'N' ? g.K : g.N;
  const size_t bytes = std::max(align_up(a_rows * g.lda * 4, 256) + align_up(b_rows * g.ldb * 4, 256) +
                                    align_up(size_t(g.M) * g.ldc * 4, 256) + scratch_for(g, form),
                                host_pipelined_bytes(g, form));
  void* arena = nullptr;
  cudaError_t e = cudaMalloc(&arena, bytes);
  if (e != cudaSuccess) return fail(UGEMM_ERR_ALLOC, "cudaMalloc(temporary arena) failed%s");
  s = host_gemm(g, precision, arena, bytes, *d, nullptr);
  cudaFree(arena);
  return s;
}

void ugemm_sgemm(char major, char transa, char transb, int M, int N, int K, float alpha,
                 const float* A, int lda, const float* B, int ldb, float beta, float* C, int ldc) {
  const int s = ugemm_sgemm_host(major, transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                 ldc, g_compat.init ? g_compat.precision : g_default_precision);
  if (s == UGEMM_OK) set_last_error(UGEMM_OK, "");
}

int ugemm_sgemm_dev(char major, char transa, char transb, int M, int N, int K, float alpha,
                    const float* A, int lda, const float* B, int ldb, float beta, float* C,
                    int ldc, int precision, void* stream) {
  Gemm g;
  ugemm_status s = make_gemm(major, transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, &g);
  if (s != UGEMM_OK) return s;
  if (g.M == 0 || g.N == 0) return UGEMM_OK;  // nothing to do, not even device set-up
  return dev_gemm(g, precision, static_cast<cudaStream_t>(stream));
}

int ugemm_sgemm_dev_ex(char major, char transa, char transb, int M, int N, int K, float alpha,
                       const float* A, int lda, const float* B, int ldb, float beta, float* C,
                       int ldc, const float* bias, int act, float slope, int precision,
                       void* stream) {
  if ((bias || act) && major != 'R' && major != 'r')
    return fail(UGEMM_ERR_ARG, "the fused epilogue takes row-major calls%s");
  if (act != 0 && act != 1) return fail(UGEMM_ERR_ARG, "act must be 0 (none) or 1 (LeakyReLU)%s");
  Gemm g;
  ugemm_status s = make_gemm(major, transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, &g);
  if (s != UGEMM_OK) return s;
  if (g.M == 0 || g.N == 0) return UGEMM_OK;
  g.epi.bias = bias;
  g.epi.act = act;
  g.epi.slope = slope;
  if (g.K == 0 || g.alpha == 0.f) {
    if (bias || act) return fail(UGEMM_ERR_UNSUPPORTED, "fused epilogue needs K > 0 and alpha != 0%s");
  }
  return dev_gemm(g, precision, static_cast<cudaStream_t>(stream));
}

size_t ugemm_workspace_bytes(char major, char transa, char transb, int M, int N, int K, int lda,
                             int ldb, int precision) {
  Gemm g;
  // Pointers only matter for alignment: assume aligned device buffers.
  static float dummy[4] __attribute__((aligned(16)));
  if (make_gemm(major, transa, transb, M, N, K, 1.f, dummy, lda, dummy, ldb, 0.f, dummy,
                (major == 'R' || major == 'r') ? N : M, &g) != UGEMM_OK)
    return 0;
  return scratch_for(g, resolve_form(precision, g));
}

int ugemm_reserve_workspace(size_t bytes) {
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceState* d = nullptr;
  ugemm_status s = device_state(&d);
  if (s != UGEMM_OK) return s;
  return ensure_workspace(*d, bytes, nullptr);
}

int ugemm_sgemm_backward(char transa, char transb, int M, int N, int K, float alpha,
                         const float* A, int lda, const float* B, int ldb, const float* dC,
                         int lddc, float beta_a, float* dA, int ldda, float beta_b, float* dB,
                         int lddb, int precision, void* stream) {
  const int ta = norm_trans(transa), tb = norm_trans(transb);
  if (!ta || !tb) return fail(UGEMM_ERR_ARG, "transpose flags must be 'N' or 'T'%s");
  if (M < 0 || N < 0 || K < 0) return fail(UGEMM_ERR_ARG, "negative dimension%s");
  if (!dC && (dA || dB)) return fail(UGEMM_ERR_ARG, "dC is NULL%s");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto flip = [](int t) { return static_cast<char>(t == 'N' ? 'T' : 'N'); };
  // Split forms: dA and dB as one persistent launch (multi.cu), so the tiles
  // of both products fill the GPU together.
  {
    Gemm gs[2];
    int n = 0;
    bool together = M > 0 && N > 0 && K > 0 && alpha != 0.f && (dA || dB);
    if (together && dA) {
      const ugemm_status s =
          ta == 'N' ? make_gemm('R', 'N', flip(tb), M, K, N, alpha, dC, lddc, B, ldb, beta_a, dA,
                                ldda, &gs[n])
                    : make_gemm('R', static_cast<char>(tb), 'T', K, M, N, alpha, B, ldb, dC, lddc,
                                beta_a, dA, ldda, &gs[n]);
      if (s != UGEMM_OK) return s;
      ++n;
    }
    if (together && dB) {
      const ugemm_status s =
          tb == 'N' ? make_gemm('R', flip(ta), 'N', K, N, M, alpha, A, lda, dC, lddc, beta_b, dB,
                                lddb, &gs[n])
                    : make_gemm('R', 'T', static_cast<char>(ta), N, K, M, alpha, dC, lddc, A, lda,
                                beta_b, dB, lddb, &gs[n]);
      if (s != UGEMM_OK) return s;
      ++n;
    }
    for (int i = 0; i < n; ++i) together = together && resolve_form(precision, gs[i]) == resolve_form(precision, gs[0]);
    const int form = n > 0 ? resolve_form(precision, gs[0]) : UGEMM_PREC_SIMT;
    if (together && is_split_form(form)) {
      std::lock_guard<std::mutex> lock(g_mu);
      DeviceState* d = nullptr;
      ugemm_status s = device_state(&d);
      if (s != UGEMM_OK) return s;
      const SplitPlan p = split_plan_for(form, gs[0]);
      s = ensure_workspace(*d, multi_scratch_bytes(gs, n, p), st);
      if (s != UGEMM_OK) return s;
      s = begin_call(d->dev_err, st);
      if (s != UGEMM_OK) return s;
      s = multi_launch(gs, n, p, Scratch{d->ws, d->ws_bytes}, d->dev_err, st);
      if (s == UGEMM_ERR_CUDA) return cuda_fail(cudaGetLastError(), "kernel launch");
      if (s != UGEMM_OK) return fail(s, "launch failed%s");
      return UGEMM_OK;
    }
  }
  if (dA) {
    ugemm_status s;
    if (ta == 'N')  // dA[MxK] = alpha dC op(B)^T
      s = static_cast<ugemm_status>(ugemm_sgemm_dev('R', 'N', flip(tb), M, K, N, alpha, dC, lddc, B,
                                                    ldb, beta_a, dA, ldda, precision, st));
    else            // dA[KxM] = alpha op(B) dC^T
      s = static_cast<ugemm_status>(ugemm_sgemm_dev('R', static_cast<char>(tb), 'T', K, M, N, alpha,
                                                    B, ldb, dC, lddc, beta_a, dA, ldda, precision, st));
    if (s != UGEMM_OK) return s;
  }
  if (dB) {
    ugemm_status s;
    if (tb == 'N')  // dB[KxN] = alpha op(A)^T dC
      s = static_cast<ugemm_status>(ugemm_sgemm_dev('R', flip(ta), 'N', K, N, M, alpha, A, lda, dC,
                                                    lddc, beta_b, dB, lddb, precision, st));
    else            // dB[NxK] = alpha dC^T op(A)
      s = static_cast<ugemm_status>(ugemm_sgemm_dev('R', 'T', static_cast<char>(ta), N, K, M, alpha,
                                                    dC, lddc, A, lda, beta_b, dB, lddb, precision, st));
    if (s != UGEMM_OK) return s;
  }
  return UGEMM_OK;
}

int ugemm_check(void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceState* d = nullptr;
  ugemm_status s = device_state(&d);
  if (s != UGEMM_OK) return s;
  int words[2] = {0, 0}, na[2] = {0, 0};
  e = cudaMemcpy(words, d->dev_err, sizeof words, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(error words)");
  int* nw = noalloc_error_words();
  if (nw) {
    e = cudaMemcpy(na, nw, sizeof na, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(error words)");
  }
  // the first recorded code wins: held codes are older than current ones
  const int code = words[1] ? words[1] : words[0] ? words[0] : na[1] ? na[1] : na[0];
  if (code == 0) return UGEMM_OK;
  if (words[0] || words[1]) cudaMemset(d->dev_err, 0, sizeof words);
  if (na[0] || na[1]) cudaMemset(nw, 0, sizeof na);
  char buf[160];
  std::snprintf(buf, sizeof buf,
                "a kernel's pipeline wait timed out (code %d) in a device-pointer call", code);
  set_last_error(UGEMM_ERR_TIMEOUT, buf);
  return UGEMM_ERR_TIMEOUT;
}

int ugemm_debug_set_error_word(int which, int code) {
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceState* d = nullptr;
  ugemm_status s = device_state(&d);
  if (s != UGEMM_OK) return s;
  int* word = which == 0 ? d->dev_err : which == 1 ? noalloc_error_words() : nullptr;
  if (!word) return fail(UGEMM_ERR_ARG, "no such error word on this device (yet)%s");
  const cudaError_t e = cudaMemcpy(word, &code, sizeof code, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? UGEMM_OK : cuda_fail(e, "cudaMemcpy(error word)");
}

int ugemm_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (sm_count) cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (cc_major) cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev);
  if (cc_minor) cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
  return UGEMM_OK;
}

}  // extern "C"
