// pipeline.cu -- overlapped host <-> device copies for the host-pointer API.
//
// The reference's sgemm_ocl (sgemm_ocl2.h:166-219) writes A, B (and C) to the
// device, runs the kernel and reads C back, one blocking step after another,
// and the reference's benchmarks time all of it (sgemm_test.c:229-232).
// Here a large host-pointer GEMM runs in two phases whose copies, GEMMs and
// copies back overlap:
//   1. k slabs.  op(A)[:, k0:k0+w] and op(B)[k0:k0+w, :] cross the host link
//      slab by slab; each slab is a rank-w update of a device accumulator
//      (the first with beta = 0, so C is not needed yet).  Per byte copied a
//      slab carries 2MN/(4(M+N)) flops, more than the GEMMs can retire at
//      the link's rate, so the GEMMs run back to back from the first slab on.
//   2. row bands.  The rest of op(B) (k >= k1) crosses once; then, band by
//      band, the rest of op(A)'s rows and the band of C.  A band's C is
//      folded into the accumulator (acc += beta * C, an axpy), the band's
//      last GEMM (k >= k1, with the bias / activation epilogue) finishes it,
//      and it goes back to the host while later bands compute -- so the
//      copy back of C overlaps the copies in, instead of following the last
//      GEMM.
// Phase 1 alone would finish every row of C at the very end (each needs all
// of k); phase 2 alone would keep the GEMMs idle until all of op(B) is in.
// With k1 about half of K both the link and the tensor cores stay busy.
// The result is the same GEMM with the k sum cut at slab boundaries (one
// FP32 add per boundary and element).
// Device staging: op(A), op(B), C and (beta != 0) the incoming C, whole, with
// 16-byte pitches so that TMA can describe them whatever the host leading
// dimensions are; in the split forms each slab and band is split into bf16
// pieces once, on its own stream, while the previous GEMM runs.
//
// Host buffers.  The reference's callers pass pageable memory (sgemm_test.c
// declares `static float A[...]` and hands it to sgemm_ocl, whose oclWrite
// copies it, sgemm_ocl2.h:173-176).  A cudaMemcpyAsync from or to pageable
// memory returns only when the copy is done, which in one host thread would
// serialise every copy and launch behind it.  So when a buffer is pageable
// the copies run from two helper host threads -- the copies in, in the order
// the GEMMs need them, and the bands of C back, each as soon as its GEMM is
// done -- while this thread launches: before a launch that needs a copy it
// waits for that copy only.  The copy engines move pageable memory nearly as
// fast as pinned memory (GB300 with a Grace host, measured: 184-196 GB/s
// in, 191 GB/s out, against 210 and 192 pinned).  Two alternatives were
// measured at 8192^3 and are kept behind UGEMM_PAGEABLE: copy kernels that
// read pageable memory through the host link's address translation
// ("kernel": 203 GB/s alone, but beside the GEMMs they ran at 121 GB/s and
// slowed the GEMMs by a quarter: 161 TFLOPS end to end) and registering the
// buffers for the call ("register": 1.9 ms of page pinning per call, 168
// TFLOPS), against 239 with pinned buffers.  Pinned buffers use the copy
// engines from this thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"
#include "split_tc.cuh"

namespace ugemm {
namespace {

constexpr int kMaxSlabs = 16, kMaxBands = 64;

struct PipeState {
  bool ready = false;
  // h2d: every copy in, in the order the GEMMs need it; prep: splits and
  // the beta * C folds; gemm[0]: the slab GEMMs, then even bands; gemm[1]:
  // odd bands; d2h: finished bands back
  cudaStream_t h2d = nullptr, d2h = nullptr, prep = nullptr, gemm[2] = {nullptr, nullptr};
  cudaEvent_t entry, acc_done, rest_in, rest_ready, last_out;
  cudaEvent_t slab_in[kMaxSlabs], slab_ready[kMaxSlabs];
  cudaEvent_t band_in[kMaxBands], band_ready[kMaxBands], band_done[kMaxBands];
};

std::mutex g_pmu;
PipeState g_pipe[64];

ugemm_status pipe_state(PipeState** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return UGEMM_ERR_CUDA;
  PipeState& p = g_pipe[dev];
  if (!p.ready) {
    const unsigned fl = cudaStreamNonBlocking;
    // the splits and folds run at the highest priority: their CTAs do not fit
    // beside a running GEMM's, so they go first whenever one ends
    int lo = 0, hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&p.prep, fl, hi) != cudaSuccess)
      return UGEMM_ERR_CUDA;
    for (cudaStream_t* s : {&p.h2d, &p.d2h, &p.gemm[0], &p.gemm[1]})
      if (cudaStreamCreateWithFlags(s, fl) != cudaSuccess) return UGEMM_ERR_CUDA;
    std::vector<cudaEvent_t*> all = {&p.entry, &p.acc_done, &p.rest_in, &p.rest_ready,
                                     &p.last_out};
    for (int i = 0; i < kMaxSlabs; ++i) { all.push_back(&p.slab_in[i]); all.push_back(&p.slab_ready[i]); }
    for (int r = 0; r < kMaxBands; ++r) {
      all.push_back(&p.band_in[r]);
      all.push_back(&p.band_ready[r]);
      all.push_back(&p.band_done[r]);
    }
    for (cudaEvent_t* e : all)
      if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return UGEMM_ERR_CUDA;
    p.ready = true;
  }
  *out = &p;
  return UGEMM_OK;
}

bool is_split(int form) {
  return form == UGEMM_PREC_BF16X6 || form == UGEMM_PREC_BF16X9 || form == UGEMM_PREC_BF16X3 ||
         form == UGEMM_PREC_FP16X3 || form == UGEMM_PREC_TF32X3;
}

int pitch4(int n) { return static_cast<int>(align_up(n, 4)); }

// A 2-D copy of `rows` rows of `width` bytes (a multiple of 4) between
// pitched buffers, either of which may be pageable host memory the device
// addresses directly.  Blocks take rows grid-stride; each thread keeps four
// 16-byte (or 4-byte) loads in flight before storing them, which covers the
// host link's latency with a few dozen CTAs.
template <typename T>
__global__ void __launch_bounds__(256) copy2d_kernel(const uint8_t* __restrict__ src, size_t spitch,
                                                     uint8_t* __restrict__ dst, size_t dpitch,
                                                     size_t width, int rows) {
  const size_t n = width / sizeof(T);
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const T* s = reinterpret_cast<const T*>(src + size_t(r) * spitch);
    T* d = reinterpret_cast<T*>(dst + size_t(r) * dpitch);
    for (size_t c = threadIdx.x; c < n; c += 4 * 256) {
      T v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const size_t i = c + size_t(u) * 256;
        if (i < n) v[u] = s[i];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const size_t i = c + size_t(u) * 256;
        if (i < n) d[i] = v[u];
      }
    }
  }
}

// CTAs of one copy kernel (UGEMM_COPY_CTAS overrides): enough bytes in
// flight for the host link.
int copy_ctas() {
  static const int n = [] {
    const char* e = std::getenv("UGEMM_COPY_CTAS");
    const int v = e ? std::atoi(e) : 0;
    return v > 0 ? v : 48;
  }();
  return n;
}

bool copy2d_launch(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, int rows,
                   cudaStream_t st) {
  if (rows <= 0 || width == 0) return true;
  const auto* s = static_cast<const uint8_t*>(src);
  auto* d = static_cast<uint8_t*>(dst);
  const int grid = std::min(rows, copy_ctas());
  const bool vec = ((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d) | spitch |
                     dpitch | width) & 15) == 0;
  prof_begin(st);
  if (vec) copy2d_kernel<float4><<<grid, 256, 0, st>>>(s, spitch, d, dpitch, width, rows);
  else copy2d_kernel<float><<<grid, 256, 0, st>>>(s, spitch, d, dpitch, width, rows);
  prof_end(st, kProfCopy);
  return cudaPeekAtLastError() == cudaSuccess;
}

// Whether the current device can read and write pageable host memory
// directly (address translation through the host's page tables).
bool device_reads_pageable() {
  static int cached[64];
  static std::once_flag once[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  std::call_once(once[dev], [dev] {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev);
    cached[dev] = v;
  });
  return cached[dev] != 0;
}

// How the copies of one host buffer cross the link: the copy engines from
// this thread (pinned or registered memory), the copy engines from a helper
// thread (pageable memory: the copy returns when done), copy kernels (reads
// of pageable memory the device addresses), or the copy engines after
// registering the buffer for the call.
enum class Xfer { kEngine, kThread, kKernel, kRegistered };

bool is_pageable(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return true;
  }
  return a.type == cudaMemoryTypeUnregistered;
}

// The buffers a call registered, released when it returns (after the
// device is idle: an early error return may leave copies in flight).
struct Registrations {
  std::vector<void*> ptrs;
  ~Registrations() {
    if (ptrs.empty()) return;
    cudaDeviceSynchronize();
    for (void* p : ptrs) cudaHostUnregister(p);
  }
};

// UGEMM_PAGEABLE selects how pageable buffers travel: "threads" (the
// default), "kernel" (reads by copy kernels where the device addresses
// pageable memory) or "register".
int pageable_mode() {
  static const int m = [] {
    const char* e = std::getenv("UGEMM_PAGEABLE");
    if (e && std::strcmp(e, "kernel") == 0) return 1;
    if (e && std::strcmp(e, "register") == 0) return 2;
    return 0;
  }();
  return m;
}

Xfer xfer_for(const void* p, size_t bytes, Registrations& regs) {
  if (!p || bytes == 0 || !is_pageable(p)) return Xfer::kEngine;
  if (pageable_mode() == 1 && device_reads_pageable()) return Xfer::kKernel;
  if (pageable_mode() == 2) {
    void* q = const_cast<void*>(p);
    if (cudaHostRegister(q, bytes, cudaHostRegisterDefault) == cudaSuccess) {
      regs.ptrs.push_back(q);
      return Xfer::kRegistered;
    }
    (void)cudaGetLastError();
  }
  return Xfer::kThread;
}

// A host thread that runs numbered steps in order (each may block) and
// counts the ones done; other threads wait for a given step.  Stopping makes
// waits fail and the thread finish after its current step.  Joined on
// destruction, so it never outlives the buffers its steps use.
class StepThread {
 public:
  ~StepThread() { stop(); }
  template <typename Step>
  void start(int n, Step step) {
    th_ = std::thread([this, n, step] {
      for (int i = 0; i < n; ++i) {
        if (stopped() || !step(i)) {
          std::lock_guard<std::mutex> l(mu_);
          failed_ = true;
          cv_.notify_all();
          return;
        }
        std::lock_guard<std::mutex> l(mu_);
        done_ = i + 1;
        cv_.notify_all();
      }
    });
  }
  bool wait(int i) {  // step i done; false if the thread failed or stopped first
    std::unique_lock<std::mutex> l(mu_);
    cv_.wait(l, [&] { return done_ > i || failed_ || stop_; });
    return done_ > i;
  }
  bool join() {  // all steps ran
    if (th_.joinable()) th_.join();
    std::lock_guard<std::mutex> l(mu_);
    return !failed_;
  }
  void stop() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
      cv_.notify_all();
    }
    if (th_.joinable()) th_.join();
  }

 private:
  bool stopped() {
    std::lock_guard<std::mutex> l(mu_);
    return stop_;
  }
  std::thread th_;
  std::mutex mu_;
  std::condition_variable cv_;
  int done_ = 0;
  bool failed_ = false, stop_ = false;
};

// A count that one thread raises and another waits on (launches recorded).
class Counter {
 public:
  void raise(int n) {
    std::lock_guard<std::mutex> l(mu_);
    n_ = n;
    cv_.notify_all();
  }
  void abort() {
    std::lock_guard<std::mutex> l(mu_);
    aborted_ = true;
    cv_.notify_all();
  }
  bool wait(int n) {
    std::unique_lock<std::mutex> l(mu_);
    cv_.wait(l, [&] { return n_ >= n || aborted_; });
    return n_ >= n;
  }

 private:
  std::mutex mu_;
  std::condition_variable cv_;
  int n_ = 0;
  bool aborted_ = false;
};

// (kThread copies are issued like kEngine ones, from the helper thread)
bool copy2d(Xfer x, void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
            int rows, cudaMemcpyKind kind, cudaStream_t st) {
  if (x == Xfer::kKernel) return copy2d_launch(dst, dpitch, src, spitch, width, rows, st);
  return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, st) == cudaSuccess;
}

// Layout of one pipelined call: k1 = depth of the slab phase (0: bands
// only), the slab width and band height, the device pitches and the bytes of
// every staging buffer.
struct Layout {
  bool split = false, fold = false;
  int k1 = 0, k2 = 0, nslab = 0, nband = 0;
  std::vector<int> slab_k0, slab_w;  // slab i: k in [slab_k0[i], slab_k0[i] + slab_w[i])
  std::vector<int> band_m0, band_h;  // band r: rows [band_m0[r], band_m0[r] + band_h[r])
  int lda_d = 0, ldb_d = 0, ldc_d = 0;
  long long a_sr = 0, a_sk = 0, b_sr = 0, b_sk = 0;
  SplitPlan plan, plan_acc;
  size_t a_bytes = 0, b_bytes = 0, c_bytes = 0, tail_acc = 0, tail_band = 0, band_ap = 0,
         rest_bp = 0, total = 0;
  std::vector<size_t> slab_ap, slab_bp;
};

// The slab GEMMs: no epilogue, it belongs to each band's last GEMM.
Gemm acc_gemm(const Gemm& g) {
  Gemm a = g;
  a.epi = Epilogue{};
  return a;
}

bool pipe_layout(const Gemm& g, int form, Layout* out) {
  Layout L;
  L.split = is_split(form);
  if (!L.split && form != UGEMM_PREC_SIMT) return false;
  if (g.K == 0 || g.alpha == 0.f || g.M < 2048) return false;
  const size_t bytes = 4 * (size_t(g.M) * g.K + size_t(g.K) * g.N + size_t(g.M) * g.N);
  if (bytes < (size_t(64) << 20)) return false;
  // bands of whole 128-row tiles, about 1024 rows each, the last quarter of
  // them halved: the last band's GEMM and copy back are what is left after
  // the last byte has crossed the link
  const int nb0 = std::min(std::max(g.M / 1024, 2), kMaxBands / 2);
  const int band = static_cast<int>(align_up(cdiv(g.M, nb0), 128));
  const int halved = cdiv(nb0, 4);
  for (int m0 = 0, r = 0; m0 < g.M; m0 += band, ++r) {
    const int h = std::min(band, g.M - m0);
    const int h0 = static_cast<int>(align_up(cdiv(h, 2), 128));
    if (r >= nb0 - halved && h0 < h) {
      L.band_h.push_back(h0);
      L.band_h.push_back(h - h0);
    } else {
      L.band_h.push_back(h);
    }
  }
  // slab phase: half of k, when k is deep enough for it to pay, in slabs of
  // an eighth, three eighths and a half of it: the first GEMM starts after
  // a small slab has crossed, and each slab's copy hides behind the
  // previous slab's GEMM
  if (g.K >= 2048) {
    const int k1 = g.K / 2 / 256 * 256;
    const int w0 = static_cast<int>(align_up(k1 / 8, 256)), w1 = static_cast<int>(align_up(3 * k1 / 8, 256));
    if (k1 >= 2048 && w0 + w1 < k1) {
      L.slab_w = {w0, w1, k1 - w0 - w1};
    } else {
      L.slab_w = {k1};
    }
  }
  L.k1 = 0;
  for (int w : L.slab_w) { L.slab_k0.push_back(L.k1); L.k1 += w; }
  for (int m0 = 0, r = 0; r < static_cast<int>(L.band_h.size()); m0 += L.band_h[r++]) L.band_m0.push_back(m0);
  L.nslab = static_cast<int>(L.slab_w.size());
  L.nband = static_cast<int>(L.band_h.size());
  L.ldc_d = pitch4(g.N);
  if (L.nband < 2 || L.nband > kMaxBands || L.nslab > kMaxSlabs || L.k1 >= g.K) return false;
  int rows = 0;
  for (int h : L.band_h) {
    if (h <= 0 || size_t(h) * L.ldc_d >= (size_t(1) << 31)) return false;
    rows += h;
  }
  for (int w : L.slab_w)
    if (w <= 0) return false;
  if (rows != g.M) return false;
  L.k2 = g.K - L.k1;
  L.fold = g.beta != 0.f && L.k1 > 0;
  // device layouts: op(A) and op(B) in their host storage order, whole
  const int a_rows = g.ta == 'N' ? g.M : g.K, a_cols = g.ta == 'N' ? g.K : g.M;
  const int b_rows = g.tb == 'N' ? g.K : g.N, b_cols = g.tb == 'N' ? g.N : g.K;
  L.lda_d = pitch4(a_cols);
  L.ldb_d = pitch4(b_cols);
  // op(A)(m, k) at dA[m*a_sr + k*a_sk]; op(B)^T(n, k) at dB[n*b_sr + k*b_sk]
  L.a_sr = g.ta == 'N' ? L.lda_d : 1;
  L.a_sk = g.ta == 'N' ? 1 : L.lda_d;
  L.b_sr = g.tb == 'N' ? 1 : L.ldb_d;
  L.b_sk = g.tb == 'N' ? L.ldb_d : 1;
  L.a_bytes = align_up(size_t(a_rows) * L.lda_d * 4, 256);
  L.b_bytes = align_up(size_t(b_rows) * L.ldb_d * 4, 256);
  L.c_bytes = align_up(size_t(g.M) * L.ldc_d * 4, 256);
  L.slab_ap.assign(L.nslab, 0);
  L.slab_bp.assign(L.nslab, 0);
  if (L.split) {
    const Gemm ga = acc_gemm(g);
    L.plan = split_plan_for(form, g);
    L.plan_acc = split_plan_for(form, ga);
    for (int i = 0; i < L.nslab; ++i) {
      Gemm gs = ga;
      gs.K = L.slab_w[i];
      L.slab_ap[i] = split_operand_bytes(L.plan.pieces, g.M, gs.K);
      L.slab_bp[i] = split_operand_bytes(L.plan.pieces, g.N, gs.K);
      L.tail_acc = std::max(L.tail_acc, tail_scratch_bytes(gs, L.plan_acc));
    }
    for (int h : L.band_h) L.band_ap = std::max(L.band_ap, split_operand_bytes(L.plan.pieces, h, L.k2));
    L.rest_bp = split_operand_bytes(L.plan.pieces, g.N, L.k2);
    for (int mb : L.band_h) {
      Gemm gb = g;
      gb.M = mb;
      gb.K = L.k2;
      L.tail_band = std::max(L.tail_band, tail_scratch_bytes(gb, L.plan));
    }
  }
  L.total = L.a_bytes + L.b_bytes + L.c_bytes * (L.fold ? 2 : 1) + L.tail_acc + 2 * L.tail_band +
            size_t(L.nband) * L.band_ap + L.rest_bp;
  for (int i = 0; i < L.nslab; ++i) L.total += L.slab_ap[i] + L.slab_bp[i];
  *out = std::move(L);
  return true;
}

}  // namespace

size_t host_pipelined_bytes(const Gemm& g, int form) {
  Layout L;
  return pipe_layout(g, form, &L) ? L.total : 0;
}

ugemm_status host_gemm_pipelined(const Gemm& g, int form, void* arena, size_t arena_bytes,
                                 int* dev_err, cudaStream_t caller) {
  Layout L;
  if (!pipe_layout(g, form, &L) || L.total > arena_bytes) return UGEMM_ERR_UNSUPPORTED;
  const bool split = L.split, fold = L.fold;
  const int k1 = L.k1, k2 = L.k2, lda_d = L.lda_d, ldb_d = L.ldb_d, ldc_d = L.ldc_d;
  const long long a_sr = L.a_sr, a_sk = L.a_sk, b_sr = L.b_sr, b_sk = L.b_sk;
  const Gemm g_acc = acc_gemm(g);

  std::lock_guard<std::mutex> lock(g_pmu);
  PipeState* ps = nullptr;
  if (pipe_state(&ps) != UGEMM_OK) return UGEMM_ERR_CUDA;
  // how each host buffer crosses the link (registrations end with the call,
  // after its last copy has been waited for)
  Registrations regs;
  const size_t a_span = ((g.ta == 'N' ? size_t(g.M) : size_t(g.K)) - 1) * g.lda +
                        (g.ta == 'N' ? g.K : g.M);
  const size_t b_span = ((g.tb == 'N' ? size_t(g.K) : size_t(g.N)) - 1) * g.ldb +
                        (g.tb == 'N' ? g.N : g.K);
  const size_t c_span = (size_t(g.M) - 1) * g.ldc + g.N;
  const Xfer xa = xfer_for(g.A, a_span * 4, regs), xb = xfer_for(g.B, b_span * 4, regs);
  const Xfer xc = xfer_for(g.C, c_span * 4, regs);
  // copies from or into pageable memory that return when done run in helper
  // threads (C goes back that way also when copy kernels read it in)
  const bool in_threaded = xa == Xfer::kThread || xb == Xfer::kThread ||
                           (g.beta != 0.f && xc == Xfer::kThread);
  const bool out_threaded = xc == Xfer::kThread || xc == Xfer::kKernel;
  uint8_t* base = static_cast<uint8_t*>(arena);
  size_t off = 0;
  auto take = [&](size_t n) { uint8_t* p = base + off; off += n; return p; };
  float* dA = reinterpret_cast<float*>(take(L.a_bytes));
  float* dB = reinterpret_cast<float*>(take(L.b_bytes));
  float* dC = reinterpret_cast<float*>(take(L.c_bytes));
  float* dCin = fold ? reinterpret_cast<float*>(take(L.c_bytes)) : dC;
  void* tail_s_acc = L.tail_acc ? take(L.tail_acc) : nullptr;
  void* tail_s_band[2] = {L.tail_band ? take(L.tail_band) : nullptr,
                          L.tail_band ? take(L.tail_band) : nullptr};
  std::vector<void*> sap(L.nslab), sbp(L.nslab), bap(L.nband);
  void* rbp = nullptr;
  if (split) {
    for (int i = 0; i < L.nslab; ++i) { sap[i] = take(L.slab_ap[i]); sbp[i] = take(L.slab_bp[i]); }
    for (int r = 0; r < L.nband; ++r) bap[r] = take(L.band_ap);
    rbp = take(L.rest_bp);
  }
  auto ck = [](cudaError_t e) { return e == cudaSuccess; };

  // The copies in, as a list in the order the GEMMs consume them; the last
  // copy of each group records the group's event.
  struct CopyIn {
    Xfer x;
    void* dst;
    size_t dpitch;
    const void* src;
    size_t spitch, width;
    int rows;
    cudaEvent_t after;
  };
  std::vector<CopyIn> ins;
  // a region of op(A) (rows m0.., k0..) or op(B) (k0.., columns n0..) from
  // the host operand into the same place of the device copy
  auto copy_a = [&](int m0, int mr, int k0, int kw) {
    const int r0 = g.ta == 'N' ? m0 : k0, c0 = g.ta == 'N' ? k0 : m0;
    const int nr = g.ta == 'N' ? mr : kw, nc = g.ta == 'N' ? kw : mr;
    ins.push_back(CopyIn{xa, dA + size_t(r0) * lda_d + c0, size_t(lda_d) * 4,
                         g.A + size_t(r0) * g.lda + c0, size_t(g.lda) * 4, size_t(nc) * 4, nr,
                         nullptr});
  };
  auto copy_b = [&](int k0, int kw) {  // all N columns of op(B), k rows k0..k0+kw
    const int r0 = g.tb == 'N' ? k0 : 0, c0 = g.tb == 'N' ? 0 : k0;
    const int nr = g.tb == 'N' ? kw : g.N, nc = g.tb == 'N' ? g.N : kw;
    ins.push_back(CopyIn{xb, dB + size_t(r0) * ldb_d + c0, size_t(ldb_d) * 4,
                         g.B + size_t(r0) * g.ldb + c0, size_t(g.ldb) * 4, size_t(nc) * 4, nr,
                         nullptr});
  };
  auto close_group = [&](cudaEvent_t e) {
    ins.back().after = e;
    return static_cast<int>(ins.size()) - 1;
  };
  auto a_view = [&](int m0, int k0) { return dA + m0 * a_sr + k0 * a_sk; };
  auto b_view = [&](int k0) { return dB + k0 * b_sk; };

  // work queued earlier on the caller's stream comes first
  if (!ck(cudaEventRecord(ps->entry, caller))) return UGEMM_ERR_CUDA;
  for (cudaStream_t s : {ps->h2d, ps->d2h, ps->prep, ps->gemm[0], ps->gemm[1]})
    if (!ck(cudaStreamWaitEvent(s, ps->entry, 0))) return UGEMM_ERR_CUDA;

  // ---- copies in, in the order the GEMMs consume them
  std::vector<int> slab_in_op(L.nslab), band_in_op(L.nband);
  for (int i = 0; i < L.nslab; ++i) {
    copy_a(0, g.M, L.slab_k0[i], L.slab_w[i]);
    copy_b(L.slab_k0[i], L.slab_w[i]);
    slab_in_op[i] = close_group(ps->slab_in[i]);
  }
  copy_b(k1, k2);
  const int rest_in_op = close_group(ps->rest_in);
  for (int r = 0; r < L.nband; ++r) {
    const int m0 = L.band_m0[r], mb = L.band_h[r];
    copy_a(m0, mb, k1, k2);
    if (g.beta != 0.f)  // beta == 0: C is not read (sgemm_ocl2.h:177)
      ins.push_back(CopyIn{xc, dCin + size_t(m0) * ldc_d, size_t(ldc_d) * 4,
                           g.C + size_t(m0) * g.ldc, size_t(g.ldc) * 4, size_t(g.N) * 4, mb,
                           nullptr});
    band_in_op[r] = close_group(ps->band_in[r]);
  }
  auto run_in = [&](int i) {
    const CopyIn& o = ins[i];
    return copy2d(o.x, o.dst, o.dpitch, o.src, o.spitch, o.width, o.rows, cudaMemcpyHostToDevice,
                  ps->h2d) &&
           (!o.after || ck(cudaEventRecord(o.after, ps->h2d)));
  };
  // the helpers are declared after everything their steps use (the counter
  // included), so they are joined first on every return; the guard declared
  // last releases a drainer still waiting for a band that an error return
  // will never launch
  Counter bands_launched;
  StepThread feeder, drainer;
  struct AbortOnExit {
    Counter& c;
    ~AbortOnExit() { c.abort(); }
  } abort_drain{bands_launched};
  if (in_threaded) {
    feeder.start(static_cast<int>(ins.size()), run_in);
  } else {
    for (int i = 0; i < static_cast<int>(ins.size()); ++i)
      if (!run_in(i)) return UGEMM_ERR_CUDA;
  }
  // before a launch that waits on a group's event: that event is recorded
  auto await_in = [&](int op) { return !in_threaded || feeder.wait(op); };
  // the bands of C back to the host, each once its GEMM is done
  auto run_out = [&](int r) {
    const int m0 = L.band_m0[r], mb = L.band_h[r];
    const Xfer x = out_threaded ? Xfer::kEngine : xc;
    return ck(cudaStreamWaitEvent(ps->d2h, ps->band_done[r], 0)) &&
           copy2d(x, g.C + size_t(m0) * g.ldc, size_t(g.ldc) * 4, dC + size_t(m0) * ldc_d,
                  size_t(ldc_d) * 4, size_t(g.N) * 4, mb, cudaMemcpyDeviceToHost, ps->d2h);
  };
  if (out_threaded)
    drainer.start(L.nband, [&](int r) { return bands_launched.wait(r + 1) && run_out(r); });

  // ---- phase 1: slab GEMMs into the accumulator dC, one after another
  cudaStream_t g0 = ps->gemm[0];
  for (int i = 0; i < L.nslab; ++i) {
    const int k0 = L.slab_k0[i], w = L.slab_w[i];
    if (!await_in(slab_in_op[i])) return UGEMM_ERR_CUDA;
    if (split) {
      cudaStreamWaitEvent(ps->prep, ps->slab_in[i], 0);
      if (split_operand_launch(L.plan.pieces, a_view(0, k0), a_sr, a_sk, g.M, w, sap[i], ps->prep,
                               L.plan.f16) != UGEMM_OK ||
          split_operand_launch(L.plan.pieces, b_view(k0), b_sr, b_sk, g.N, w, sbp[i], ps->prep,
                               L.plan.f16) != UGEMM_OK)
        return UGEMM_ERR_CUDA;
      if (!ck(cudaEventRecord(ps->slab_ready[i], ps->prep))) return UGEMM_ERR_CUDA;
      cudaStreamWaitEvent(g0, ps->slab_ready[i], 0);
    } else {
      cudaStreamWaitEvent(g0, ps->slab_in[i], 0);
    }
    Gemm gs = g_acc;
    gs.K = w;
    gs.A = a_view(0, k0);
    gs.lda = lda_d;
    gs.B = b_view(k0);
    gs.ldb = ldb_d;
    gs.C = dC;
    gs.ldc = ldc_d;
    gs.beta = i == 0 ? 0.f : 1.f;
    ugemm_status st = split ? split_gemm_on_pieces(gs, L.plan_acc, sap[i], sbp[i], tail_s_acc, dev_err, g0)
                            : simt_launch(gs, simt_pick_tile(gs), Scratch{nullptr, 0}, dev_err, g0);
    if (st != UGEMM_OK) return st;
  }
  if (!ck(cudaEventRecord(ps->acc_done, g0))) return UGEMM_ERR_CUDA;

  // ---- phase 2: the rest of op(B), then band by band
  if (!await_in(rest_in_op)) return UGEMM_ERR_CUDA;
  cudaStreamWaitEvent(ps->prep, ps->rest_in, 0);
  if (split && split_operand_launch(L.plan.pieces, b_view(k1), b_sr, b_sk, g.N, k2, rbp,
                                    ps->prep, L.plan.f16) != UGEMM_OK)
    return UGEMM_ERR_CUDA;
  if (!ck(cudaEventRecord(ps->rest_ready, ps->prep))) return UGEMM_ERR_CUDA;
  for (int r = 0; r < L.nband; ++r) {
    const int m0 = L.band_m0[r], mb = L.band_h[r];
    cudaStream_t gs_st = ps->gemm[r & 1];
    if (!await_in(band_in_op[r])) return UGEMM_ERR_CUDA;
    cudaStreamWaitEvent(ps->prep, ps->band_in[r], 0);
    if (split && split_operand_launch(L.plan.pieces, a_view(m0, k1), a_sr, a_sk, mb, k2, bap[r],
                                      ps->prep, L.plan.f16) != UGEMM_OK)
      return UGEMM_ERR_CUDA;
    if (fold) {  // acc += beta * C, once the slab GEMMs are done with acc
      if (r == 0) cudaStreamWaitEvent(ps->prep, ps->acc_done, 0);
      const int st = ugemm_saxpy(mb * ldc_d, g.beta, dCin + size_t(m0) * ldc_d, 1,
                                 dC + size_t(m0) * ldc_d, 1, ps->prep);
      if (st != UGEMM_OK) return UGEMM_ERR_CUDA;
    }
    if (!ck(cudaEventRecord(ps->band_ready[r], ps->prep))) return UGEMM_ERR_CUDA;
    cudaStreamWaitEvent(gs_st, ps->band_ready[r], 0);
    cudaStreamWaitEvent(gs_st, ps->rest_ready, 0);
    cudaStreamWaitEvent(gs_st, ps->acc_done, 0);
    Gemm gb = g;
    gb.M = mb;
    gb.K = k2;
    gb.A = a_view(m0, k1);
    gb.lda = lda_d;
    gb.B = b_view(k1);
    gb.ldb = ldb_d;
    gb.C = dC + size_t(m0) * ldc_d;
    gb.ldc = ldc_d;
    if (k1 > 0) gb.beta = 1.f;       // acc (with beta * C folded in)
    if (gb.epi.bias) gb.epi.bias += m0;  // per-row bias follows the band
    ugemm_status st = split ? split_gemm_on_pieces(gb, L.plan, bap[r], rbp, tail_s_band[r & 1],
                                                   dev_err, gs_st)
                            : simt_launch(gb, simt_pick_tile(gb), Scratch{nullptr, 0}, dev_err,
                                          gs_st);
    if (st != UGEMM_OK || !ck(cudaEventRecord(ps->band_done[r], gs_st))) return UGEMM_ERR_CUDA;
    bands_launched.raise(r + 1);
  }
  // ---- finished bands back to the host, each as soon as its GEMM is done
  if (out_threaded) {
    if (!drainer.join()) return UGEMM_ERR_CUDA;
  } else {
    for (int r = 0; r < L.nband; ++r)
      if (!run_out(r)) return UGEMM_ERR_CUDA;
  }
  if (in_threaded && !feeder.join()) return UGEMM_ERR_CUDA;
  // the caller's stream resumes after the last copy back
  if (!ck(cudaEventRecord(ps->last_out, ps->d2h))) return UGEMM_ERR_CUDA;
  cudaStreamWaitEvent(caller, ps->last_out, 0);
  return cudaStreamSynchronize(ps->d2h) == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace ugemm
