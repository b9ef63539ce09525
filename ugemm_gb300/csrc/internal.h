// internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/sgemm_cuda.h"

namespace ugemm {

// A row-major GEMM after argument normalisation (column-major calls are
// rewritten as the transposed row-major problem before they get here):
//   C[M x N] = alpha * op(A)[M x K] * op(B)[K x N] + beta * C
// ta == 'N': A is M x K (lda >= K);  ta == 'T': A is K x M (lda >= M).
// tb == 'N': B is K x N (ldb >= N);  tb == 'T': B is N x K (ldb >= K).
// beta == 0 means C is written without being read.
// Optional fused epilogue: C = act(alpha*op(A)op(B) + beta*C + bias[row]),
// act = LeakyReLU(slope) when `act` is non-zero (slope 0: ReLU).  This is the
// reference's post-GEMM loop of gl_convolution_LReLU (sgemm_gl1.h:210-217),
// which adds the per-channel bias and applies a 0.1 leak, moved into the
// GEMM epilogue.  Plain data, shared with the kernels.
struct Epilogue {
  const float* bias = nullptr;
  int act = 0;
  float slope = 0.1f;
};

// An operand read as the im2col matrix of a CNHW activation x without
// materialising it (implicit GEMM): entry (tap, pix), tap = c*k*k + ki*k + kj,
// pix = (b*Ho + i)*Wo + j, is x[c][b][i*stride - pad + ki][j*stride - pad + kj],
// 0 outside the image -- the reference's im2col (sgemm_ocl1.h:81-119) for a
// batch of images side by side.
// Division by a run-time constant d >= 1 of 0 <= x < 2^31 with one
// multiply-high, an add and a shift: q = (umulhi(x, m) + x) >> s with
// s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1 (the round-up method of
// Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994).
struct FastDiv {
  uint32_t d = 1, m = 1, s = 0;
  FastDiv() = default;
  explicit FastDiv(uint32_t div) : d(div) {
    while ((uint64_t(1) << s) < div) ++s;
    m = static_cast<uint32_t>(((uint64_t(1) << 32) * ((uint64_t(1) << s) - div)) / div + 1);
  }
#ifdef __CUDACC__
  __device__ __forceinline__ int operator()(int x) const {
    const uint32_t u = static_cast<uint32_t>(x);
    return static_cast<int>((__umulhi(u, m) + u) >> s);
  }
#endif
};

struct Im2col {
  const float* x = nullptr;
  int C = 0, B = 0, H = 0, W = 0, k = 0, pad = 0, stride = 1, Ho = 0, Wo = 0;
  FastDiv by_kk, by_k, by_hw, by_wo;  // k*k, k, Ho*Wo, Wo
};
inline Im2col make_im2col(const float* x, int C, int B, int H, int W, int k, int pad, int stride,
                          int Ho, int Wo) {
  Im2col g;
  g.x = x;
  g.C = C; g.B = B; g.H = H; g.W = W; g.k = k; g.pad = pad; g.stride = stride; g.Ho = Ho; g.Wo = Wo;
  g.by_kk = FastDiv(static_cast<uint32_t>(k * k));
  g.by_k = FastDiv(static_cast<uint32_t>(k));
  g.by_hw = FastDiv(static_cast<uint32_t>(Ho * Wo));
  g.by_wo = FastDiv(static_cast<uint32_t>(Wo));
  return g;
}

struct Gemm {
  char ta, tb;
  int M, N, K;
  float alpha, beta;
  const float* A;
  int lda;
  const float* B;
  int ldb;
  float* C;
  int ldc;
  Epilogue epi{};
  // grouped plans only: B is the im2col matrix of b_im2col->x (K x N taps x
  // pixels when tb == 'N', N x K when tb == 'T'); B and ldb are then unused
  const Im2col* b_im2col = nullptr;
};

#ifdef __CUDACC__
__device__ __forceinline__ float epilogue_apply(float v, const Epilogue& e, int row) {
  if (e.bias) v += e.bias[row];
  if (e.act) v = v > 0.f ? v : v * e.slope;
  return v;
}

// An im2col row (tap) and column (pixel) as coordinates; consecutive pixels
// step along j, then i, then b.
struct Im2colTap { int c, ki, kj; };
struct Im2colPix { int b, i, j; };

__device__ __forceinline__ Im2colTap im2col_tap(const Im2col& g, int tap) {
  const int c = g.by_kk(tap), t = tap - c * g.k * g.k, ki = g.by_k(t);
  return Im2colTap{c, ki, t - ki * g.k};
}
__device__ __forceinline__ Im2colPix im2col_pix(const Im2col& g, int pix) {
  const int b = g.by_hw(pix), q = pix - b * g.Ho * g.Wo, i = g.by_wo(q);
  return Im2colPix{b, i, q - i * g.Wo};
}
__device__ __forceinline__ void im2col_next(const Im2col& g, Im2colPix& p) {
  if (++p.j == g.Wo) {
    p.j = 0;
    if (++p.i == g.Ho) { p.i = 0; ++p.b; }
  }
}
__device__ __forceinline__ float im2col_load(const Im2col& g, const Im2colTap& t,
                                             const Im2colPix& p) {
  const int yy = p.i * g.stride - g.pad + t.ki, xx = p.j * g.stride - g.pad + t.kj;
  if (yy < 0 || yy >= g.H || xx < 0 || xx >= g.W) return 0.f;
  return g.x[((static_cast<long long>(t.c) * g.B + p.b) * g.H + yy) * g.W + xx];
}
#endif

// Device scratch handed to a launcher.  `bytes` is what is available at `ptr`.
struct Scratch {
  void* ptr;
  size_t bytes;
};

// Tile configurations of the SIMT kernel (rows x cols of C per CTA).
// 128x128 and 64x64 use 8 compute warps plus a TMA producer warp; the "np"
// configurations drop the producer warp (thread 0 issues the copies), which
// lifts the per-thread register limit from 168 to 255.
enum SimtTile : int {
  kSimt128x128 = 0,
  kSimt64x64 = 1,
  kSimt128x256 = 2,    // 8 x 16 per thread, producer-less
  kSimt128x128np = 3,  // 8 x 8 per thread, producer-less
  kSimtTileCount = 4
};

// Split-precision tensor-core variants.
struct SplitPlan {
  int pieces;        // bf16 pieces per FP32 operand (2 or 3)
  int products;      // number of piece products accumulated (3, 6 or 9)
  int block_n;       // CTA tile width (128 or 256)
  int chunk_kb = 0;  // k-blocks per main-accumulator chunk (0: library default)
  bool f16 = false;  // FP16x3: scaled fp16 pieces (pieces == 2) instead of bf16
  bool epi = false;  // some problem carries a bias or activation: launch the
                     // kernel instantiation that has the fused epilogue
  bool fused = false;  // grouped launches of three bf16 pieces, 128-wide
                       // tiles: the GEMM kernel splits the FP32 operands
                       // itself (no pre-pass, no pieces in memory)
};

// --- tensor maps -------------------------------------------------------
bool encode_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, int elem_bytes,
                    const void* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                    uint32_t box_inner, uint32_t box_outer, CUtensorMapSwizzle swz);
bool encode_tmap_3d(CUtensorMap* map, CUtensorMapDataType dtype, int elem_bytes,
                    const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t stride1,
                    uint64_t stride2, uint32_t b0, uint32_t b1, uint32_t b2,
                    CUtensorMapSwizzle swz);

// --- SIMT path ---------------------------------------------------------
size_t simt_scratch_bytes(const Gemm& g);
ugemm_status simt_launch(const Gemm& g, int tile, Scratch ws, int* dev_err, cudaStream_t st);
int simt_pick_tile(const Gemm& g);

// --- split-precision tensor-core path ----------------------------------
size_t split_scratch_bytes(const Gemm& g, const SplitPlan& p);
ugemm_status split_launch(const Gemm& g, const SplitPlan& p, Scratch ws, int* dev_err,
                          cudaStream_t st);
SplitPlan split_plan_for(int precision, const Gemm& g);

// --- small helpers -----------------------------------------------------
// Raise a kernel's dynamic shared-memory limit on the current device, once
// per device (the attribute belongs to the device's context).  `done` is the
// caller's per-kernel record of devices already set; a race only repeats an
// idempotent call.
template <typename Kernel>
bool smem_attr_once(Kernel kern, size_t bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  const uint64_t bit = uint64_t(1) << dev;
  if (done.load(std::memory_order_acquire) & bit) return true;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(bytes)) != cudaSuccess)
    return false;
  done.fetch_or(bit, std::memory_order_release);
  return true;
}
ugemm_status scale_c_launch(const Gemm& g, cudaStream_t st);  // C = beta*C (or 0)
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// Split-K: one GEMM cut into k slices, slice s having written
// alpha * (its partial product) to part + s*M*N (row-major, ld N).  The
// reduce forms C = sum_s part_s + beta*C (C not read when beta == 0), then
// the optional bias / activation, summing the slices in a fixed order.
struct ReduceJob {
  const float* part;
  float* C;
  int M, N, ldc, slices;
  float beta;
  Epilogue epi;
};
ugemm_status splitk_reduce_launch(const ReduceJob* jobs, int njobs, long long max_mn,
                                  cudaStream_t st);

// Up to kMultiMax split-precision GEMMs (and split-K slices of them) in one
// persistent launch, scratch in the caller's workspace (multi.cu).
constexpr int kMultiMax = 4;
bool multi_wanted(const Gemm& g, const SplitPlan& p);  // under-filled, deep k
size_t multi_scratch_bytes(const Gemm* gs, int n, const SplitPlan& p);
ugemm_status multi_launch(const Gemm* gs, int n, const SplitPlan& p, Scratch ws, int* dev_err,
                          cudaStream_t st);

// Grouped plans: the builder behind ugemm_grouped_plan_create (validated
// problems, longest k first inside), default tile configuration and the
// autotuner's cache.  config == nullptr: the default configuration.
ugemm_status grouped_plan_build(const Gemm* gs, int count, int form,
                                const ugemm_tile_config* config, int flags,
                                ugemm_grouped_plan** out);
ugemm_tile_config default_grouped_config(int form);
bool tuned_config(int count, const ugemm_problem* problems, int precision, ugemm_tile_config* cfg);
int split_default_chunk_kb(int K);

// Host-pointer GEMM with overlapped copies (k slabs, then row bands of C); returns
// UGEMM_ERR_UNSUPPORTED when the call is too small or the arena too tight,
// in which case the caller runs the plain copy-compute-copy sequence.
// Device arena bytes the pipelined host path needs for this call (0: the
// call is not pipelined).
size_t host_pipelined_bytes(const Gemm& g, int form);
ugemm_status host_gemm_pipelined(const Gemm& g, int form, void* arena, size_t arena_bytes,
                                 int* dev_err, cudaStream_t caller);

// Per-thread last error, shared by the void compat entry points.
void set_last_error(ugemm_status s, const std::string& msg);

// The allocation-free entry point's two error words on the current device
// ([0] written by its kernels, [1] the code held for ugemm_check), or null
// before its first call on the device.
int* noalloc_error_words();

}  // namespace ugemm

namespace ugemm {
// Optional per-kernel timing (CUDA events on the launching stream), enabled by
// ugemm_profile_enable; used by the benchmark to attribute time to kernels.
enum ProfKind : int { kProfSimt = 0, kProfSplitPrep = 1, kProfSplitGemm = 2, kProfAux = 3,
                      kProfGrouped = 4, kProfControl = 5, kProfCopy = 6, kProfKinds = 7 };
void prof_begin(cudaStream_t st);
void prof_end(cudaStream_t st, int kind);
}  // namespace ugemm
