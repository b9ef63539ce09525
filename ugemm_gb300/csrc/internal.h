// internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

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
};

#ifdef __CUDACC__
__device__ __forceinline__ float epilogue_apply(float v, const Epilogue& e, int row) {
  if (e.bias) v += e.bias[row];
  if (e.act) v = v > 0.f ? v : v * e.slope;
  return v;
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
  bool epi = false;  // some problem carries a bias or activation: launch the
                     // kernel instantiation that has the fused epilogue
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

// Grouped plans: default tile configuration and the autotuner's cache.
ugemm_tile_config default_grouped_config(int form);
bool tuned_config(int count, const ugemm_problem* problems, int precision, ugemm_tile_config* cfg);
int split_default_chunk_kb();

// Host-pointer GEMM with overlapped copies (row bands of C); returns
// UGEMM_ERR_UNSUPPORTED when the call is too small or the arena too tight,
// in which case the caller runs the plain copy-compute-copy sequence.
ugemm_status host_gemm_pipelined(const Gemm& g, int form, void* arena, size_t arena_bytes,
                                 int* dev_err, cudaStream_t caller);

// Per-thread last error, shared by the void compat entry points.
void set_last_error(ugemm_status s, const std::string& msg);

}  // namespace ugemm

namespace ugemm {
// Optional per-kernel timing (CUDA events on the launching stream), enabled by
// ugemm_profile_enable; used by the benchmark to attribute time to kernels.
enum ProfKind : int { kProfSimt = 0, kProfSplitPrep = 1, kProfSplitGemm = 2, kProfAux = 3,
                      kProfGrouped = 4, kProfKinds = 5 };
void prof_begin(cudaStream_t st);
void prof_end(cudaStream_t st, int kind);
}  // namespace ugemm
