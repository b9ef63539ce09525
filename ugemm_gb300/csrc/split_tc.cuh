// split_tc.cuh -- types shared by the split-precision tensor-core kernels
// (split_tc.cu) and the grouped GEMM planner (grouped.cu).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include <vector>

#include "internal.h"

namespace ugemm {

constexpr int kTcBM = 128;       // rows of C per CTA tile (UMMA M)
constexpr int kTcKB = 32;        // k depth of one pipeline stage (64-byte bf16 rows)
constexpr int kTcEpiWarps = 8;   // two per TMEM lane quarter
constexpr int kTcThreads = (2 + kTcEpiWarps) * 32;
// Fused launches (the operands split inside the GEMM kernel): warp 0's TMA
// copies bring raw FP32 tiles of the operands into a ring of kTcRawStages
// stages, which converter threads split into the three bf16 pieces of a
// piece stage (kTcFusedPieceStages of them); the MMA issuer reads those as
// it reads pre-split pieces.  128-wide tiles: kTcConvWarps more warps after
// the epilogue warps (six: sixteen warps in all, 128 registers each), raw
// stages 32 k deep.  256-wide tiles: the accumulator of a 128 x 256 tile
// needs 128 registers in each epilogue thread, so there is no register room
// for more warps; the eight epilogue warps convert as well (ten warps, up to
// 200 registers each), and the raw stages are 16 k deep, so that two piece
// stages and three raw stages fit in shared memory.
constexpr int kTcConvWarps = 6;
constexpr int kTcConvThreads = kTcConvWarps * 32;
constexpr int kTcFusedThreads = kTcThreads + kTcConvThreads;
constexpr int kTcFusedPieceStages = 2;
constexpr int kTcRawStages = 3;
// threads, converter threads and raw stage depth of a fused launch
__host__ __device__ constexpr int fused_threads(int bn) {
  return bn == 256 ? kTcThreads : kTcFusedThreads;
}
__host__ __device__ constexpr int fused_conv_threads(int bn) {
  return bn == 256 ? kTcEpiWarps * 32 : kTcConvThreads;
}
__host__ __device__ constexpr int fused_raw_k(int bn) { return bn == 256 ? kTcKB / 2 : kTcKB; }
// 256-wide fused launches keep the drained chunks of the main accumulator
// in global memory (L2) instead of registers: 128 x 256 FP32 per CTA.
constexpr size_t kTcFusedSumBytes = size_t(kTcBM) * 256 * 4;
constexpr int kTcRaster = 8;     // tile rows per raster group (L2 reuse)

// FP16x3 form: every row of an operand's K-major piece matrix -- a row of
// op(A), a column of op(B) -- is scaled by its own power of two 2^e, chosen
// from that row's largest magnitude m so that m * 2^e lies in [2^14, 2^15),
// and written as two fp16 pieces h0 = fp16(x 2^e), h1 = fp16(x 2^e - h0)
// (11 + 11 significand bits; the rest, < 2^-22 |x| 2^e, is dropped with the
// h1*g1 product).  The scale keeps fp16 from overflowing (largest 65504) and
// keeps both pieces of the row's large elements normal (h1 >= 2^-14); being
// per row and per column, it follows rows and columns of very different
// magnitudes, so one large element or one large row does not push the rest
// of the operand below fp16's range.  C[i][j] is then the accumulator times
// 2^-(eA[i] + eB[j]).  `bits` is the IEEE pattern of m (a row word written by
// atomicMax); an all-zero or non-finite m gives e = 0.  e lies in
// [-113, 163]: the largest finite float needs -113, the smallest subnormal
// 163.
__host__ __device__ __forceinline__ int f16_scale_exp(unsigned bits) {
  if (bits == 0u || bits >= 0x7F800000u) return 0;
  const int biased = static_cast<int>(bits >> 23);
  return 14 - (biased == 0 ? -127 : biased - 127);
}
// 2^e for -126 <= e <= 127, exactly.
__host__ __device__ __forceinline__ float pow2f(int e) {
  union { unsigned u; float f; } v;
  v.u = static_cast<unsigned>(127 + e) << 23;
  return v.f;
}
// x * 2^e.  One multiplication by a normal power of two when 2^e is one;
// otherwise two, each by a normal power of two, splitting e in halves (|e|
// is clamped to 252, beyond which any finite FP32 accumulator underflows to
// zero or the operand scales could not produce it).  A multiplication by a
// power of two is exact unless its result is subnormal, so scaling up is
// exact and scaling down rounds only results that are subnormal anyway.
__host__ __device__ __forceinline__ float scale_pow2(float x, int e) {
  if (e >= -126 && e <= 127) return x * pow2f(e);
  e = e < -252 ? -252 : (e > 252 ? 252 : e);
  const int e1 = e / 2;
  return (x * pow2f(e1)) * pow2f(e - e1);
}

// Tile `local` of a tiles_m x tiles_n GEMM: raster groups of kTcRaster tile
// rows walked column by column, so consecutive tiles share operand rows in L2.
__host__ __device__ __forceinline__ void tc_raster(int local, int tiles_m, int tiles_n,
                                                   int block_n, int& m0, int& n0) {
  const int per_group = kTcRaster * tiles_n;
  const int first_m = (local / per_group) * kTcRaster;
  const int group_rows = tiles_m - first_m < kTcRaster ? tiles_m - first_m : kTcRaster;
  m0 = (first_m + (local % per_group) % group_rows) * kTcBM;
  n0 = ((local % per_group) / group_rows) * block_n;
}

// WIDE: stages of 128-byte rows (128-byte swizzle; 64 16-bit elements deep,
// the TF32 form's 32 tf32 elements) instead of 64-byte ones.
template <int NP, int BN, bool WIDE = false>
struct TcShape {
  static constexpr int KB = WIDE ? 2 * kTcKB : kTcKB;  // k depth of a stage
  static constexpr int A_PLANE = kTcBM * KB * 2;  // bytes of one A piece tile
  static constexpr int B_PLANE = BN * KB * 2;
  static constexpr int A_BYTES = NP * A_PLANE;
  static constexpr int B_BYTES = NP * B_PLANE;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int FIT = (224 * 1024) / STAGE_BYTES;
  static constexpr int STAGES = FIT > 4 ? 4 : FIT;
  // 128-wide tiles stage each epilogue warp's 32 x 32 output block in shared
  // memory (padded rows) so C is written row by row, coalesced; 256-wide
  // tiles have no room left and store straight from registers.
  static constexpr bool STAGE_C = (BN == 128);
  static constexpr size_t STAGE_C_BYTES = STAGE_C ? size_t(kTcEpiWarps) * 32 * 33 * 4 : 0;
  // 256-wide tiles of grouped launches stage 8 rows x 32 columns per warp
  // at a time: what the stage ring leaves of shared memory
  static constexpr bool STAGE_C8 = (BN == 256);
  static constexpr size_t STAGE_C8_BYTES = STAGE_C8 ? size_t(kTcEpiWarps) * 8 * 33 * 4 : 0;
  static constexpr size_t SMEM =
      1024 + size_t(STAGES) * STAGE_BYTES + 256 + STAGE_C_BYTES + STAGE_C8_BYTES;
  // fused launches: kTcFusedPieceStages piece stages, then kTcRawStages raw
  // FP32 stages (the a tile, then the b tile, RAW_K deep)
  static constexpr int RAW_K = fused_raw_k(BN);
  static constexpr int RAW_A = kTcBM * RAW_K * 4;
  static constexpr int RAW_BYTES = RAW_A + BN * RAW_K * 4;
  static constexpr size_t FUSED_RING =
      size_t(kTcFusedPieceStages) * STAGE_BYTES + size_t(kTcRawStages) * RAW_BYTES;
  static constexpr size_t SMEM_FUSED = 1024 + FUSED_RING + 256 + STAGE_C_BYTES + STAGE_C8_BYTES;
  // main + correction accumulators, double-buffered across tiles when they fit
  static constexpr int ACC_BUFS = (4 * BN <= 512) ? 2 : 1;
  static constexpr uint32_t TMEM_COLS = ACC_BUFS * 2 * BN;
  static_assert(STAGES >= 2, "pipeline needs two stages");
  static_assert(SMEM <= 232448, "shared memory budget");
};

// One GEMM as the persistent kernel sees it (device-resident for groups).
// M and N are the kernel's rows (operand "a" of the maps) and columns
// (operand "b").  Grouped plans may also set
//   kb0  > 0: the problem is one k slice [kb0, kb0 + nkb) of a split-K GEMM;
//   swap = 1: the kernel computes C^T = op(B)^T op(A)^T, so kernel row r and
//             column c are C's element (c, r), stored at C[c * ldc + r], and
//             a bias is indexed by the kernel column.
struct TcProblem {
  float* C;
  int M, N, ldc;
  float alpha, beta;
  int nkb;              // stages of the kernel's k depth (split_stage_k)
  int tiles_m, tiles_n;
  int tile_start;       // first global tile index of this problem
  int kb0 = 0;
  int swap = 0;
  int map = 0;          // tensor maps of this problem: maps[2 * map], maps[2 * map + 1]
  Epilogue epi;
  // FP16x3 form: the largest magnitude of every kernel row (fmax_a[r], a row
  // of the kernel's a operand) and column (fmax_b[c], a row of its b
  // operand), from which f16_scale_exp gives the scales the epilogue undoes.
  // Null otherwise.
  const unsigned* fmax_a = nullptr;
  const unsigned* fmax_b = nullptr;
  // fused launches: whether the raw tile of the kernel's a (b) operand has k
  // contiguous (the map's box is {32 k, rows}, 128-byte swizzle) or rows
  // contiguous (box {rows, 32 k}, no swizzle); maps[2 * map] and
  // maps[2 * map + 1] then describe the FP32 sources
  int kc_a = 1, kc_b = 1;
  // fused 256-wide launches (set in the `single` record only): the chunk
  // sums of the epilogue warps, kTcFusedSumBytes per persistent CTA
  float* chunk_sums = nullptr;
};

// One operand to split in the batched pre-pass.
struct SplitJob {
  const float* src;
  long long sr, sk;     // element (r, k) at src[r*sr + k*sk]
  __nv_bfloat16* dst;   // [planes][rows][Kp] pieces (32-bit ones for TF32 jobs)
  int rows, K, Kp;
  int tile_start;       // first 32x64 tile index of this job
  // implicit im2col operand (src unused): 1 = rows are pixels and k taps,
  // 2 = rows are taps and k pixels; 0 = plain strided matrix
  int gather = 0;
  Im2col im;
  // FP16x3 form: `rows` words that receive the largest magnitude of each row
  // (operand_max_batched_kernel), from which each row's power-of-two scale
  // follows; null: bf16 pieces.
  unsigned* fmax = nullptr;
};

int split_kp(int K);
int split_default_chunk_kb(int K);
// Bytes of one operand's pieces [pieces][rows][Kp]; two-piece operands also
// carry a trailer of one word per row (rounded up to 256 bytes) that holds
// the row's largest magnitude (split_fmax_word), used by the FP16x3 form.
size_t split_operand_bytes(int pieces, int rows, int K);
unsigned* split_fmax_word(const void* pieces_base, int pieces, int rows, int K);
void split_operand_strides(const Gemm& g, long long* a_sr, long long* a_sk, long long* b_sr,
                           long long* b_sk);
// Piece layouts, by the code that SplitPlan::pieces and the functions below
// take: 3 = three 16-bit pieces (BF16x6/x9), 2 = two 16-bit pieces (BF16x3,
// FP16x3), kPiecesTf32 = two 32-bit TF32 pieces (TF32x3).
constexpr int kPiecesTf32 = 4;
constexpr int piece_planes(int code) { return code == kPiecesTf32 ? 2 : code; }
constexpr int piece_bytes(int code) { return code == kPiecesTf32 ? 4 : 2; }
// The GEMM kernel instantiation a layout runs on: TF32 stages have the
// shape of the two-piece 16-bit ones (two planes of 128-byte rows).
constexpr int kernel_np(int code) { return code == kPiecesTf32 ? 2 : code; }
// k depth of one pipeline stage: 32 elements in every layout -- 64-byte
// rows with the 64-byte swizzle for 16-bit pieces, 128-byte rows with the
// 128-byte swizzle for TF32 pieces.  The tensor maps' boxes and every
// launch's TcProblem::nkb follow it.  (Two-piece 16-bit operands once took
// 64-deep stages of 128-byte rows, two 96 KB stages at 256-wide tiles, to
// halve a per-stage cost of the MMA issuer; with that cost gone, 32-deep
// stages in a four-stage ring are faster: FP16x3 GEMM at 8192^3 1.93 ->
// 1.88 ms.)
constexpr int split_stage_k(int /*code*/) { return kTcKB; }
// Whether a kernel instantiation has the 128-byte-row shape (TcShape WIDE):
// the TF32 form's stages, on the two-piece instantiation.
constexpr bool tc_wide(int np, bool tf32) { return np == 2 && tf32; }
// Stages of the kernel's depth over K, and a chunk of `chunk_kb` 32-deep
// k-blocks in stages.
inline int split_nkb(int pieces, int K) {
  return (split_kp(K) + split_stage_k(pieces) - 1) / split_stage_k(pieces);
}
inline int split_chunk_stages(int pieces, int chunk_kb) {
  const int c = chunk_kb / (split_stage_k(pieces) / kTcKB);
  return c > 0 ? c : 1;
}
bool split_encode_maps(int pieces, int block_n, const void* ap, int M, const void* bp, int N,
                       int K, CUtensorMap* ta, CUtensorMap* tb);
TcProblem split_problem(const Gemm& g, int pieces, int block_n, int tile_start);
// Map of rows [0, rows) of a piece array whose planes are plane_rows long
// (a view starting inside the array: base points at its first row).
bool split_encode_view(int pieces, int box_rows, const void* base, int rows, int plane_rows, int K,
                       CUtensorMap* map);

// Wave tail of one split GEMM (multi.cu): when the tiles' last wave would
// occupy less than half of the SMs, its tiles -- whole tile columns of the
// last raster group, a rectangle [r0, M) x [c0, N) of C -- run as two k
// slices in one grouped launch plus a reduce, after the other tiles.
struct TailPlan {
  bool use = false;
  int main_tiles = 0;  // tiles the single-GEMM kernel runs (raster order prefix)
  int r0 = 0, c0 = 0;  // first row and column of the tail rectangle
};
TailPlan tail_plan(const Gemm& g, const SplitPlan& p);
size_t tail_scratch_bytes(const Gemm& g, const SplitPlan& p);
ugemm_status tail_launch(const Gemm& g, const SplitPlan& p, const TailPlan& tail,
                         const void* a_pieces, const void* b_pieces, void* scratch, int* dev_err,
                         cudaStream_t st);
// probs/tiles: a grouped launch's problem records and its tile table (from
// split_tile_table, for a grid of exactly max_ctas CTAs); both null for one
// GEMM (`single`).
// p.fused (grouped only): `maps` describe the FP32 operands, not pieces.
ugemm_status split_gemm_launch(const SplitPlan& p, const CUtensorMap& ta, const CUtensorMap& tb,
                               const TcProblem& single, const CUtensorMap* maps,
                               const TcProblem* probs, const int4* tiles, int total_tiles,
                               int chunk_kb, int max_ctas, int* dev_err, cudaStream_t st);
// The TMA map of a fused launch's FP32 operand stored as R rows x Cc columns
// (leading dimension ld elements): kcontig, the kernel reads k along the
// columns (box {box_k, box_rows}; 128-byte swizzle for 32-deep boxes, 64-byte
// for 16-deep ones); else rows along them (box {box_rows, box_k}).  False if
// TMA cannot describe it (alignment).
bool fused_encode_map(const float* base, long long ld, int R, int Cc, bool kcontig, int box_rows,
                      int box_k, CUtensorMap* map);
// Tile table of a grouped launch of `grid` persistent CTAs: grid ranges
// {first, end, 0, 0} into the records that follow, one {problem, m0, n0, 0}
// per tile (raster order within a problem), dealt longest first to the
// least-loaded CTA (round_robin: in problem order, tile i to CTA i % grid).
std::vector<int4> split_tile_table(const TcProblem* probs, int nprob, int block_n, int grid,
                                   bool round_robin = false);
// The batched pre-pass of a grouped plan.  fmax_words (FP16x3 plans): the
// jobs' `fmax` row words, nwords of them contiguous, cleared and filled
// before the split.
// A few split jobs passed by value (split_param_launch): tile_start of each
// job is its first 32 x 64 tile in the launch.  bf16 and TF32 pieces only
// (the FP16x3 form's row maxima take their own passes).
constexpr int kSplitTableJobs = 8;
struct SplitJobTable {
  SplitJob jobs[kSplitTableJobs];
};
static_assert(sizeof(SplitJobTable) <= 4000, "split job table must fit the kernel parameter space");
ugemm_status split_param_launch(int pieces, const SplitJobTable& t, int njobs, int total_tiles,
                                cudaStream_t st);
ugemm_status split_batched_launch(int pieces, const SplitJob* jobs, int njobs, int total_tiles,
                                  cudaStream_t st, unsigned* fmax_words = nullptr, int nwords = 0);
// Split one operand into its pieces at dst (split_operand_bytes of room).
// f16: FP16x3 pieces -- the largest magnitude of every row is first found
// into the operand's trailer words (cleared here), then each row's pieces
// are scaled by its own.
ugemm_status split_operand_launch(int pieces, const float* src, long long sr, long long sk,
                                  int rows, int K, void* dst, cudaStream_t st, bool f16 = false);
// GEMM on operands already split; with tail_scratch (tail_scratch_bytes of
// it), a short last wave of tiles runs as the wave-tail launch.
ugemm_status split_gemm_on_pieces(const Gemm& g, const SplitPlan& p, const void* a_pieces,
                                  const void* b_pieces, void* tail_scratch, int* dev_err,
                                  cudaStream_t st);

}  // namespace ugemm
