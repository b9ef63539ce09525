// simt.cuh -- types shared by the FP32 SIMT kernels (simt.cu) and the
// grouped GEMM planner (grouped.cu).
#pragma once

#include <cuda.h>

#include "internal.h"

namespace ugemm {

constexpr int kBK = 32;            // k depth of one pipeline stage (128-byte k rows)
constexpr int kStages = 4;         // TMA ring depth
constexpr int kConsumerWarps = 8;  // 16 x 16 compute threads
constexpr int kThreads = (kConsumerWarps + 1) * 32;
constexpr int kRaster = 8;         // rows of tiles per raster group (L2 reuse)

template <int TM, int TN>
struct SimtShape {
  static constexpr int BM = 16 * TM;
  static constexpr int BN = 16 * TN;
  static constexpr int A_BYTES = BM * kBK * 4;
  static constexpr int B_BYTES = BN * kBK * 4;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr size_t SMEM = 1024 + size_t(kStages) * STAGE_BYTES + 2 * kStages * 8;
};

// One problem of the grouped SIMT kernel (device-resident table).
struct SimtProblem {
  float* C;
  int M, N, ldc;
  float alpha, beta;
  int nkt;              // k tiles of kBK
  int tiles_m, tiles_n;
  int tile_start;
  Epilogue epi;
  int kt0 = 0;          // first k tile (a split-K slice of a grouped plan)
};

// One operand of the batched FP32 pack: op(X) (rows x K) -> dst[k][r] with
// row length ld (rows contiguous, the layout the SIMT kernel reads fastest).
struct PackJob {
  const float* src;
  long long sr, sk;
  float* dst;
  int rows, K, ld;
  int tile_start;       // first 32 x 64 tile of this job
  // implicit im2col operand (src unused): 1 = rows are pixels and k taps,
  // 2 = rows are taps and k pixels; 0 = plain strided matrix
  int gather = 0;
  Im2col im;
};

ugemm_status simt_grouped_launch(int tile, const CUtensorMap* maps, const SimtProblem* probs,
                                 int nprob, int total_tiles, int max_ctas, int* dev_err,
                                 cudaStream_t st);
ugemm_status pack_batched_launch(const PackJob* jobs, int njobs, int total_tiles, cudaStream_t st);
bool simt_encode_grouped(int tile, const float* a, int M, const float* b, int N, int K, int ld_a,
                         int ld_b, CUtensorMap* ta, CUtensorMap* tb);
int simt_block(int tile);

}  // namespace ugemm
