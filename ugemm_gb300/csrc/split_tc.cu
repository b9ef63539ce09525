// split_tc.cu -- split-precision SGEMM on the 5th-generation tensor cores
// (the "precision" form; no counterpart in the reference, whose only GPU
// kernels are the FP32 OpenCL/GLSL ones).
//
// Each FP32 operand element x is written as a sum of bf16 pieces
//     x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1)
// (exact for three pieces: 8+8+8 significand bits cover FP32's 24).  The
// product A*B is the sum of piece products A_i*B_j, each a tcgen05.mma
// (kind::f16, bf16 x bf16 -> FP32 in TMEM):
//     BF16x9: all nine products;  BF16x6: drop a1b2, a2b1, a2b2 (~2^-24 each);
//     BF16x3: two pieces, a0b0 + a0b1 + a1b0 (~2^-16; for error studies).
//
// Accuracy.  The tensor core adds each MMA's result into the FP32
// accumulator with truncation (measured: the error grows linearly in K and
// is biased toward zero), so one long TMEM accumulation is ~30x less accurate
// than an FP32 FMA loop at K = 8192.  This kernel therefore keeps
//   * the main product a0*b0 in its own TMEM accumulator, restarted every
//     `chunk_kb` k-blocks: the epilogue warps drain each chunk into FP32
//     registers (round-to-nearest adds), so truncation only ever acts on a
//     short partial sum;
//   * all correction products (~2^-8 of the main term) in a second TMEM
//     accumulator over the whole K, issued before the main product of each
//     k-block so a chunk drain overlaps the correction MMAs.
// Result: normwise error below the plain FP32 SIMT kernel's at every K.
//
// Pipeline (persistent: one CTA per SM walks a static list of output tiles,
// which serves one GEMM or a group of independent GEMMs):
//   1. split kernel: reads op(A)/op(B) in any transpose and leading
//      dimension, writes the pieces as K-major bf16 planes [pieces][rows][Kp]
//      (Kp = K rounded up to 32, zero padded);
//   2. GEMM kernel, 10 warps:
//        warp 0   TMA producer: one 3-D TMA per operand per stage brings all
//                 pieces of a 32-deep k slice (64-byte swizzle; TF32
//                 pieces: 128-byte rows and swizzle) into a 3-4 stage ring
//                 (mbarrier full/empty pairs);
//        warp 1   allocates TMEM (2 x BN columns: main + corrections) and,
//                 from one thread, issues the tcgen05.mma stream;
//        warps 2-9  epilogue: chunk drains, then alpha/beta and the store of
//                 the 128 x BN tile (one TMEM lane per row; two warps per
//                 lane quarter, each owning half of the columns).
// All mbarrier waits are bounded (ptx.cuh); on a timeout the kernel records
// an error, abandons its remaining work and still frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cfloat>

#include <algorithm>
#include <cstdlib>
#include <functional>
#include <queue>
#include <utility>
#include <vector>

#include "internal.h"
#include "ptx.cuh"
#include "split_tc.cuh"

namespace ugemm {
namespace {

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

__device__ __forceinline__ void fence_tensormap(const CUtensorMap* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                   reinterpret_cast<uint64_t>(map))
               : "memory");
}

struct TileCoord { int p, m0, n0; };

// Tiles of this CTA: a grouped launch walks its own slice of the planned tile
// list (tiles[blockIdx.x] = {first, end}; the records follow the grid's
// ranges), one GEMM strides through its tiles by the grid size.
struct TileRange { int first, end, step; };

template <bool GROUPED>
__device__ __forceinline__ TileRange tile_range(const int4* tiles, int total_tiles) {
  if constexpr (GROUPED) {
    const int4 r = tiles[blockIdx.x];
    return TileRange{r.x, r.y, 1};
  } else {
    return TileRange{static_cast<int>(blockIdx.x), total_tiles, static_cast<int>(gridDim.x)};
  }
}

// Tile t of one GEMM in raster order (tc_raster).  Grouped launches read the
// same coordinates from their tile table, one 16-byte record {problem, m0,
// n0} per tile, built when the launch is planned: a persistent CTA then pays
// two dependent loads per tile instead of a binary search through the
// problem records (each step an L2 round trip).
template <int BN, bool GROUPED>
__device__ __forceinline__ TileCoord tile_coord(const TcProblem& single, const TcProblem* probs,
                                                const int4* tiles, int t, TcProblem& P) {
  TileCoord tc;
  if constexpr (GROUPED) {
    const int4 r = tiles[gridDim.x + t];
    tc.p = r.x;
    tc.m0 = r.y;
    tc.n0 = r.z;
    P = probs[r.x];
  } else {
    tc.p = 0;
    P = single;
    tc_raster(t - P.tile_start, P.tiles_m, P.tiles_n, BN, tc.m0, tc.n0);
  }
  return tc;
}

// The end of a tile's epilogue once acc holds its sums (this warp's HALF
// columns of its lane quarter's 32 rows): the FP16x3 scales, alpha/beta (C is
// read only when beta != 0), the bias / activation (EPI instantiations only)
// and the stores.  stage_base: the shared-memory staging area after the ring.
template <int NP, int BN, bool GROUPED, bool EPI>
__device__ __forceinline__ void epi_store(const TcProblem& P, const TileCoord& tc,
                                          float (&acc)[BN / 2], int warp, int lane,
                                          float* stage_base) {
  using S = TcShape<NP, BN, false>;  // only its BN-dependent staging is read here
  constexpr int HALF = BN / 2;
  const int ew = warp - 2;
  const int q = warp & 3;
  const int col_off = (ew >> 2) * HALF;
  const int n_live = GROUPED ? P.N - tc.n0 - col_off : HALF;
  (void)n_live;
  if constexpr (NP == 2) {  // FP16x3: undo the rows' and columns' power-of-two scales
    if (P.fmax_a != nullptr) {
      // this lane's row; lane l fetches the scales of columns l, l + 32, ...
      // of the warp's half and hands them to the other lanes by shuffle
      const int row = tc.m0 + q * 32 + lane;
      const int ea = row < P.M ? f16_scale_exp(P.fmax_a[row]) : 0;
      int eb[HALF / 32];
#pragma unroll
      for (int c32 = 0; c32 < HALF / 32; ++c32) {
        const int col = tc.n0 + col_off + c32 * 32 + lane;
        eb[c32] = col < P.N ? f16_scale_exp(P.fmax_b[col]) : 0;
      }
#pragma unroll
      for (int j = 0; j < HALF; ++j)
        acc[j] = scale_pow2(acc[j], -(ea + __shfl_sync(0xffffffffu, eb[j / 32], j % 32)));
    }
  }
  // alpha/beta epilogue (C not read when beta == 0).  The bias /
  // activation exists only in the EPI instantiation, so the plain kernel's
  // epilogue carries no code for it.
  const bool has_epi = EPI && (P.epi.bias != nullptr || P.epi.act != 0);
  if (GROUPED && P.swap) {
    // transposed problem: this lane's kernel row is a C column, so for a
    // fixed register the warp writes 32 consecutive floats of one C row
    const int r = tc.m0 + q * 32 + lane;
    if (r < P.M) {
#pragma unroll
      for (int j = 0; j < HALF; ++j) {
        const int c = tc.n0 + col_off + j;
        if (c < P.N) {
          float* cp = P.C + static_cast<size_t>(c) * P.ldc + r;
          float v = P.alpha * acc[j];
          if (P.beta != 0.f) v += P.beta * *cp;
          if (has_epi) v = epilogue_apply(v, P.epi, c);
          *cp = v;
        }
      }
    }
    return;
  }
  if constexpr (GROUPED && S::STAGE_C8) {
    // 256-wide tiles: each 32 x 32 block goes through shared memory 8
    // rows at a time (lanes 8p..8p+7 hold rows 8p..8p+7), so every store
    // instruction still writes one 128-byte row segment
    float* stage = stage_base + ew * 8 * 33;
    const int col = tc.n0 + col_off + lane;
#pragma unroll
    for (int c32 = 0; c32 < HALF / 32; ++c32) {
      if (c32 * 32 >= n_live) break;
      const int cc = col + c32 * 32;
#pragma unroll
      for (int pass = 0; pass < 4; ++pass) {
        if ((lane >> 3) == pass) {
#pragma unroll
          for (int j = 0; j < 32; ++j) stage[(lane & 7) * 33 + j] = acc[c32 * 32 + j];
        }
        __syncwarp();
        if (cc < P.N) {
          for (int rr = 0; rr < 8; ++rr) {
            const int row = tc.m0 + q * 32 + pass * 8 + rr;
            if (row >= P.M) break;
            float* cp = P.C + static_cast<size_t>(row) * P.ldc + cc;
            float v = P.alpha * stage[rr * 33 + lane];
            if (P.beta != 0.f) v += P.beta * *cp;
            if (has_epi) v = epilogue_apply(v, P.epi, row);
            *cp = v;
          }
        }
        __syncwarp();
      }
    }
    return;
  }
  if constexpr (S::STAGE_C) {
    // transpose each 32 x 32 block through shared memory: lane = column,
    // one 128-byte row segment per store instruction
    float* stage = stage_base + ew * 32 * 33;
    const int col = tc.n0 + col_off + lane;
#pragma unroll
    for (int c32 = 0; c32 < HALF / 32; ++c32) {
#pragma unroll
      for (int j = 0; j < 32; ++j) stage[lane * 33 + j] = acc[c32 * 32 + j];
      __syncwarp();
      const int cc = col + c32 * 32;
      if (cc < P.N) {
        if (has_epi) {
          for (int rr = 0; rr < 32; ++rr) {
            const int row = tc.m0 + q * 32 + rr;
            if (row >= P.M) break;
            float* cp = P.C + static_cast<size_t>(row) * P.ldc + cc;
            float v = P.alpha * stage[rr * 33 + lane];
            if (P.beta != 0.f) v += P.beta * *cp;
            *cp = epilogue_apply(v, P.epi, row);
          }
        } else {
          for (int rr = 0; rr < 32; ++rr) {
            const int row = tc.m0 + q * 32 + rr;
            if (row >= P.M) break;
            float* cp = P.C + static_cast<size_t>(row) * P.ldc + cc;
            float v = P.alpha * stage[rr * 33 + lane];
            if (P.beta != 0.f) v += P.beta * *cp;
            *cp = v;
          }
        }
      }
      __syncwarp();
    }
    return;
  }
  const int row = tc.m0 + q * 32 + lane;
  if (row < P.M) {
    float* crow = P.C + static_cast<size_t>(row) * P.ldc;
    const int col0 = tc.n0 + col_off;
    const bool vec = ((P.ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(P.C) & 15) == 0);
    if (has_epi) {
#pragma unroll
      for (int j = 0; j < HALF; ++j)
        if (col0 + j < P.N) {
          float v = P.alpha * acc[j];
          if (P.beta != 0.f) v += P.beta * crow[col0 + j];
          crow[col0 + j] = epilogue_apply(v, P.epi, row);
        }
    } else if (vec && col0 + HALF <= P.N) {
#pragma unroll
      for (int j = 0; j < HALF; j += 4) {
        float4 v = make_float4(P.alpha * acc[j], P.alpha * acc[j + 1], P.alpha * acc[j + 2],
                               P.alpha * acc[j + 3]);
        if (P.beta != 0.f) {
          const float4 o = *reinterpret_cast<const float4*>(crow + col0 + j);
          v.x += P.beta * o.x; v.y += P.beta * o.y; v.z += P.beta * o.z; v.w += P.beta * o.w;
        }
        *reinterpret_cast<float4*>(crow + col0 + j) = v;
      }
    } else {
#pragma unroll
      for (int j = 0; j < HALF; ++j)
        if (col0 + j < P.N) {
          float v = P.alpha * acc[j];
          if (P.beta != 0.f) v += P.beta * crow[col0 + j];
          crow[col0 + j] = v;
        }
    }
  }
}

// Adds the accumulator columns this warp owns (TMEM address t: its lane
// quarter, first column) to acc, 32 columns at a time; grouped launches skip
// the slices past the tile's n_live result columns.
template <int HALF, bool GROUPED>
__device__ __forceinline__ void acc_add_tmem(uint32_t t, float (&acc)[HALF], int n_live) {
#pragma unroll
  for (int c32 = 0; c32 < HALF / 32; ++c32) {
    if (GROUPED && c32 * 32 >= n_live) break;
    uint32_t r[32];
    tmem_ld_32x32b_x32(t + c32 * 32, r);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[c32 * 32 + j] += __uint_as_float(r[j]);
  }
}

// The converter warps of a fused launch (defined with the split helpers).
template <int NP, int BN>
__device__ void fused_convert(const TcProblem* __restrict__ probs, const int4* __restrict__ tiles,
                              uint8_t* pieces, uint8_t* raw, uint64_t* full, uint64_t* empty,
                              uint64_t* raw_full, uint64_t* raw_empty, int ct, int* err);
// The epilogue warps of a 256-wide fused launch, which also convert.
template <int NP, int BN, bool EPI>
__device__ void fused_dual(const TcProblem* __restrict__ probs, const int4* __restrict__ tiles,
                           float* chunk_sums, uint8_t* smem, uint32_t tmem, uint64_t* full,
                           uint64_t* empty, uint64_t* raw_full, uint64_t* raw_empty,
                           uint64_t* main_full, uint64_t* main_empty, uint64_t* tile_full,
                           uint64_t* tmem_empty, uint64_t* stage_free, int chunk_kb, int warp,
                           int lane, int* err);

// Correction products in issue order, (a piece << 2) | b piece; the main
// product a0*b0 is issued after them.
__host__ __device__ constexpr uint32_t corr_code(int p) {
  return p == 0 ? 0x1 : p == 1 ? 0x4 : p == 2 ? 0x2 : p == 3 ? 0x5 : p == 4 ? 0x8
       : p == 5 ? 0x6 : p == 6 ? 0x9 : 0xA;
}

// The MMA issuer (one thread).  Per k-block: wait for the stage, issue the
// correction products into their accumulator, the main product into its
// (restarted at each chunk once the epilogue drained it), commit the stage
// free; per tile, commit the accumulators full.  Everything per k-block is
// compile-time but the stage: the descriptors are those of stage 0 plus the
// stage's offset (the address field counts 16-byte units, and shared
// memory stays below 256 KB, so the field never carries), the product
// count is a template parameter, and the chunk position is a counter
// rather than a remainder (a run-time division cost ~400 cycles per
// k-block in the issuing thread, a gap in which the tensor pipe drained).
template <int NP, int BN, bool GROUPED, bool TF32, bool FUSED, int NPROD>
__device__ __forceinline__ void mma_issue_loop(const TcProblem& single,
                                               const TcProblem* __restrict__ probs,
                                               const int4* __restrict__ tiles, int total_tiles,
                                               uint8_t* smem, uint32_t tmem, uint64_t* full,
                                               uint64_t* empty, uint64_t* main_full,
                                               uint64_t* main_empty, uint64_t* tile_full,
                                               uint64_t* tmem_empty, int chunk_kb, int fmt,
                                               int* err) {
  constexpr bool WIDE = tc_wide(NP, TF32);
  using S = TcShape<NP, BN, WIDE>;
  constexpr int KK = S::KB / 16;  // k steps of 32 bytes per row in a stage
  constexpr uint32_t SBO = WIDE ? 1024 : 512, SWZ = WIDE ? 2 : 4;
  constexpr int NST = FUSED ? kTcFusedPieceStages : S::STAGES;
  constexpr int NB = S::ACC_BUFS;
  // instruction descriptor operand format: bf16 pieces (1), the FP16x3
  // form's fp16 pieces (0) or the TF32x3 form's tf32 pieces (2); one k step
  // is 32 bytes of a row in each: 16 16-bit or 8 tf32 elements
  const uint32_t ifmt = TF32 ? 2u : (NP == 2 && fmt == 1 ? 0u : 1u);
  const uint32_t idesc_full = umma_idesc(ifmt, ifmt, kTcBM, BN);
  // 128-wide tiles whose first correction is A0 B1: the pair A0 [B0; B1]
  constexpr bool MERGE = !TF32 && BN == 128 && NPROD >= 3 && corr_code(0) == 0x1;
  const uint32_t idesc_pair = umma_idesc(ifmt, ifmt, kTcBM, 2 * BN);
  const uint32_t base = smem_u32(smem);
  const uint64_t da0 = umma_smem_desc(base, SBO, SWZ);
  const uint64_t db0 = umma_smem_desc(base + S::A_BYTES, SBO, SWZ);
  uint32_t s = 0, ph = 0, ntile = 0;
  uint32_t nbound[NB] = {};
  const TileRange tr = tile_range<GROUPED>(tiles, total_tiles);
  for (int t = tr.first; t < tr.end; t += tr.step, ++ntile) {
    TcProblem P;
    const TileCoord tc = tile_coord<BN, GROUPED>(single, probs, tiles, t, P);
    // a group's narrow problems and right-edge tiles multiply only the
    // columns that exist (UMMA N in steps of 16)
    uint32_t idesc = idesc_full;
    if constexpr (GROUPED) {
      const int n_rem = P.N - tc.n0;
      if (n_rem < BN)
        idesc = umma_idesc(ifmt, ifmt, kTcBM, static_cast<uint32_t>((n_rem + 15) & ~15));
    }
    const uint32_t buf = NB == 1 ? 0u : ntile % NB, use = ntile / NB;
    const uint32_t t_main = tmem + buf * 2 * BN, t_corr = t_main + BN;
    // the epilogue must have read this buffer's previous tile
    if (use > 0 && !mbar_wait(&tmem_empty[buf], (use - 1) & 1, err, kDevTimeoutAccum)) return;
    tc_fence_after();
    // the descriptors of stage st; the MMAs of its corrections and main product
    auto corrections = [&](uint32_t st, int kbi) {
      const uint64_t so = (st * static_cast<uint32_t>(S::STAGE_BYTES)) >> 4;
      const uint64_t da = da0 + so, db = db0 + so;
#pragma unroll
      for (int p = 0; p < NPROD - 1; ++p) {
        const uint32_t ia = corr_code(p) >> 2, ib = corr_code(p) & 3;
#pragma unroll
        for (int kk = 0; kk < KK; ++kk) {
          const uint64_t a = da + ((ia * S::A_PLANE + kk * 32) >> 4);
          const uint64_t b = db + ((ib * S::B_PLANE + kk * 32) >> 4);
          if constexpr (TF32) umma_tf32(t_corr, a, b, idesc, (kbi | p | kk) != 0);
          else umma_bf16(t_corr, a, b, idesc, (kbi | p | kk) != 0);
        }
      }
    };
    // A full-width 128-wide tile's main product and first correction, A0 B0
    // into the main accumulator and A0 B1 into the correction accumulator
    // right after it in tensor memory, as one 128 x 256 MMA per k step: the
    // B0 and B1 planes are adjacent in the stage (rows 0-127 and 128-255 of
    // one 256-row operand), so A0 is read once for both.  Only where both
    // accumulate (not at a chunk start, not in a tile's first k-block).
    auto merged_first = [&](uint32_t st) {
      const uint64_t so = (st * static_cast<uint32_t>(S::STAGE_BYTES)) >> 4;
      const uint64_t da = da0 + so, db = db0 + so;
#pragma unroll
      for (int kk = 0; kk < KK; ++kk)
        umma_bf16(t_main, da + ((kk * 32) >> 4), db + ((kk * 32) >> 4), idesc_pair, true);
#pragma unroll
      for (int p = 1; p < NPROD - 1; ++p) {
        const uint32_t ia = corr_code(p) >> 2, ib = corr_code(p) & 3;
#pragma unroll
        for (int kk = 0; kk < KK; ++kk)
          umma_bf16(t_corr, da + ((ia * S::A_PLANE + kk * 32) >> 4),
                    db + ((ib * S::B_PLANE + kk * 32) >> 4), idesc, true);
      }
    };
    auto main_product = [&](uint32_t st, bool restart) {
      const uint64_t so = (st * static_cast<uint32_t>(S::STAGE_BYTES)) >> 4;
      const uint64_t da = da0 + so, db = db0 + so;
#pragma unroll
      for (int kk = 0; kk < KK; ++kk) {
        const uint64_t a = da + ((kk * 32) >> 4), b = db + ((kk * 32) >> 4);
        if constexpr (TF32) umma_tf32(t_main, a, b, idesc, !(restart && kk == 0));
        else umma_bf16(t_main, a, b, idesc, !(restart && kk == 0));
      }
    };
    int cpos = 0;  // the k-block's position in its chunk
    const bool pair_ok = MERGE && idesc == idesc_full;
    for (int kb = 0; kb < P.nkb;) {
      if (!mbar_wait(&full[s], ph, err, kDevTimeoutFull)) return;
      tc_fence_after();
      if (pair_ok && cpos != 0) {
        merged_first(s);
        umma_commit(&empty[s]);
        ++kb;
        if (++cpos == chunk_kb) {
          cpos = 0;
          if (kb < P.nkb) umma_commit(&main_full[buf]);
        }
        if (++s == NST) {
          s = 0;
          ph ^= 1;
        }
        continue;
      }
      corrections(s, kb);
      // A new chunk restarts the main accumulator once the epilogue has
      // drained the last one.  While that drain runs, the corrections of the
      // next stages already in shared memory (the rest of the ring, within
      // this chunk) go ahead, so the tensor pipe does not wait; each
      // accumulator still receives its products in stage order (the same
      // bits).  Without this, every chunk start cost ~850 cycles of idle
      // tensor pipe in the three-product form.
      int ahead = 0;
      if (cpos == 0 && kb > 0) {
        uint32_t s2 = s + 1 == NST ? 0 : s + 1, ph2 = s + 1 == NST ? ph ^ 1 : ph;
        while (ahead < NST - 1 && ahead + 1 < chunk_kb && kb + 1 + ahead < P.nkb &&
               !mbar_test_wait(&main_empty[buf], nbound[buf] & 1) && mbar_test_wait(&full[s2], ph2)) {
          tc_fence_after();
          corrections(s2, kb + 1 + ahead);
          ++ahead;
          if (++s2 == NST) {
            s2 = 0;
            ph2 ^= 1;
          }
        }
        if (!mbar_wait(&main_empty[buf], nbound[buf] & 1, err, kDevTimeoutAccum)) return;
        ++nbound[buf];
        tc_fence_after();
      }
      // the main products of this stage and of those whose corrections went
      // ahead, each stage released once its MMAs complete
      for (int a = 0; a <= ahead; ++a, ++kb) {
        main_product(s, cpos == 0);
        umma_commit(&empty[s]);
        if (++cpos == chunk_kb) {
          cpos = 0;
          if (kb + 1 < P.nkb) umma_commit(&main_full[buf]);
        }
        if (++s == NST) {
          s = 0;
          ph ^= 1;
        }
      }
    }
    umma_commit(&tile_full[buf]);
  }
}

// TF32: the TF32x3 form's instantiation (two planes of 32-deep tf32
// stages, tcgen05 kind::tf32), a template parameter so that the 16-bit
// instantiations' MMA issue loop carries no branch on the format.
// FUSED (grouped launches of three bf16 pieces): instead of TMA copies of
// pieces made by a pre-pass, TMA copies of the FP32 operand tiles land in a
// raw ring, and converter warps split them and store the pieces into a
// piece ring in the layout the piece copies would have had (K-major, 64-byte
// rows, 64-byte swizzle), so the MMA issuer and the epilogue run unchanged
// and the results are the same bits.
template <int NP, int BN, bool GROUPED, bool EPI, bool TF32 = false, bool FUSED = false>
__global__ void __launch_bounds__(FUSED ? fused_threads(BN) : kTcThreads, 1)
    split_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    const __grid_constant__ TcProblem single, const CUtensorMap* __restrict__ maps,
                    const TcProblem* __restrict__ probs, const int4* __restrict__ tiles,
                    int total_tiles, int nprod,
                    int chunk_kb, int fmt, int* err) {
  // fmt: 16-bit piece format, 0 bf16, 1 fp16 (FP16x3); TF32 instantiations
  // read two planes of 32-deep stages with the 128-byte rows of the
  // two-piece 16-bit shape
  static_assert(!TF32 || NP == 2, "TF32 pieces come in two planes");
  static_assert(!FUSED || (NP == 3 && GROUPED && !TF32), "fused: grouped bf16x3-piece launches");
  // 256-wide fused tiles: the epilogue warps are the converters
  constexpr bool DUAL = FUSED && BN == 256;
  constexpr bool WIDE = tc_wide(NP, TF32);
  using S = TcShape<NP, BN, WIDE>;
  constexpr int KB = S::KB;
  // K-major operand tiles: 8-row groups of 128-byte rows (128-byte swizzle)
  // or of 64-byte rows (64-byte swizzle); one k16 MMA step is 32 bytes
  constexpr uint32_t SBO = WIDE ? 1024 : 512, SWZ = WIDE ? 2 : 4;
  // stages of pieces the MMA issuer reads; a fused launch's raw stages follow
  constexpr int NST = FUSED ? kTcFusedPieceStages : S::STAGES;
  constexpr int RST = FUSED ? kTcRawStages : 0;
  constexpr size_t RING = FUSED ? S::FUSED_RING : size_t(S::STAGES) * S::STAGE_BYTES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + RING);
  uint64_t* empty = full + NST;
  uint64_t* raw_full = empty + NST;   // fused: a raw stage's copies landed
  uint64_t* raw_empty = raw_full + RST;  // fused: the converters read it
  // one set per TMEM accumulator buffer (two when 2 x 2 x BN columns fit)
  constexpr int NB = S::ACC_BUFS;
  uint64_t* main_full = raw_empty + RST;   // a main-product chunk is complete
  uint64_t* main_empty = main_full + NB;     // the epilogue drained it
  uint64_t* tile_full = main_empty + NB;     // all MMAs of a tile are complete
  uint64_t* tmem_empty = tile_full + NB;     // the epilogue read both accumulators
  uint64_t* stage_free = tmem_empty + NB;    // 256-wide fused: a tile's final epilogue is done
                                             // with the piece stage it parks sums in
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(stage_free + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      // a fused piece stage is written by the converter threads, each of
      // which arrives once its stores are visible to the tensor core
      mbar_init(&full[s], FUSED ? fused_conv_threads(BN) : 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < RST; ++s) {
      mbar_init(&raw_full[s], 1);
      mbar_init(&raw_empty[s], fused_conv_threads(BN));
    }
    for (int b = 0; b < NB; ++b) {
      mbar_init(&main_full[b], 1);
      mbar_init(&main_empty[b], kTcEpiWarps);
      mbar_init(&tile_full[b], 1);
      mbar_init(&tmem_empty[b], kTcEpiWarps);
    }
    mbar_init(stage_free, kTcEpiWarps);
    fence_barrier_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, S::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (FUSED && !DUAL && warp >= 2 + kTcEpiWarps) {
    // ------------------------------------------------- fused converters
    // threads of warps 12 and 13 first (see fused_convert)
    static_assert(kTcConvWarps == 6 && 2 + kTcEpiWarps == 10, "converter warps 10-15");
    if constexpr (FUSED && !DUAL)
      fused_convert<NP, BN>(probs, tiles, smem, smem + NST * S::STAGE_BYTES, full, empty,
                            raw_full, raw_empty, ((warp - 2 - kTcEpiWarps + 4) % 6) * 32 + lane,
                            err);
  } else if (FUSED && warp == 0) {
    // ------------------------------------------- fused raw TMA producer
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      const TileRange tr = tile_range<GROUPED>(tiles, total_tiles);
      uint8_t* raw = smem + NST * S::STAGE_BYTES;
      for (int t = tr.first; ok && t < tr.end; t += tr.step) {
        TcProblem P;
        const TileCoord tc = tile_coord<BN, GROUPED>(single, probs, tiles, t, P);
        const CUtensorMap* ma = &maps[2 * P.map];
        const CUtensorMap* mb = &maps[2 * P.map + 1];
        fence_tensormap(ma);
        fence_tensormap(mb);
        // each piece stage from kTcKB / RAW_K raw stages
        for (int kr = 0; ok && kr < P.nkb * (kTcKB / S::RAW_K); ++kr, ++it) {
          const int s = it % RST;
          const uint32_t ph = (it / RST) & 1;
          if (!mbar_wait(&raw_empty[s], ph ^ 1, err, kDevTimeoutEmpty)) { ok = false; break; }
          uint8_t* ra = raw + s * S::RAW_BYTES;
          const int k0 = P.kb0 * kTcKB + kr * S::RAW_K;
          mbar_arrive_expect_tx(&raw_full[s], S::RAW_BYTES);
          if (P.kc_a) tma_load_2d(ra, ma, &raw_full[s], k0, tc.m0);
          else tma_load_2d(ra, ma, &raw_full[s], tc.m0, k0);
          if (P.kc_b) tma_load_2d(ra + S::RAW_A, mb, &raw_full[s], k0, tc.n0);
          else tma_load_2d(ra + S::RAW_A, mb, &raw_full[s], tc.n0, k0);
        }
      }
      if (!ok) {  // let copies still in flight land before the CTA exits
        for (uint32_t j = (it > uint32_t(RST) ? it - RST : 0); j < it; ++j)
          mbar_wait(&raw_full[j % RST], (j / RST) & 1, nullptr, 0);
      }
    }
  } else if (warp == 0) {
    // ------------------------------------------------------ TMA producer
    if (lane == 0) {
      if (!GROUPED) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
      }
      uint32_t it = 0;
      bool ok = true;
      const TileRange tr = tile_range<GROUPED>(tiles, total_tiles);
      for (int t = tr.first; ok && t < tr.end; t += tr.step) {
        TcProblem P;
        const TileCoord tc = tile_coord<BN, GROUPED>(single, probs, tiles, t, P);
        const CUtensorMap* ma = GROUPED ? &maps[2 * P.map] : &tmA;
        const CUtensorMap* mb = GROUPED ? &maps[2 * P.map + 1] : &tmB;
        if (GROUPED) {
          fence_tensormap(ma);
          fence_tensormap(mb);
        }
        const int kb0 = GROUPED ? P.kb0 : 0;  // first k-block of a split-K slice
        constexpr int kx = TF32 ? KB / 2 : KB;  // elements of k per stage
        for (int kb = 0; kb < P.nkb; ++kb, ++it) {
          const int s = it % S::STAGES;
          const uint32_t ph = (it / S::STAGES) & 1;
          if (!mbar_wait(&empty[s], ph ^ 1, err, kDevTimeoutEmpty)) { ok = false; break; }
          uint8_t* sa = smem + s * S::STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], S::STAGE_BYTES);
          tma_load_3d(sa, ma, &full[s], (kb0 + kb) * kx, tc.m0, 0);
          tma_load_3d(sa + S::A_BYTES, mb, &full[s], (kb0 + kb) * kx, tc.n0, 0);
        }
      }
      if (!ok) {  // let copies still in flight land before the CTA exits
        for (uint32_t j = (it > uint32_t(S::STAGES) ? it - S::STAGES : 0); j < it; ++j)
          mbar_wait(&full[j % S::STAGES], (j / S::STAGES) & 1, nullptr, 0);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------ MMA issuer
    if (lane == 0) {
      // the product count as a compile-time constant: two-piece forms have
      // three products, three-piece ones six (BF16x6) or nine (BF16x9)
      if constexpr (NP == 2)
        mma_issue_loop<NP, BN, GROUPED, TF32, FUSED, 3>(single, probs, tiles, total_tiles, smem,
                                                        tmem, full, empty, main_full, main_empty,
                                                        tile_full, tmem_empty, chunk_kb, fmt, err);
      else if (nprod == 9)
        mma_issue_loop<NP, BN, GROUPED, TF32, FUSED, 9>(single, probs, tiles, total_tiles, smem,
                                                        tmem, full, empty, main_full, main_empty,
                                                        tile_full, tmem_empty, chunk_kb, fmt, err);
      else
        mma_issue_loop<NP, BN, GROUPED, TF32, FUSED, 6>(single, probs, tiles, total_tiles, smem,
                                                        tmem, full, empty, main_full, main_empty,
                                                        tile_full, tmem_empty, chunk_kb, fmt, err);
    }
    __syncwarp();
  } else if (DUAL) {
    // ---------------------------------- epilogue warps that also convert
    if constexpr (DUAL)
      fused_dual<NP, BN, EPI>(probs, tiles, single.chunk_sums, smem, tmem, full, empty,
                              raw_full, raw_empty, main_full, main_empty, tile_full, tmem_empty,
                              stage_free, chunk_kb, warp, lane, err);
  } else if (warp < 2 + kTcEpiWarps) {
    // ------------------------------------------------------ epilogue warps
    constexpr int HALF = BN / 2;  // columns per epilogue warp
    const int ew = warp - 2;
    const int q = warp & 3;       // TMEM lane quarter this warp may access
    const int col_off = (ew >> 2) * HALF;
    const uint32_t lane_base = static_cast<uint32_t>(q * 32) << 16;
    uint32_t ntile = 0;
    uint32_t nbound[NB] = {};
    bool ok = true;
    const TileRange tr = tile_range<GROUPED>(tiles, total_tiles);
    for (int t = tr.first; ok && t < tr.end; t += tr.step, ++ntile) {
      TcProblem P;
      const TileCoord tc = tile_coord<BN, GROUPED>(single, probs, tiles, t, P);
      const uint32_t buf = ntile % NB, use = ntile / NB;
      const uint32_t t_buf = tmem + buf * 2 * BN + lane_base + col_off;
      float acc[HALF];
#pragma unroll
      for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
      const int nchunks = (P.nkb + chunk_kb - 1) / chunk_kb;
      // columns of this warp's half that hold results (grouped: narrow tiles)
      const int n_live = GROUPED ? P.N - tc.n0 - col_off : HALF;
      for (int c = 0; c + 1 < nchunks; ++c) {
        if (!__all_sync(0xffffffffu,
                        mbar_wait(&main_full[buf], nbound[buf] & 1, err, kDevTimeoutAccum))) {
          ok = false;
          break;
        }
        ++nbound[buf];
        tc_fence_after();
        acc_add_tmem<HALF, GROUPED>(t_buf, acc, n_live);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&main_empty[buf]);
      }
      if (!ok) break;
      if (!__all_sync(0xffffffffu, mbar_wait(&tile_full[buf], use & 1, err, kDevTimeoutAccum)))
        break;
      tc_fence_after();
      // last main chunk, then the corrections (one 32-column slice live at a time)
      acc_add_tmem<HALF, GROUPED>(t_buf, acc, n_live);
      acc_add_tmem<HALF, GROUPED>(t_buf + BN, acc, n_live);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tmem_empty[buf]);
      epi_store<NP, BN, GROUPED, EPI>(P, tc, acc, warp, lane,
                                      reinterpret_cast<float*>(smem + RING + 256));
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, S::TMEM_COLS);
  }
}

// ---------------------------------------------------------------- split pass
// r - p for a packed pair p of 16-bit pieces (x in the low half, y in the
// high half) as two mixed-precision FMAs, p * -1 + r, that read the 16-bit
// halves directly: no widening of the pieces to FP32 first.  The difference
// is exact in FP32 (p is r rounded to 8 or 11 significant bits), so this is
// the same value as the subtraction after widening.  The split is bound by
// the integer/conversion pipe in the fused converters; the FMAs run on the
// FP32 pipe (fused 256-problem group: 164 -> 151 us).
__device__ __forceinline__ float2 sub_pieces_bf16x2(uint32_t p, float2 r) {
  float2 d;
  asm("{\n\t.reg .b16 lo, hi, m1;\n\tmov.b32 {lo, hi}, %2;\n\tmov.b16 m1, 0xBF80;\n\t"
      "fma.rn.f32.bf16 %0, lo, m1, %3;\n\tfma.rn.f32.bf16 %1, hi, m1, %4;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "r"(p), "f"(r.x), "f"(r.y));
  return d;
}
__device__ __forceinline__ float2 sub_pieces_f16x2(uint32_t p, float2 r) {
  float2 d;
  asm("{\n\t.reg .b16 lo, hi, m1;\n\tmov.b32 {lo, hi}, %2;\n\tmov.b16 m1, 0xBC00;\n\t"
      "fma.rn.f32.f16 %0, lo, m1, %3;\n\tfma.rn.f32.f16 %1, hi, m1, %4;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "r"(p), "f"(r.x), "f"(r.y));
  return d;
}

// Pieces of two consecutive k of one row, each piece plane as one packed
// 16-bit pair: bf16 pieces (FMT 0: x0 = bf16(x), x1 = bf16(x - x0), ...) or
// the FP16x3 form's two fp16 pieces of x * 2^e (FMT 1; e = the row's
// f16_scale_exp; only two-piece operands use it).
template <int NP, int FMT>
__device__ __forceinline__ void pieces_pair(float x0, float x1, int e, uint32_t (&out)[NP]) {
  if constexpr (FMT == 1) {
    // paired conversions (each element rounded to nearest, as single ones)
    const float y0 = scale_pow2(x0, e), y1 = scale_pow2(x1, e);
    const __half2 hi = __float22half2_rn(make_float2(y0, y1));
    out[0] = *reinterpret_cast<const uint32_t*>(&hi);
    const __half2 lo = __float22half2_rn(sub_pieces_f16x2(out[0], make_float2(y0, y1)));
    out[1] = *reinterpret_cast<const uint32_t*>(&lo);
    return;
  }
  // one paired conversion per piece (the same rounding as two single ones)
  float2 rem = make_float2(x0, x1);
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    if (NP == 3 && p == 2) {
      // what is left after two bf16 pieces has at most 8 significant bits
      // (x0 takes the top 8 of x's 24, x1 the top 8 of the <= 16 left), so
      // its upper half is already the bf16 value: taken without a
      // conversion instruction (those issue at a fraction of the FP32 rate).
      // It differs from rounding only below bf16's normal range (|r| <
      // 2^-126), by less than 2^-133.
      out[p] = __byte_perm(__float_as_uint(rem.x), __float_as_uint(rem.y), 0x7632);
      break;
    }
    const __nv_bfloat162 two = __float22bfloat162_rn(rem);
    out[p] = *reinterpret_cast<const uint32_t*>(&two);
    if (p + 1 < NP) rem = sub_pieces_bf16x2(out[p], rem);
  }
}

// Magnitude of x if it is finite, else 0: the FP16x3 scale follows the
// operand's finite elements, so an infinity (which stays infinite under any
// scale) does not leave the other elements unscaled and overflowing fp16.
__device__ __forceinline__ float finite_abs(float x) {
  const float a = fabsf(x);
  return a <= FLT_MAX ? a : 0.f;  // false for inf and NaN
}

// Scale exponent of row r of an operand's FP16x3 pieces (0 for bf16 pieces).
__device__ __forceinline__ int f16_row_exp(const unsigned* fmax, int r) {
  return fmax ? f16_scale_exp(fmax[r]) : 0;
}

// x rounded to TF32 (10 stored significand bits, round to nearest, ties
// away from zero), as an FP32 bit pattern with the low 13 bits clear.
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// The pieces of 8 consecutive k of one row (v[0..7]) into the planes at
// dst + p * plane + off: one 16-byte store per plane of 16-bit pieces, two
// per plane of TF32 pieces (FMT 2: x0 = tf32(x), x1 = tf32(x - x0); x - x0
// is exact in FP32, and x0 + x1 keeps 22 significant bits of x).
template <int NP, int FMT>
__device__ __forceinline__ void store_pieces8(__nv_bfloat16* __restrict__ dst, size_t plane,
                                              size_t off, const float (&v)[8], int ex) {
  if constexpr (FMT == 2) {
    uint32_t hi[8], lo[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      hi[e] = to_tf32(v[e]);
      lo[e] = to_tf32(v[e] - __uint_as_float(hi[e]));
    }
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    uint4* p0 = reinterpret_cast<uint4*>(d + off);
    uint4* p1 = reinterpret_cast<uint4*>(d + plane + off);
    p0[0] = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    p0[1] = make_uint4(hi[4], hi[5], hi[6], hi[7]);
    p1[0] = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    p1[1] = make_uint4(lo[4], lo[5], lo[6], lo[7]);
  } else {
    uint32_t packed[NP][4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      uint32_t two[NP];
      pieces_pair<NP, FMT>(v[e], v[e + 1], ex, two);
#pragma unroll
      for (int p = 0; p < NP; ++p) packed[p][e / 2] = two[p];
    }
#pragma unroll
    for (int p = 0; p < NP; ++p)
      *reinterpret_cast<uint4*>(dst + p * plane + off) =
          make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
  }
}

// One 32-row x 64-k tile of op(X) (element (r, k) at src[r*sr + k*sk]) into
// NP bf16 planes dst[p][rows][Kp], through shared memory so that both source
// layouts are read coalesced: float4 loads along the contiguous dimension
// when the operand allows it, one 16-byte store of 8 k per plane per thread.
// Zero for k >= K.
template <int NP, int FMT>
__device__ __forceinline__ void split_tile(const float* __restrict__ src, long long sr,
                                           long long sk, int rows, int K, int Kp,
                                           __nv_bfloat16* __restrict__ dst, int r0, int k0,
                                           float (*tile)[65], const unsigned* fmax) {
  const int t = threadIdx.x;
  const bool kcontig = sk == 1;
  const long long other = kcontig ? sr : sk;
  const bool vec = ((reinterpret_cast<uintptr_t>(src) & 15) == 0) && ((other & 3) == 0);
  if (kcontig) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int idx = t + 256 * i, rr = idx >> 4, c4 = (idx & 15) * 4;
      const int r = r0 + rr, k = k0 + c4;
      float v[4];
      if (vec && r < rows && k + 3 < K) {
        const float4 x = *reinterpret_cast<const float4*>(src + r * sr + k);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = (r < rows && k + e < K) ? src[r * sr + k + e] : 0.f;
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) tile[rr][c4 + e] = v[e];
    }
  } else {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int idx = t + 256 * i, kk = idx >> 3, q4 = (idx & 7) * 4;
      const int r = r0 + q4, k = k0 + kk;
      float v[4];
      if (vec && r + 3 < rows && k < K) {
        const float4 x = *reinterpret_cast<const float4*>(src + r + k * sk);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = (r + e < rows && k < K) ? src[(r + e) * sr + k * sk] : 0.f;
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) tile[q4 + e][kk] = v[e];
    }
  }
  __syncthreads();
  const int rr = t >> 3, g8 = (t & 7) * 8;
  const int r = r0 + rr, k = k0 + g8;
  if (r < rows && k < Kp) {
    const size_t plane = static_cast<size_t>(rows) * Kp;
    const int ex = FMT == 1 ? f16_row_exp(fmax, r) : 0;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = tile[rr][g8 + e];
    store_pieces8<NP, FMT>(dst, plane, static_cast<size_t>(r) * Kp + k, v, ex);
  }
}

template <int NP, int FMT>
__global__ void __launch_bounds__(256) split_pieces_kernel(const float* __restrict__ src,
                                                           long long sr, long long sk, int rows,
                                                           int K, int Kp,
                                                           __nv_bfloat16* __restrict__ dst,
                                                           const unsigned* fmax) {
  __shared__ float tile[32][65];
  split_tile<NP, FMT>(src, sr, sk, rows, K, Kp, dst, blockIdx.y * 32, blockIdx.x * 64, tile, fmax);
}

// Raw values of one 32 x 64 tile, read with the same float4 pattern as
// split_tile, kept in registers so the next tile's loads overlap the current
// tile's split and stores.
struct RawTile {
  float v[2][4];
};

__device__ __forceinline__ void load_raw(const SplitJob& j, int r0, int k0, RawTile& out) {
  const int t = threadIdx.x;
  if (j.gather) {  // implicit im2col: the same thread layout, gathered from x
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int idx = t + 256 * i;
      // 4 consecutive pixels at one tap: rows are taps and k pixels (2), or
      // rows are pixels and k taps (1)
      int tap, pix, n;
      if (j.gather == 2) {
        const int rr = idx >> 4, c4 = (idx & 15) * 4;
        tap = r0 + rr;
        pix = k0 + c4;
        n = tap < j.rows ? j.K - pix : 0;
      } else {
        const int kk = idx >> 3, q4 = (idx & 7) * 4;
        tap = k0 + kk;
        pix = r0 + q4;
        n = tap < j.K ? j.rows - pix : 0;
      }
      const Im2colTap tp = im2col_tap(j.im, tap);
      Im2colPix px = im2col_pix(j.im, pix);
      if ((j.im.Wo & 3) == 0) {
        // pix is a multiple of 4, so the 4 pixels lie in one image row (and
        // all exist when the first does): one row address, one bounds test
        // per pixel, no walk
        const int yy = px.i * j.im.stride - j.im.pad + tp.ki;
        const int x0 = px.j * j.im.stride - j.im.pad + tp.kj;
        const bool ok = n > 0 && static_cast<unsigned>(yy) < static_cast<unsigned>(j.im.H);
        const float* row = j.im.x + ((static_cast<long long>(tp.c) * j.im.B + px.b) * j.im.H +
                                     (ok ? yy : 0)) * static_cast<long long>(j.im.W);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int xx = x0 + e * j.im.stride;
          out.v[i][e] =
              (ok && static_cast<unsigned>(xx) < static_cast<unsigned>(j.im.W)) ? row[xx] : 0.f;
        }
        continue;
      }
      // walk the image row: one address per row, a step of `stride` per pixel
      int xx = px.j * j.im.stride - j.im.pad + tp.kj;
      int yy = px.i * j.im.stride - j.im.pad + tp.ki;
      const float* row = j.im.x + ((static_cast<long long>(tp.c) * j.im.B + px.b) * j.im.H + yy) *
                                      static_cast<long long>(j.im.W);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        out.v[i][e] = (e < n && yy >= 0 && yy < j.im.H && xx >= 0 && xx < j.im.W) ? row[xx] : 0.f;
        if (++px.j == j.im.Wo) {  // next image row (or image)
          px.j = 0;
          if (++px.i == j.im.Ho) { px.i = 0; ++px.b; }
          xx = -j.im.pad + tp.kj;
          yy = px.i * j.im.stride - j.im.pad + tp.ki;
          row = j.im.x + ((static_cast<long long>(tp.c) * j.im.B + px.b) * j.im.H + yy) *
                             static_cast<long long>(j.im.W);
        } else {
          xx += j.im.stride;
        }
      }
    }
    return;
  }
  const bool kcontig = j.sk == 1;
  const long long other = kcontig ? j.sr : j.sk;
  const bool vec = ((reinterpret_cast<uintptr_t>(j.src) & 15) == 0) && ((other & 3) == 0);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int idx = t + 256 * i;
    if (kcontig) {
      const int rr = idx >> 4, c4 = (idx & 15) * 4, r = r0 + rr, k = k0 + c4;
      if (vec && r < j.rows && k + 3 < j.K) {
        const float4 x = *reinterpret_cast<const float4*>(j.src + r * j.sr + k);
        out.v[i][0] = x.x; out.v[i][1] = x.y; out.v[i][2] = x.z; out.v[i][3] = x.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          out.v[i][e] = (r < j.rows && k + e < j.K) ? j.src[r * j.sr + k + e] : 0.f;
      }
    } else {
      const int kk = idx >> 3, q4 = (idx & 7) * 4, r = r0 + q4, k = k0 + kk;
      if (vec && r + 3 < j.rows && k < j.K) {
        const float4 x = *reinterpret_cast<const float4*>(j.src + r + k * j.sk);
        out.v[i][0] = x.x; out.v[i][1] = x.y; out.v[i][2] = x.z; out.v[i][3] = x.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          out.v[i][e] = (r + e < j.rows && k < j.K) ? j.src[(r + e) * j.sr + k * j.sk] : 0.f;
      }
    }
  }
}

__device__ __forceinline__ void raw_to_smem(const SplitJob& j, const RawTile& in, float (*tile)[65]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int idx = t + 256 * i;
    if (j.sk == 1) {
      const int rr = idx >> 4, c4 = (idx & 15) * 4;
#pragma unroll
      for (int e = 0; e < 4; ++e) tile[rr][c4 + e] = in.v[i][e];
    } else {
      const int kk = idx >> 3, q4 = (idx & 7) * 4;
#pragma unroll
      for (int e = 0; e < 4; ++e) tile[q4 + e][kk] = in.v[i][e];
    }
  }
}

// bf16 pieces of one tile from shared memory: 8 consecutive k of one row per
// thread, one 16-byte store per plane.
template <int NP, int FMT>
__device__ __forceinline__ void split_store(const SplitJob& j, int r0, int k0, float (*tile)[65]) {
  const int t = threadIdx.x;
  const int rr = t >> 3, g8 = (t & 7) * 8;
  const int r = r0 + rr, k = k0 + g8;
  if (r >= j.rows || k >= j.Kp) return;
  const size_t plane = static_cast<size_t>(j.rows) * j.Kp;
  const int ex = FMT == 1 ? f16_row_exp(j.fmax, r) : 0;
  float v[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = tile[rr][g8 + e];
  store_pieces8<NP, FMT>(j.dst, plane, static_cast<size_t>(r) * j.Kp + k, v, ex);
}

// Many operands in one launch.  Blocks walk the tiles grid-stride; the next
// tile's loads are issued before the current tile is split and stored, and
// the jobs' first-tile indices are cached in shared memory so finding a
// tile's job is a search in shared memory, not a chain of global loads.
constexpr int kJobCache = 2048;

__device__ __forceinline__ int find_job(const int* starts, const SplitJob* jobs, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const int st = n <= kJobCache ? starts[mid] : jobs[mid].tile_start;
    if (st <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void tile_origin(const SplitJob& j, int b, int& r0, int& k0) {
  const int local = b - j.tile_start;
  const int tiles_k = (j.Kp + 63) / 64;
  r0 = (local / tiles_k) * 32;
  k0 = (local % tiles_k) * 64;
}

template <int NP, int FMT>
__device__ __forceinline__ void split_batched_body(const SplitJob* __restrict__ jobs, int njobs,
                                                   int total_tiles) {
  __shared__ float tile[32][65];
  __shared__ int starts[kJobCache];
  const int cached = min(njobs, kJobCache);
  for (int i = threadIdx.x; i < cached; i += blockDim.x) starts[i] = jobs[i].tile_start;
  __syncthreads();
  int b = blockIdx.x;
  if (b >= total_tiles) return;
  SplitJob cur = jobs[find_job(starts, jobs, njobs, b)];
  int r0, k0;
  tile_origin(cur, b, r0, k0);
  RawTile raw;
  load_raw(cur, r0, k0, raw);
  for (; b < total_tiles; b += gridDim.x) {
    raw_to_smem(cur, raw, tile);
    const int nb = b + gridDim.x;
    SplitJob nxt = cur;
    int nr0 = 0, nk0 = 0;
    if (nb < total_tiles) {  // next tile's loads in flight during this tile's stores
      nxt = jobs[find_job(starts, jobs, njobs, nb)];
      tile_origin(nxt, nb, nr0, nk0);
      load_raw(nxt, nr0, nk0, raw);
    }
    __syncthreads();
    split_store<NP, FMT>(cur, r0, k0, tile);
    __syncthreads();
    cur = nxt;
    r0 = nr0;
    k0 = nk0;
  }
}

template <int NP, int FMT>
__global__ void __launch_bounds__(256) split_pieces_batched_kernel(const SplitJob* __restrict__ jobs,
                                                                   int njobs, int total_tiles) {
  split_batched_body<NP, FMT>(jobs, njobs, total_tiles);
}

// The same for a few operands whose job records travel as the kernel's
// parameter (read through the constant cache): nothing to write to device
// memory first, so a sequence of launches stays capture-safe without a table.
template <int NP, int FMT>
__global__ void __launch_bounds__(256) split_pieces_param_kernel(
    const __grid_constant__ SplitJobTable t, int njobs, int total_tiles) {
  split_batched_body<NP, FMT>(t.jobs, njobs, total_tiles);
}

// FP16x3 form, first step of the split: the largest finite magnitude of
// every row of op(X), folded into the job's row words (j.fmax[r]) with
// atomicMax on the IEEE pattern, which orders non-negative floats like their
// values.  A tile (32 rows x 64 k, loaded as the split loads it, implicit
// im2col gathers included) goes through shared memory so that both source
// layouts reduce the same way: 8 threads per row, 8 values each, then a
// shuffle reduction and one atomicMax per row and tile.  NaNs and infinities
// are skipped: they propagate through the pieces whatever the scale.
__device__ __forceinline__ void tile_row_max(const SplitJob& j, int r0, int k0, float (*tile)[65]) {
  RawTile raw;
  load_raw(j, r0, k0, raw);
  raw_to_smem(j, raw, tile);
  __syncthreads();
  const int t = threadIdx.x, rr = t >> 3, g8 = (t & 7) * 8;
  float m = 0.f;
#pragma unroll
  for (int e = 0; e < 8; ++e) m = fmaxf(m, finite_abs(tile[rr][g8 + e]));
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((t & 7) == 0 && r0 + rr < j.rows && m > 0.f) atomicMax(j.fmax + r0 + rr, __float_as_uint(m));
  __syncthreads();
}

// One operand stored as a plain strided matrix, read once at full width
// with nothing staged in shared memory until the end: element (r, k) at
// src[r*sr + k*sk].  KCONTIG (sk == 1): 16 threads per row walk its k range
// with float4 loads, 16 rows per block; otherwise (sr == 1: rows are
// consecutive in memory) a thread keeps the maxima of 4 consecutive rows
// (one float4 per k) and 4 threads share a k range, 256 rows per block.
// Block (x, y) takes row band x and the y-th run of `kper` k; a shuffle or
// shared-memory reduction ends with one atomicMax per row and block.
template <bool KCONTIG, bool VEC>
__global__ void __launch_bounds__(256) operand_row_max_kernel(const float* __restrict__ src,
                                                              long long sr, long long sk, int rows,
                                                              int K, int kper, unsigned* words) {
  const int t = threadIdx.x;
  const int k0 = blockIdx.y * kper, k1 = min(K, k0 + kper);
  if constexpr (KCONTIG) {
    const int r = blockIdx.x * 16 + (t >> 4), l = t & 15;
    float m = 0.f;
    if (r < rows) {
      const float* row = src + r * sr;
      if (VEC) {  // k0 and kper are multiples of 4 here; four loads in flight
        int k = k0 + 4 * l;
        for (; k + 192 + 3 < k1; k += 256) {
          float4 v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) v[u] = *reinterpret_cast<const float4*>(row + k + 64 * u);
#pragma unroll
          for (int u = 0; u < 4; ++u)
            m = fmaxf(m, fmaxf(fmaxf(finite_abs(v[u].x), finite_abs(v[u].y)),
                               fmaxf(finite_abs(v[u].z), finite_abs(v[u].w))));
        }
        for (; k < k1; k += 64) {
          if (k + 3 < k1) {
            const float4 v = *reinterpret_cast<const float4*>(row + k);
            m = fmaxf(m, fmaxf(fmaxf(finite_abs(v.x), finite_abs(v.y)),
                               fmaxf(finite_abs(v.z), finite_abs(v.w))));
          } else {
            for (int e = k; e < k1; ++e) m = fmaxf(m, finite_abs(row[e]));
          }
        }
      } else {
        for (int k = k0 + l; k < k1; k += 16) m = fmaxf(m, finite_abs(row[k]));
      }
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (l == 0 && r < rows && m > 0.f) atomicMax(words + r, __float_as_uint(m));
  } else {
    __shared__ float part[4][256];
    const int q = t & 63, ty = t >> 6, r0 = blockIdx.x * 256 + 4 * q;
    float m[4] = {0.f, 0.f, 0.f, 0.f};
    int k = k0 + ty;
    if (VEC && r0 + 3 < rows) {  // four loads in flight
      for (; k + 12 < k1; k += 16) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          v[u] = *reinterpret_cast<const float4*>(src + (k + 4 * u) * sk + r0);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          m[0] = fmaxf(m[0], finite_abs(v[u].x));
          m[1] = fmaxf(m[1], finite_abs(v[u].y));
          m[2] = fmaxf(m[2], finite_abs(v[u].z));
          m[3] = fmaxf(m[3], finite_abs(v[u].w));
        }
      }
    }
    for (; k < k1; k += 4) {
      const float* p = src + k * sk + r0;
      if (VEC && r0 + 3 < rows) {
        const float4 v = *reinterpret_cast<const float4*>(p);
        m[0] = fmaxf(m[0], finite_abs(v.x));
        m[1] = fmaxf(m[1], finite_abs(v.y));
        m[2] = fmaxf(m[2], finite_abs(v.z));
        m[3] = fmaxf(m[3], finite_abs(v.w));
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (r0 + e < rows) m[e] = fmaxf(m[e], finite_abs(p[e]));
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) part[ty][4 * q + e] = m[e];
    __syncthreads();
    const int r = blockIdx.x * 256 + t;
    const float v = fmaxf(fmaxf(part[0][t], part[1][t]), fmaxf(part[2][t], part[3][t]));
    if (r < rows && v > 0.f) atomicMax(words + r, __float_as_uint(v));
  }
}

// FP16x3 split of an operand whose rows are contiguous in k (sk == 1), 16-byte
// aligned, with K <= kRowSplitK: one block per row keeps the whole row in
// registers (32 values a thread), takes its largest finite magnitude, writes
// the row's word and splits the registers -- one read of the operand instead
// of a row-maximum pass and a split pass that reads it again.  Same word,
// same scale and same pieces as the two passes.
constexpr int kRowSplitK = 8192;
__global__ void __launch_bounds__(256) split_rows_f16_kernel(const float* __restrict__ src,
                                                             long long sr, int K, int Kp,
                                                             __nv_bfloat16* __restrict__ dst,
                                                             int rows, unsigned* words) {
  constexpr int CH = kRowSplitK / (256 * 8);  // 8-k chunks a thread
  __shared__ float part[8];
  const int t = threadIdx.x, r = blockIdx.x;
  const float* row = src + r * sr;
  float v[CH][8];
  float m = 0.f;
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const int k0 = 2048 * j + 8 * t;
    if (k0 + 7 < K) {
      const float4 lo = *reinterpret_cast<const float4*>(row + k0);
      const float4 hi = *reinterpret_cast<const float4*>(row + k0 + 4);
      v[j][0] = lo.x; v[j][1] = lo.y; v[j][2] = lo.z; v[j][3] = lo.w;
      v[j][4] = hi.x; v[j][5] = hi.y; v[j][6] = hi.z; v[j][7] = hi.w;
    } else {
#pragma unroll
      for (int e = 0; e < 8; ++e) v[j][e] = k0 + e < K ? row[k0 + e] : 0.f;
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) m = fmaxf(m, finite_abs(v[j][e]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((t & 31) == 0) part[t >> 5] = m;
  __syncthreads();
  m = part[0];
#pragma unroll
  for (int w = 1; w < 8; ++w) m = fmaxf(m, part[w]);
  const unsigned bits = __float_as_uint(m);
  if (t == 0) words[r] = bits;
  const int ex = f16_scale_exp(bits);
  const size_t plane = static_cast<size_t>(rows) * Kp;
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const int k0 = 2048 * j + 8 * t;
    if (k0 < Kp) store_pieces8<2, 1>(dst, plane, static_cast<size_t>(r) * Kp + k0, v[j], ex);
  }
}

// One operand of any strides through the tiled reduction, tiles grid-stride.
__global__ void __launch_bounds__(256) operand_max_single_kernel(const __grid_constant__ SplitJob j,
                                                                 int total_tiles) {
  __shared__ float tile[32][65];
  for (int b = blockIdx.x; b < total_tiles; b += gridDim.x) {
    int r0, k0;
    tile_origin(j, b, r0, k0);
    tile_row_max(j, r0, k0, tile);
  }
}

// Many operands (grouped plans): blocks walk all jobs' tiles grid-stride.
__global__ void __launch_bounds__(256) operand_max_batched_kernel(const SplitJob* __restrict__ jobs,
                                                                  int njobs, int total_tiles) {
  __shared__ float tile[32][65];
  __shared__ int starts[kJobCache];
  const int cached = min(njobs, kJobCache);
  for (int i = threadIdx.x; i < cached; i += blockDim.x) starts[i] = jobs[i].tile_start;
  __syncthreads();
  for (int b = blockIdx.x; b < total_tiles; b += gridDim.x) {
    const SplitJob j = jobs[find_job(starts, jobs, njobs, b)];
    int r0, k0;
    tile_origin(j, b, r0, k0);
    tile_row_max(j, r0, k0, tile);
  }
}

// --------------------------------------------------------- fused converters
// A fused stage is the kernel's a tile (128 rows) and b tile (BN rows), 32 k
// deep, in the raw ring as TMA wrote it: a tile whose source has k
// contiguous is [rows][32] floats in 128-byte rows with the 128-byte swizzle
// (16-byte unit u of row r at unit u ^ (r & 7)), one whose source has rows
// contiguous is [32][rows] floats, unswizzled.  Converter thread ct takes 8-k
// chunks (row, c), k in [8c, 8c + 8): along rows where the tile is [32][rows]
// (consecutive threads read consecutive words), else four chunks of a row
// per four threads (each reads two 16-byte units).  It first loads all of
// its chunks of the stage into registers, then waits for the piece stage,
// splits each value into three bf16 pieces as the pre-pass does and stores
// them as 16-byte rows of the three planes at the 64-byte-swizzled position
// the piece copies would have had (byte offset r * 64 + 16 c, its 16-byte
// unit index XORed with bits 1-2 of the row), then makes its stores visible
// to the tensor core (fence.proxy.async) and arrives on the piece stage's
// full barrier and the raw stage's empty barrier.  (Loading a stage's
// chunks two at a time between stores left each load's latency exposed:
// 13% slower at 4096^3.)
//
// The split is bound by the integer/conversion pipe, so the chunks' raw and
// piece offsets are computed once per tile, not per stage (256-problem
// group: 150 -> 140 us).  The converter warps are warps 10-15 of the CTA, on
// SM sub-partitions 2, 3, 0, 1, 2, 3: the caller numbers the threads of
// warps 12 and 13, alone on theirs, first, so that the chunks left over
// after five rounds (threads 0-63 take a sixth) fall to them (140 -> 137 us).
template <int NP, int BN>
__device__ void fused_convert(const TcProblem* __restrict__ probs, const int4* __restrict__ tiles,
                              uint8_t* pieces, uint8_t* raw, uint64_t* full, uint64_t* empty,
                              uint64_t* raw_full, uint64_t* raw_empty, int ct, int* err) {
  using S = TcShape<NP, BN, false>;
  constexpr int CH_A = kTcBM * (kTcKB / 8);
  constexpr int CH = CH_A + BN * (kTcKB / 8);
  constexpr int PER = (CH + kTcConvThreads - 1) / kTcConvThreads;
  static_assert(CH_A % 32 == 0 && kTcConvThreads % 32 == 0,
                "a warp's chunks are all of one operand");
  static_assert(kTcKB == 32 && S::RAW_K == kTcKB,
                "32-deep stages: 128-byte raw rows, 64-byte piece rows");
  static_assert(S::RAW_A % 32 == 0, "bit 4 of a raw offset is bit 0 of its 16-byte unit");
  const int4 range = tiles[blockIdx.x];
  uint32_t it = 0;
  for (int t = range.x; t < range.y; ++t) {
    const int4 rec = tiles[gridDim.x + t];
    const TcProblem& P = probs[rec.x];
    const int nkb = P.nkb, kc_a = P.kc_a, kc_b = P.kc_b;
    // this tile's chunk offsets: raw bytes from the raw stage (for a
    // [rows][32] tile the first of its two units; the second is at bit 4
    // flipped: unit (2c + 1) ^ (r & 7) = ((2c) ^ (r & 7)) ^ 1) and piece bytes
    // from the piece stage
    uint32_t ldo[PER], sto[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int ch = ct + kTcConvThreads * i;
      const bool is_a = ch < CH_A;
      const int local = is_a ? ch : ch - CH_A, nrows = is_a ? kTcBM : BN;
      const bool kc = is_a ? kc_a : kc_b;
      const int r = kc ? local >> 2 : local % nrows, c = kc ? local & 3 : local / nrows;
      ldo[i] = (is_a ? 0u : uint32_t(S::RAW_A)) +
               (kc ? uint32_t(r * 128 + (((2 * c) ^ (r & 7)) << 4))
                   : uint32_t(((8 * c) * nrows + r) * 4));
      sto[i] = (is_a ? 0u : uint32_t(S::A_BYTES)) + static_cast<uint32_t>(r) * 64 +
               ((c ^ ((r >> 1) & 3)) << 4);
    }
    for (int kb = 0; kb < nkb; ++kb, ++it) {
      const int rs = it % kTcRawStages, ps = it % kTcFusedPieceStages;
      if (!__all_sync(0xffffffffu,
                      mbar_wait(&raw_full[rs], (it / kTcRawStages) & 1, err, kDevTimeoutFull)))
        return;
      const uint8_t* ra = raw + rs * S::RAW_BYTES;
      float v[PER][8];
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int ch = ct + kTcConvThreads * i;
        if (CH % kTcConvThreads != 0 && ch >= CH) continue;
        const bool is_a = ch < CH_A;
        if (is_a ? kc_a : kc_b) {  // [rows][32] floats, 128-byte swizzle
          const float4 lo = *reinterpret_cast<const float4*>(ra + ldo[i]);
          const float4 hi = *reinterpret_cast<const float4*>(ra + (ldo[i] ^ 16u));
          v[i][0] = lo.x; v[i][1] = lo.y; v[i][2] = lo.z; v[i][3] = lo.w;
          v[i][4] = hi.x; v[i][5] = hi.y; v[i][6] = hi.z; v[i][7] = hi.w;
        } else {  // [32][rows] floats
          const int nrows = is_a ? kTcBM : BN;
          const float* col = reinterpret_cast<const float*>(ra + ldo[i]);
#pragma unroll
          for (int e = 0; e < 8; ++e) v[i][e] = col[e * nrows];
        }
      }
      if (!__all_sync(0xffffffffu, mbar_wait(&empty[ps], ((it / kTcFusedPieceStages) & 1) ^ 1,
                                              err, kDevTimeoutEmpty)))
        return;
      uint8_t* pa = pieces + ps * S::STAGE_BYTES;
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int ch = ct + kTcConvThreads * i;
        if (CH % kTcConvThreads != 0 && ch >= CH) continue;
        const int plane = ch < CH_A ? S::A_PLANE : S::B_PLANE;
        uint32_t packed[NP][4];
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          uint32_t two[NP];
          pieces_pair<NP, 0>(v[i][e], v[i][e + 1], 0, two);
#pragma unroll
          for (int p = 0; p < NP; ++p) packed[p][e / 2] = two[p];
        }
#pragma unroll
        for (int p = 0; p < NP; ++p)
          *reinterpret_cast<uint4*>(pa + sto[i] + p * plane) =
              make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
      }
      // the stores and the raw loads, ordered before the tensor core reads
      // the pieces and before the next copy overwrites the raw stage (a
      // copy is an async-proxy write: releasing the raw stage right after
      // the loads, without this fence, let copies land in it while its
      // loads were in flight -- wrong results on the GPU)
      fence_proxy_async();
      mbar_arrive(&full[ps]);
      mbar_arrive(&raw_empty[rs]);
    }
  }
}


// Final epilogue of a fused 256-wide tile (the use-th of this CTA), in two
// halves of the warp's 128 columns so that no more than 64 sums are in
// registers at once: per half, the drained chunk sums (for the first half
// read while the last MMAs run), then the last main chunk and the
// corrections -- the order of the other launches, so the same bits -- the
// first half parked in `stage` (this warp's 32 x 65 floats of the piece
// stage that no MMA reads until the warps convert into it again), then TMEM
// is released and both halves stored: rows of 32 consecutive columns per
// store instruction, or for a transposed problem (swap: the kernel row is a
// C column) 32 consecutive floats of one C row.  P is a copy: fields read
// through a pointer to the problem table would be reloaded after every
// store to C (the compiler cannot rule out that they alias).
template <int NP, int BN, bool EPI>
__device__ __forceinline__ bool fused_dual_finish(const TcProblem P, const TileCoord& tc,
                                                  const float* sums, uint32_t t_acc,
                                                  uint64_t* tile_full, uint64_t* tmem_empty,
                                                  uint64_t* stage_free, uint32_t use,
                                                  int chunk_kb, int warp, int lane, float* stage,
                                                  int* err) {
  constexpr int HALF = BN / 2, Q = HALF / 2;
  const int ew = warp - 2, q = warp & 3, col_off = (ew >> 2) * HALF;
  const int n_live = P.N - tc.n0 - col_off;
  const bool drained = P.nkb > chunk_kb;
  float a[Q];
#pragma unroll
  for (int half = 0; half < 2; ++half) {
#pragma unroll
    for (int j = 0; j < Q; ++j)
      a[j] = drained && half * Q + j < n_live ? sums[(half * Q + j) * 32] : 0.f;
    if (half == 0) {
      if (!__all_sync(0xffffffffu, mbar_wait(&tile_full[0], use & 1, err, kDevTimeoutAccum)))
        return false;
      tc_fence_after();
    }
#pragma unroll
    for (int part = 0; part < 2; ++part) {
#pragma unroll
      for (int c16 = 0; c16 < Q / 16; ++c16) {
        if (half * Q + c16 * 16 >= n_live) break;
        uint32_t r[16];
        tmem_ld_32x32b_x16(t_acc + part * BN + half * Q + c16 * 16, r);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) a[c16 * 16 + j] += __uint_as_float(r[j]);
      }
    }
    if (half == 0) {
#pragma unroll
      for (int j = 0; j < Q; ++j) stage[lane * 65 + j] = a[j];
    }
  }
  tc_fence_before();
  __syncwarp();
  if (lane == 0) mbar_arrive(&tmem_empty[0]);
  const bool has_epi = EPI && (P.epi.bias != nullptr || P.epi.act != 0);
  const int row0 = tc.m0 + q * 32;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    if (half == 1) {  // the second half goes through the same staging rows
      __syncwarp();
#pragma unroll
      for (int j = 0; j < Q; ++j) stage[lane * 65 + j] = a[j];
    }
    __syncwarp();
    const int c_base = tc.n0 + col_off + half * Q;  // first kernel column of the half
    if (P.swap) {
      const int r = row0 + lane;
      if (r < P.M) {
#pragma unroll 8
        for (int j = 0; j < Q; ++j) {
          const int c = c_base + j;
          if (c < P.N) {
            float* cp = P.C + static_cast<size_t>(c) * P.ldc + r;
            float v = P.alpha * stage[lane * 65 + j];
            if (P.beta != 0.f) v += P.beta * *cp;
            if (has_epi) v = epilogue_apply(v, P.epi, c);
            *cp = v;
          }
        }
      }
      continue;
    }
#pragma unroll
    for (int c32 = 0; c32 < Q / 32; ++c32) {
      const int c = c_base + c32 * 32 + lane;
      if (c < P.N) {
        for (int rr = 0; rr < 32; ++rr) {
          const int row = row0 + rr;
          if (row >= P.M) break;
          float* cp = P.C + static_cast<size_t>(row) * P.ldc + c;
          float v = P.alpha * stage[rr * 65 + c32 * 32 + lane];
          if (P.beta != 0.f) v += P.beta * *cp;
          if (has_epi) v = epilogue_apply(v, P.epi, row);
          *cp = v;
        }
      }
    }
  }
  __syncwarp();
  if (lane == 0) mbar_arrive(stage_free);  // this warp no longer reads `stage`
  return true;
}

// The eight epilogue warps of a 256-wide fused launch, which convert too
// (ten warps in all, at most 168 registers each: three warps share one
// scheduler's 16K registers).  Each piece stage comes from two 16-deep raw
// stages: a tile whose source has k contiguous is [rows][16] floats in
// 64-byte rows with the 64-byte swizzle (16-byte unit u of row r at
// u ^ ((r >> 1) & 3)), one whose source has rows contiguous is [16][rows]
// floats.  Thread ct (0..255) converts three 8-k chunks of each raw stage:
// one of the a tile (row ct / 2, or column-major position ct), two of the b
// tile, loaded first, then converted and stored, and the raw stage released
// after a proxy fence, as in fused_convert.  A 128 x 256 accumulator would take 128 registers of every
// thread, so the drained chunks of the main accumulator are summed in the
// CTA's 128 KB of `chunk_sums` (L2-resident; laid out so that a warp's
// access to one column is 32 consecutive floats) rather than in registers;
// the sums are added in the order the other launches use, so the results
// are the same bits.  Between stages the warps do their epilogue work in an
// order that lets the MMA issuer run ahead: a chunk is drained after the
// first stage of the next chunk has been converted, and a tile's final
// epilogue (TMEM read, release, stores) runs after the first stage of the
// next tile has been converted, so the MMAs of that stage can start as soon
// as the accumulators are released.  TMEM holds one tile (main + correction
// accumulators, 2 x 256 columns).
template <int NP, int BN, bool EPI>
__device__ void fused_dual(const TcProblem* __restrict__ probs, const int4* __restrict__ tiles,
                           float* chunk_sums, uint8_t* smem, uint32_t tmem, uint64_t* full,
                           uint64_t* empty, uint64_t* raw_full, uint64_t* raw_empty,
                           uint64_t* main_full, uint64_t* main_empty, uint64_t* tile_full,
                           uint64_t* tmem_empty, uint64_t* stage_free, int chunk_kb, int warp,
                           int lane, int* err) {
  using S = TcShape<NP, BN, false>;
  constexpr int HALF = BN / 2;
  constexpr int SUB = kTcKB / S::RAW_K;  // raw stages per piece stage
  constexpr int CPR = S::RAW_K / 8;      // 8-k chunks per row of a raw stage
  constexpr int CH_A = kTcBM * CPR;
  constexpr int CH = CH_A + BN * CPR;
  constexpr int NT = fused_conv_threads(BN);
  constexpr int PER = CH / NT;
  static_assert(S::ACC_BUFS == 1 && SUB == 2 && CPR == 2, "256-wide fused tiles");
  static_assert(CH % NT == 0 && CH_A == NT, "pass 0 converts the a tile, the others the b tile");
  static_assert(size_t(kTcEpiWarps) * HALF * 32 * 4 == kTcFusedSumBytes, "chunk sum layout");
  const int ew = warp - 2, ct = ew * 32 + lane;
  const int q = warp & 3, col_off = (ew >> 2) * HALF;
  const uint32_t t_acc = tmem + (static_cast<uint32_t>(q * 32) << 16) + col_off;
  uint8_t* raw = smem + kTcFusedPieceStages * S::STAGE_BYTES;
  static_assert(size_t(kTcEpiWarps) * 32 * 65 * 4 <= size_t(S::STAGE_BYTES),
                "the final epilogue stages half a tile in a piece stage");
  // this thread's column j of the chunk sums: sums[j * 32]
  float* sums = chunk_sums + (size_t(blockIdx.x) * kTcEpiWarps + ew) * HALF * 32 + lane;
  const int4 range = tiles[blockIdx.x];
  uint32_t it = 0, rit = 0, nbound = 0, ntile = 0;
  uint32_t nfin = 0, nfin_seen = 0;    // final epilogues done, and waited for
  int4 pend = make_int4(-1, 0, 0, 0);  // tile record whose final epilogue is due


  for (int t = range.x; t < range.y; ++t) {
    const int4 rec = tiles[gridDim.x + t];
    const int nkb = probs[rec.x].nkb, kc_a = probs[rec.x].kc_a, kc_b = probs[rec.x].kc_b;
    for (int kb = 0; kb < nkb; ++kb, ++it) {
      const int ps = it % kTcFusedPieceStages;
      uint8_t* pa = smem + ps * S::STAGE_BYTES;
#pragma unroll 1
      for (int h = 0; h < SUB; ++h, ++rit) {
        const int rs = rit % kTcRawStages;
        if (!__all_sync(0xffffffffu, mbar_wait(&raw_full[rs], (rit / kTcRawStages) & 1, err,
                                                kDevTimeoutFull)))
          return;
        const uint8_t* ra = raw + rs * S::RAW_BYTES;
        float v[PER][8];
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const bool is_a = i == 0;
          const int local = is_a ? ct : ct + NT * i - CH_A, nrows = is_a ? kTcBM : BN;
          const uint8_t* src = is_a ? ra : ra + S::RAW_A;
          if (is_a ? kc_a : kc_b) {  // [rows][16] floats, 64-byte swizzle
            const int r = local / CPR, c = local % CPR, sw = (r >> 1) & 3;
            const uint8_t* row = src + r * (S::RAW_K * 4);
            const float4 lo = *reinterpret_cast<const float4*>(row + (((2 * c) ^ sw) << 4));
            const float4 hi = *reinterpret_cast<const float4*>(row + (((2 * c + 1) ^ sw) << 4));
            v[i][0] = lo.x; v[i][1] = lo.y; v[i][2] = lo.z; v[i][3] = lo.w;
            v[i][4] = hi.x; v[i][5] = hi.y; v[i][6] = hi.z; v[i][7] = hi.w;
          } else {  // [16][rows] floats
            const int r = local % nrows, c = local / nrows;
            const float* col = reinterpret_cast<const float*>(src) + (8 * c) * nrows + r;
#pragma unroll
            for (int e = 0; e < 8; ++e) v[i][e] = col[e * nrows];
          }
        }
        if (h == 0) {
          if (!__all_sync(0xffffffffu, mbar_wait(&empty[ps], ((it / kTcFusedPieceStages) & 1) ^ 1,
                                                 err, kDevTimeoutEmpty)))
            return;
          // the stage after a tile's final epilogue held that epilogue's
          // parked sums: every warp must be done with them
          if (nfin != nfin_seen) {
            if (!__all_sync(0xffffffffu,
                            mbar_wait(stage_free, (nfin - 1) & 1, err, kDevTimeoutAccum)))
              return;
            nfin_seen = nfin;
          }
        }
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const bool is_a = i == 0;
          const int local = is_a ? ct : ct + NT * i - CH_A, nrows = is_a ? kTcBM : BN;
          const bool kc = is_a ? kc_a : kc_b;
          const int r = kc ? local / CPR : local % nrows;
          const int c = h * CPR + (kc ? local % CPR : local / nrows);  // 8-k chunk of the stage
          uint32_t packed[NP][4];
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            uint32_t two[NP];
            pieces_pair<NP, 0>(v[i][e], v[i][e + 1], 0, two);
#pragma unroll
            for (int p = 0; p < NP; ++p) packed[p][e / 2] = two[p];
          }
          uint8_t* base = is_a ? pa : pa + S::A_BYTES;
          const int plane = is_a ? S::A_PLANE : S::B_PLANE;
          const uint32_t off = static_cast<uint32_t>(r) * 64 + ((c ^ ((r >> 1) & 3)) << 4);
#pragma unroll
          for (int p = 0; p < NP; ++p)
            *reinterpret_cast<uint4*>(base + p * plane + off) =
                make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
        }
        // the raw stage's loads and these stores, ordered before the next
        // copy into the raw stage and the tensor core's reads (async proxy)
        fence_proxy_async();
        mbar_arrive(&raw_empty[rs]);
      }
      mbar_arrive(&full[ps]);
      if (kb == 0) {
        // the piece stage after the one just converted is free: the last
        // MMAs that read it belong to the finished tile
        if (pend.x >= 0 &&
            !fused_dual_finish<NP, BN, EPI>(
                probs[pend.x], TileCoord{pend.x, pend.y, pend.z}, sums, t_acc, tile_full,
                tmem_empty, stage_free, ntile - 1, chunk_kb, warp, lane,
                reinterpret_cast<float*>(smem + ((it + 1) % kTcFusedPieceStages) * S::STAGE_BYTES) +
                    ew * 32 * 65,
                err))
          return;
        if (pend.x >= 0) ++nfin;
      } else if (kb % chunk_kb == 0) {
        // the chunk that ended at stage kb - 1: the tile's first one is
        // stored, later ones added (TMEM read half a warp's columns at a
        // time; the accumulator is released once all of it is read)
        if (!__all_sync(0xffffffffu, mbar_wait(&main_full[0], nbound & 1, err, kDevTimeoutAccum)))
          return;
        ++nbound;
        tc_fence_after();
        const int n_live = probs[rec.x].N - rec.z - col_off;
        const bool first = kb == chunk_kb;
        // 32 columns at a time: the old sums are loaded together (one L2
        // round trip per slice, not one per column) while TMEM is read
#pragma unroll
        for (int c32 = 0; c32 < HALF / 32; ++c32) {
          float old[32];
          uint32_t r[32];
          const bool live = c32 * 32 < n_live;
          if (live) {
#pragma unroll
            for (int j = 0; j < 32; ++j) old[j] = first ? 0.f : sums[(c32 * 32 + j) * 32];
            tmem_ld_32x32b_x32(t_acc + c32 * 32, r);
            tmem_ld_wait();
          }
          if (c32 == HALF / 32 - 1) {  // all of the chunk read: release it
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&main_empty[0]);
          }
          if (live) {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (c32 * 32 + j < n_live) sums[(c32 * 32 + j) * 32] = old[j] + __uint_as_float(r[j]);
          }
        }
      }
    }
    pend = rec;
    ++ntile;
  }
  if (pend.x >= 0)
    fused_dual_finish<NP, BN, EPI>(
        probs[pend.x], TileCoord{pend.x, pend.y, pend.z}, sums, t_acc, tile_full, tmem_empty,
        stage_free, ntile - 1, chunk_kb, warp, lane,
        reinterpret_cast<float*>(smem + (it % kTcFusedPieceStages) * S::STAGE_BYTES) + ew * 32 * 65,
        err);
}

template <int NP, int FMT>
void launch_split(const float* src, long long sr, long long sk, int rows, int K, int Kp,
                  __nv_bfloat16* dst, cudaStream_t st, const unsigned* fmax = nullptr) {
  dim3 grid(cdiv(Kp, 64), cdiv(rows, 32));
  prof_begin(st);
  split_pieces_kernel<NP, FMT><<<grid, 256, 0, st>>>(src, sr, sk, rows, K, Kp, dst, fmax);
  prof_end(st, kProfSplitPrep);
}

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

template <int NP, int BN, bool GROUPED, bool EPI, bool TF32, bool FUSED = false>
ugemm_status launch_kernel(const CUtensorMap& ta, const CUtensorMap& tb, const TcProblem& single,
                           const CUtensorMap* maps, const TcProblem* probs, const int4* tiles,
                           int total_tiles, int nprod, int chunk_kb, int max_ctas, int fmt,
                           int* dev_err, cudaStream_t st) {
  using S = TcShape<NP, BN, tc_wide(NP, TF32)>;
  auto kern = split_tc_kernel<NP, BN, GROUPED, EPI, TF32, FUSED>;
  static std::atomic<uint64_t> attr_done{0};  // per instantiation and device
  constexpr size_t kSmem = FUSED ? S::SMEM_FUSED : S::SMEM;
  static_assert(kSmem <= 232448, "shared memory budget");
  if (!smem_attr_once(kern, kSmem, attr_done)) return UGEMM_ERR_CUDA;
  const int grid = std::max(1, std::min(total_tiles, max_ctas > 0 ? max_ctas : sm_count()));
  prof_begin(st);
  kern<<<grid, FUSED ? fused_threads(BN) : kTcThreads, kSmem, st>>>(
      ta, tb, single, maps, probs, tiles, total_tiles, nprod, chunk_kb, fmt, dev_err);
  prof_end(st, GROUPED ? kProfGrouped : kProfSplitGemm);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

int kp_of(int K) { return static_cast<int>(align_up(std::max(K, 1), kTcKB)); }

}  // namespace

std::vector<int4> split_tile_table(const TcProblem* probs, int nprob, int block_n, int grid,
                                   bool round_robin) {
  std::vector<int4> rec;
  std::vector<int> cost;
  for (int p = 0; p < nprob; ++p) {
    const TcProblem& P = probs[p];
    for (int local = 0; local < P.tiles_m * P.tiles_n; ++local) {
      int m0, n0;
      tc_raster(local, P.tiles_m, P.tiles_n, block_n, m0, n0);
      rec.push_back(make_int4(p, m0, n0, 0));
      // a tile's time: its k-blocks plus about three of fixed cost (pipeline
      // start, final drain, epilogue); narrow tiles are not cheaper, their
      // stages carry the full tile box
      cost.push_back(P.nkb + 3);
    }
  }
  // longest-processing-time first: each tile, longest first, goes to the CTA
  // with the least work so far (measured on the 256-problem group with
  // 256-wide tiles: 135.5 us against 141.3 us dealt round robin)
  std::vector<int> order(rec.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = static_cast<int>(i);
  std::vector<std::vector<int>> lists(grid);
  if (round_robin) {
    for (int i : order) lists[i % grid].push_back(i);
  } else {
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    using Load = std::pair<long long, int>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int c = 0; c < grid; ++c) heap.push({0, c});
    for (int i : order) {
      const Load l = heap.top();
      heap.pop();
      lists[l.second].push_back(i);
      heap.push({l.first + cost[i], l.second});
    }
  }
  std::vector<int4> table(grid + rec.size());
  int next = 0;
  for (int c = 0; c < grid; ++c) {
    table[c] = make_int4(next, next + static_cast<int>(lists[c].size()), 0, 0);
    for (int i : lists[c]) table[grid + next++] = rec[i];
  }
  return table;
}

// Depth of the main accumulator's chunks, in 32-deep k-blocks, for a GEMM
// of depth K (UGEMM_CHUNK_K overrides).  Each chunk is summed in TMEM, whose
// adds truncate, then drained into FP32 registers with round-to-nearest
// adds: shorter chunks are more accurate and cost drains.  Measured on
// GB300: 128 costs nothing against 256 at 8192^3 and takes the error at
// 4096^3 from 3.6e-7 to 2.3e-7; at k <= 1024, where FP32 SIMT's own error is
// smallest (a few products dominate each element when the values span many
// binades), 64 keeps both split forms at or below it for about 5% of time.
int split_default_chunk_kb(int K) {
  static const int forced = [] {
    const char* e = std::getenv("UGEMM_CHUNK_K");
    return e ? std::max(1, std::atoi(e) / kTcKB) : 0;
  }();
  if (forced) return forced;
  // 64 deep up to k = 1024 (where FP32 SIMT's own error is smallest), 128
  // up to 4096, 256 beyond: every chunk start makes the main accumulator
  // wait for a drain, and at 8192^3 halving their number saves 4% of the
  // FP16x3 GEMM for an error of 3.6e-7 instead of 2.4e-7 (FP32 SIMT: 1.6e-6)
  return K <= 1024 ? 2 : (K <= 4096 ? 4 : 8);
}

SplitPlan split_plan_for(int precision, const Gemm& g) {
  SplitPlan p;
  switch (precision) {
    case UGEMM_PREC_BF16X9: p.pieces = 3; p.products = 9; break;
    case UGEMM_PREC_BF16X3: p.pieces = 2; p.products = 3; break;
    case UGEMM_PREC_FP16X3: p.pieces = 2; p.products = 3; p.f16 = true; break;
    case UGEMM_PREC_TF32X3: p.pieces = kPiecesTf32; p.products = 3; break;
    default: p.pieces = 3; p.products = 6; break;
  }
  p.block_n = (g.N > 128) ? 256 : 128;
  p.epi = g.epi.bias != nullptr || g.epi.act != 0;
  return p;
}

size_t split_operand_bytes(int pieces, int rows, int K) {
  return align_up(size_t(piece_planes(pieces)) * rows * kp_of(K) * piece_bytes(pieces), 256) +
         (pieces == 2 ? align_up(size_t(std::max(rows, 1)) * sizeof(unsigned), 256) : 0);
}

unsigned* split_fmax_word(const void* pieces_base, int pieces, int rows, int K) {
  return reinterpret_cast<unsigned*>(const_cast<uint8_t*>(static_cast<const uint8_t*>(pieces_base)) +
                                     align_up(size_t(pieces) * rows * kp_of(K) * 2, 256));
}

size_t split_scratch_bytes(const Gemm& g, const SplitPlan& p) {
  return split_operand_bytes(p.pieces, g.M, g.K) + split_operand_bytes(p.pieces, g.N, g.K) +
         tail_scratch_bytes(g, p);
}

// Boxes of one stage: split_stage_k(pieces) deep, the swizzle as wide as a
// row of the box (128 bytes for TF32 pieces, 64 for 16-bit ones).
CUtensorMapSwizzle split_swizzle(int pieces) {
  return split_stage_k(pieces) * piece_bytes(pieces) == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                                            : CU_TENSOR_MAP_SWIZZLE_64B;
}

CUtensorMapDataType piece_dtype(int pieces) {
  return pieces == kPiecesTf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
}

bool split_encode_view(int pieces, int box_rows, const void* base, int rows, int plane_rows, int K,
                       CUtensorMap* map) {
  const int Kp = kp_of(K), eb = piece_bytes(pieces), np = piece_planes(pieces);
  const uint64_t row = uint64_t(Kp) * eb;
  return encode_tmap_3d(map, piece_dtype(pieces), eb, base, Kp, rows, np, row, row * plane_rows,
                        split_stage_k(pieces), box_rows, np, split_swizzle(pieces));
}

bool split_encode_maps(int pieces, int block_n, const void* ap, int M, const void* bp, int N,
                       int K, CUtensorMap* ta, CUtensorMap* tb) {
  const int Kp = kp_of(K), eb = piece_bytes(pieces), np = piece_planes(pieces);
  const uint64_t row = uint64_t(Kp) * eb;
  const uint32_t kb = split_stage_k(pieces);
  const CUtensorMapSwizzle sw = split_swizzle(pieces);
  const CUtensorMapDataType dt = piece_dtype(pieces);
  return encode_tmap_3d(ta, dt, eb, ap, Kp, M, np, row, row * M, kb, kTcBM, np, sw) &&
         encode_tmap_3d(tb, dt, eb, bp, Kp, N, np, row, row * N, kb, block_n, np, sw);
}

TcProblem split_problem(const Gemm& g, int pieces, int block_n, int tile_start) {
  TcProblem P;
  P.C = g.C;
  P.M = g.M;
  P.N = g.N;
  P.ldc = g.ldc;
  P.alpha = g.alpha;
  P.beta = g.beta;
  P.nkb = split_nkb(pieces, g.K);
  P.tiles_m = cdiv(g.M, kTcBM);
  P.tiles_n = cdiv(g.N, block_n);
  P.tile_start = tile_start;
  P.epi = g.epi;
  return P;
}

// op(A)[m][k]: 'N' -> A[m*lda + k];  'T' -> A[k*lda + m]
// op(B)^T[n][k]: 'N' -> B[k*ldb + n]; 'T' -> B[n*ldb + k]
void split_operand_strides(const Gemm& g, long long* a_sr, long long* a_sk, long long* b_sr,
                           long long* b_sk) {
  *a_sr = g.ta == 'N' ? g.lda : 1;
  *a_sk = g.ta == 'N' ? 1 : g.lda;
  *b_sr = g.tb == 'N' ? 1 : g.ldb;
  *b_sk = g.tb == 'N' ? g.ldb : 1;
}

ugemm_status split_launch(const Gemm& g, const SplitPlan& p, Scratch ws, int* dev_err,
                          cudaStream_t st) {
  if (split_scratch_bytes(g, p) > ws.bytes) return UGEMM_ERR_ARENA_TOO_SMALL;
  // scratch: [A pieces | B pieces | wave-tail partial tiles and table]
  uint8_t* ap = static_cast<uint8_t*>(ws.ptr);
  uint8_t* bp = ap + split_operand_bytes(p.pieces, g.M, g.K);
  uint8_t* tail_scratch = bp + split_operand_bytes(p.pieces, g.N, g.K);
  long long a_sr, a_sk, b_sr, b_sk;
  split_operand_strides(g, &a_sr, &a_sk, &b_sr, &b_sk);
  ugemm_status s = UGEMM_OK;
  if (!p.f16 && g.M > 0 && g.N > 0 && g.K > 0) {
    // both operands in one launch (the FP16x3 split takes row-maximum
    // passes of its own first)
    SplitJobTable jt{};
    const int kp = kp_of(g.K), tk = cdiv(kp, 64), ta = cdiv(g.M, 32) * tk;
    jt.jobs[0] = SplitJob{g.A, a_sr, a_sk, reinterpret_cast<__nv_bfloat16*>(ap), g.M, g.K, kp, 0};
    jt.jobs[1] = SplitJob{g.B, b_sr, b_sk, reinterpret_cast<__nv_bfloat16*>(bp), g.N, g.K, kp, ta};
    s = split_param_launch(p.pieces, jt, 2, ta + cdiv(g.N, 32) * tk, st);
  } else {
    s = split_operand_launch(p.pieces, g.A, a_sr, a_sk, g.M, g.K, ap, st, p.f16);
    if (s == UGEMM_OK) s = split_operand_launch(p.pieces, g.B, b_sr, b_sk, g.N, g.K, bp, st, p.f16);
  }
  if (s != UGEMM_OK) return s;
  return split_gemm_on_pieces(g, p, ap, bp, tail_scratch, dev_err, st);
}

ugemm_status split_gemm_launch(const SplitPlan& p, const CUtensorMap& ta, const CUtensorMap& tb,
                               const TcProblem& single, const CUtensorMap* maps,
                               const TcProblem* probs, const int4* tiles, int total_tiles,
                               int chunk_kb,
                               int max_ctas, int* dev_err, cudaStream_t st) {
  const bool grouped = probs != nullptr;
  if (p.fused) {  // grouped launches of three bf16 pieces only
    if (p.pieces != 3 || !grouped || (p.block_n == 256 && single.chunk_sums == nullptr))
      return UGEMM_ERR_ARG;
#define UGEMM_FUSED_CASE(BN, EPI)                                                                \
  if (p.block_n == BN && p.epi == EPI)                                                          \
    return launch_kernel<3, BN, true, EPI, false, true>(ta, tb, single, maps, probs, tiles,     \
                                                        total_tiles, p.products, chunk_kb,      \
                                                        max_ctas, 0, dev_err, st);
    UGEMM_FUSED_CASE(128, false)
    UGEMM_FUSED_CASE(128, true)
    UGEMM_FUSED_CASE(256, false)
    UGEMM_FUSED_CASE(256, true)
#undef UGEMM_FUSED_CASE
    return UGEMM_ERR_ARG;
  }
  const int fmt = p.f16 ? 1 : 0;
  const bool tf32 = p.pieces == kPiecesTf32;
#define UGEMM_SPLIT_CASE(NP, BN, GR, EPI, T)                                                     \
  if (kernel_np(p.pieces) == NP && p.block_n == BN && grouped == GR && p.epi == EPI && tf32 == T) \
    return launch_kernel<NP, BN, GR, EPI, T>(ta, tb, single, maps, probs, tiles, total_tiles,     \
                                             p.products, chunk_kb, max_ctas, fmt, dev_err, st);
#define UGEMM_SPLIT_CASES(NP, BN, T)    \
  UGEMM_SPLIT_CASE(NP, BN, false, false, T) \
  UGEMM_SPLIT_CASE(NP, BN, false, true, T)  \
  UGEMM_SPLIT_CASE(NP, BN, true, false, T)  \
  UGEMM_SPLIT_CASE(NP, BN, true, true, T)
  UGEMM_SPLIT_CASES(3, 256, false)
  UGEMM_SPLIT_CASES(3, 128, false)
  UGEMM_SPLIT_CASES(2, 256, false)
  UGEMM_SPLIT_CASES(2, 128, false)
  UGEMM_SPLIT_CASES(2, 256, true)
  UGEMM_SPLIT_CASES(2, 128, true)
#undef UGEMM_SPLIT_CASES
#undef UGEMM_SPLIT_CASE
  return UGEMM_ERR_ARG;
}

ugemm_status split_batched_launch(int pieces, const SplitJob* jobs, int njobs, int total_tiles,
                                  cudaStream_t st, unsigned* fmax_words, int nwords) {
  if (total_tiles <= 0) return UGEMM_OK;
  const int grid = std::min(total_tiles, sm_count() * 8);
  if (fmax_words) {  // FP16x3: the largest magnitude of every job's rows first
    if (pieces != 2) return UGEMM_ERR_ARG;
    if (cudaMemsetAsync(fmax_words, 0, sizeof(unsigned) * nwords, st) != cudaSuccess)
      return UGEMM_ERR_CUDA;
    prof_begin(st);
    operand_max_batched_kernel<<<grid, 256, 0, st>>>(jobs, njobs, total_tiles);
    prof_end(st, kProfSplitPrep);
    prof_begin(st);
    split_pieces_batched_kernel<2, 1><<<grid, 256, 0, st>>>(jobs, njobs, total_tiles);
    prof_end(st, kProfSplitPrep);
    return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
  }
  prof_begin(st);
  if (pieces == 3) split_pieces_batched_kernel<3, 0><<<grid, 256, 0, st>>>(jobs, njobs, total_tiles);
  else if (pieces == kPiecesTf32) split_pieces_batched_kernel<2, 2><<<grid, 256, 0, st>>>(jobs, njobs, total_tiles);
  else split_pieces_batched_kernel<2, 0><<<grid, 256, 0, st>>>(jobs, njobs, total_tiles);
  prof_end(st, kProfSplitPrep);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

ugemm_status split_param_launch(int pieces, const SplitJobTable& t, int njobs, int total_tiles,
                                cudaStream_t st) {
  if (total_tiles <= 0) return UGEMM_OK;
  if (njobs < 1 || njobs > kSplitTableJobs) return UGEMM_ERR_ARG;
  const int grid = std::min(total_tiles, sm_count() * 8);
  prof_begin(st);
  if (pieces == 3) split_pieces_param_kernel<3, 0><<<grid, 256, 0, st>>>(t, njobs, total_tiles);
  else if (pieces == kPiecesTf32) split_pieces_param_kernel<2, 2><<<grid, 256, 0, st>>>(t, njobs, total_tiles);
  else if (pieces == 2) split_pieces_param_kernel<2, 0><<<grid, 256, 0, st>>>(t, njobs, total_tiles);
  else { prof_end(st, kProfSplitPrep); return UGEMM_ERR_ARG; }
  prof_end(st, kProfSplitPrep);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

int split_kp(int K) { return kp_of(K); }

bool fused_encode_map(const float* base, long long ld, int R, int Cc, bool kcontig, int box_rows,
                      int box_k, CUtensorMap* map) {
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld & 3) || R < 1 || Cc < 1) return false;
  if (box_k != kTcKB && box_k != kTcKB / 2) return false;
  // the stored matrix: R rows of Cc floats; the box is box_k k by box_rows
  // rows of the kernel operand, k along the columns (kcontig: rows of
  // 4 * box_k bytes, swizzled over that width) or along the rows
  return kcontig ? encode_tmap_2d(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, Cc, R, ld * 4ull,
                                  box_k, box_rows,
                                  box_k == kTcKB ? CU_TENSOR_MAP_SWIZZLE_128B
                                                 : CU_TENSOR_MAP_SWIZZLE_64B)
                 : encode_tmap_2d(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, Cc, R, ld * 4ull,
                                  box_rows, box_k, CU_TENSOR_MAP_SWIZZLE_NONE);
}

}  // namespace ugemm

namespace ugemm {

// Split one operand (element (r, k) at src[r*sr + k*sk]) into its planes
// [planes][rows][Kp] of pieces at dst (layout code `pieces`).
ugemm_status split_operand_launch(int pieces, const float* src, long long sr, long long sk,
                                  int rows, int K, void* dst, cudaStream_t st, bool f16) {
  const int Kp = kp_of(K);
  auto* d = static_cast<__nv_bfloat16*>(dst);
  if (f16) {
    if (pieces != 2) return UGEMM_ERR_ARG;
    unsigned* words = split_fmax_word(dst, 2, rows, K);
    if (sk == 1 && rows > 0 && K > 0 && Kp <= kRowSplitK &&
        (reinterpret_cast<uintptr_t>(src) & 15) == 0 && (sr & 3) == 0) {
      // rows contiguous in k: maximum and split in one pass over the operand
      prof_begin(st);
      split_rows_f16_kernel<<<rows, 256, 0, st>>>(src, sr, K, Kp, d, rows, words);
      prof_end(st, kProfSplitPrep);
      return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
    }
    if (cudaMemsetAsync(words, 0, sizeof(unsigned) * std::max(rows, 1), st) != cudaSuccess)
      return UGEMM_ERR_CUDA;
    if (rows > 0 && K > 0) {
      // row bands x runs of k, about eight blocks per SM
      const bool kcontig = sk == 1;
      const long long other = kcontig ? sr : sk;
      const bool vec = ((reinterpret_cast<uintptr_t>(src) & 15) == 0) && ((other & 3) == 0);
      const int band = kcontig ? 16 : 256, bands = cdiv(rows, band);
      const int want_y = std::max(1, std::min(cdiv(K, 256), cdiv(sm_count() * 8, bands)));
      const int kper = static_cast<int>(align_up(cdiv(K, want_y), 64));
      const dim3 grid(bands, cdiv(K, kper));
      prof_begin(st);
      if (kcontig) {
        if (vec) operand_row_max_kernel<true, true><<<grid, 256, 0, st>>>(src, sr, sk, rows, K, kper, words);
        else operand_row_max_kernel<true, false><<<grid, 256, 0, st>>>(src, sr, sk, rows, K, kper, words);
      } else if (sr == 1) {
        if (vec) operand_row_max_kernel<false, true><<<grid, 256, 0, st>>>(src, sr, sk, rows, K, kper, words);
        else operand_row_max_kernel<false, false><<<grid, 256, 0, st>>>(src, sr, sk, rows, K, kper, words);
      } else {  // neither layout contiguous (not produced by the callers): the tiled reduction
        SplitJob j{src, sr, sk, d, rows, K, Kp, 0};
        j.fmax = words;
        const int tiles = cdiv(rows, 32) * cdiv(Kp, 64);
        j.tile_start = 0;
        operand_max_single_kernel<<<std::min(tiles, sm_count() * 8), 256, 0, st>>>(j, tiles);
      }
      prof_end(st, kProfSplitPrep);
    }
    launch_split<2, 1>(src, sr, sk, rows, K, Kp, d, st, words);
  } else if (pieces == 3) {
    launch_split<3, 0>(src, sr, sk, rows, K, Kp, d, st);
  } else if (pieces == kPiecesTf32) {
    launch_split<2, 2>(src, sr, sk, rows, K, Kp, d, st);
  } else {
    launch_split<2, 0>(src, sr, sk, rows, K, Kp, d, st);
  }
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

// GEMM on pieces already split: C = alpha * A*B^T-pieces + beta * C.
ugemm_status split_gemm_on_pieces(const Gemm& g, const SplitPlan& p, const void* a_pieces,
                                  const void* b_pieces, void* tail_scratch, int* dev_err,
                                  cudaStream_t st) {
  CUtensorMap ta, tb;
  if (!split_encode_maps(p.pieces, p.block_n, a_pieces, g.M, b_pieces, g.N, g.K, &ta, &tb))
    return UGEMM_ERR_CUDA;
  TcProblem P = split_problem(g, p.pieces, p.block_n, 0);
  if (p.f16) {
    P.fmax_a = split_fmax_word(a_pieces, 2, g.M, g.K);
    P.fmax_b = split_fmax_word(b_pieces, 2, g.N, g.K);
  }
  const int chunk =
      split_chunk_stages(p.pieces, p.chunk_kb > 0 ? p.chunk_kb : split_default_chunk_kb(g.K));
  // a partial last wave of tiles runs as two k slices (multi.cu)
  const TailPlan tail = tail_scratch ? tail_plan(g, p) : TailPlan{};
  ugemm_status s = split_gemm_launch(p, ta, tb, P, nullptr, nullptr, nullptr,
                                     tail.use ? tail.main_tiles : P.tiles_m * P.tiles_n, chunk, 0,
                                     dev_err, st);
  if (s != UGEMM_OK || !tail.use) return s;
  return tail_launch(g, p, tail, a_pieces, b_pieces, tail_scratch, dev_err, st);
}

}  // namespace ugemm
