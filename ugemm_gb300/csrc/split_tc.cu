// split_tc.cu -- split-precision SGEMM on the 5th-generation tensor cores
// (the "precision" form; no counterpart in the reference, whose only GPU
// kernels are the FP32 OpenCL/GLSL ones).
//
// Each FP32 operand element x is written as a sum of bf16 pieces
//     x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1)
// which is exact for three pieces (8+8+8 significand bits cover FP32's 24).
// C = alpha * sum over piece products (ai, bj) of A_i * B_j + beta * C, with
// every piece product computed by tcgen05.mma (kind::f16, bf16 x bf16 ->
// FP32 accumulate in TMEM):
//     BF16x9: all nine products            (products exact, FP32 accumulate)
//     BF16x6: drop a1b2, a2b1, a2b2        (each ~2^-24 relative)
//     BF16x3: two pieces, a0b0+a0b1+a1b0   (~2^-16 relative; for studies)
//
// Pipeline:
//   1. split kernel (one HBM pass per operand): reads op(A) / op(B) in any
//      transpose and leading dimension, writes the pieces as K-major bf16
//      planes [pieces][rows][Kp] (Kp = K rounded up to 32, zero padded);
//   2. GEMM kernel, one CTA per 128 x BN tile of C, 6 warps:
//        warp 0  TMA producer: one 3-D TMA per operand per stage brings all
//                pieces of a 32-deep k slice (64-byte swizzle) into a
//                3-4 stage ring (mbarrier full/empty pairs);
//        warp 1  allocates TMEM (BN fp32 columns) and, from one thread,
//                issues the tcgen05.mma stream; tcgen05.commit frees stages;
//        warps 2-5  epilogue: tcgen05.ld the 128 x BN accumulator (one TMEM
//                lane per row), alpha/beta, store C (guarded for ragged M, N).
// All mbarrier waits are bounded (ptx.cuh); on a timeout the kernel records
// an error, skips its remaining work and still frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"
#include "ptx.cuh"

namespace ugemm {
namespace {

constexpr int kBM = 128;        // rows of C per CTA (UMMA M)
constexpr int kKB = 32;         // k depth of one stage (bf16: 64 bytes per row)
constexpr int kRowBytes = kKB * 2;
constexpr int kThreads = 192;   // 6 warps
constexpr int kRaster = 8;

// Piece products in issue order, encoded (ia << 2) | ib.
__constant__ uint8_t kProducts[9] = {0x0, 0x1, 0x4, 0x2, 0x5, 0x8, 0x6, 0x9, 0xA};

template <int NP, int BN>
struct TcShape {
  static constexpr int A_PLANE = kBM * kRowBytes;   // bytes of one A piece tile
  static constexpr int B_PLANE = BN * kRowBytes;
  static constexpr int A_BYTES = NP * A_PLANE;
  static constexpr int B_BYTES = NP * B_PLANE;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int STAGES = (220 * 1024) / STAGE_BYTES > 4 ? 4 : (220 * 1024) / STAGE_BYTES;
  static constexpr size_t SMEM = 1024 + size_t(STAGES) * STAGE_BYTES + 256;
  static_assert(STAGES >= 2, "pipeline needs two stages");
};

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

template <int NP, int BN>
__global__ void __launch_bounds__(kThreads, 1)
    split_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    float* __restrict__ C, int M, int N, int ldc, float alpha, float beta, int nkb,
                    int nprod, int tiles_m, int tiles_n, int* err) {
  using S = TcShape<NP, BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S::STAGES * S::STAGE_BYTES);
  uint64_t* empty = full + S::STAGES;
  uint64_t* accum = empty + S::STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);

  const int b = blockIdx.x;
  const int per_group = kRaster * tiles_n;
  const int first_m = (b / per_group) * kRaster;
  const int group_rows = min(tiles_m - first_m, kRaster);
  const int tile_m = first_m + (b % per_group) % group_rows;
  const int tile_n = (b % per_group) / group_rows;
  const int m0 = tile_m * kBM, n0 = tile_n * BN;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    fence_barrier_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, BN);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      int issued = 0;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % S::STAGES;
        const uint32_t ph = (kb / S::STAGES) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1, err, kDevTimeoutEmpty)) break;
        uint8_t* sa = smem + s * S::STAGE_BYTES;
        mbar_arrive_expect_tx(&full[s], S::STAGE_BYTES);
        tma_load_3d(sa, &tmA, &full[s], kb * kKB, m0, 0);
        tma_load_3d(sa + S::A_BYTES, &tmB, &full[s], kb * kKB, n0, 0);
        issued = kb + 1;
      }
      // After a fault elsewhere, let in-flight copies land before exit.
      if (issued < nkb && issued > 0) {
        for (int kb = max(0, issued - S::STAGES); kb < issued; ++kb)
          mbar_wait(&full[kb % S::STAGES], (kb / S::STAGES) & 1, nullptr, 0);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = umma_idesc(1, 1, kBM, BN);
      const uint32_t a_base = smem_u32(smem);
      uint32_t acc_flag = 0;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % S::STAGES;
        const uint32_t ph = (kb / S::STAGES) & 1;
        if (!mbar_wait(&full[s], ph, err, kDevTimeoutFull)) break;
        tc_fence_after();
        const uint32_t sa = a_base + s * S::STAGE_BYTES;
        const uint32_t sb = sa + S::A_BYTES;
        for (int p = 0; p < nprod; ++p) {
          const uint32_t code = kProducts[p];
          const uint32_t ia = code >> 2, ib = code & 3;
#pragma unroll
          for (int kk = 0; kk < kKB / 16; ++kk) {
            const uint64_t ad = umma_smem_desc(sa + ia * S::A_PLANE + kk * 32, 512, 4);
            const uint64_t bd = umma_smem_desc(sb + ib * S::B_PLANE + kk * 32, 512, 4);
            umma_bf16(tmem, ad, bd, idesc, acc_flag);
            acc_flag = 1;
          }
        }
        umma_commit(&empty[s]);
      }
      umma_commit(accum);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ epilogue warps 2..5
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int row = m0 + q * 32 + lane;
    const bool wait_ok = __all_sync(0xffffffffu, mbar_wait(accum, 0, err, kDevTimeoutAccum));
    tc_fence_after();
    if (wait_ok) {  // warp-uniform: tcgen05.ld is .sync.aligned
      const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
      float* crow = C + static_cast<size_t>(row) * ldc;
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        uint32_t r[32];
        tmem_ld_32x32b_x32(tmem + (static_cast<uint32_t>(q * 32) << 16) + c * 32, r);
        tmem_ld_wait();
        if (row < M) {
          const int col0 = n0 + c * 32;
          if (vec && col0 + 32 <= N) {
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
              float4 v = make_float4(alpha * __uint_as_float(r[j]), alpha * __uint_as_float(r[j + 1]),
                                     alpha * __uint_as_float(r[j + 2]),
                                     alpha * __uint_as_float(r[j + 3]));
              if (beta != 0.f) {
                const float4 o = *reinterpret_cast<const float4*>(crow + col0 + j);
                v.x += beta * o.x; v.y += beta * o.y; v.z += beta * o.z; v.w += beta * o.w;
              }
              *reinterpret_cast<float4*>(crow + col0 + j) = v;
            }
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (col0 + j < N) {
                float v = alpha * __uint_as_float(r[j]);
                if (beta != 0.f) v += beta * crow[col0 + j];
                crow[col0 + j] = v;
              }
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, BN);
  }
}

// Split op(X) (rows x K, element (r, k) at src[r*sr + k*sk]) into NP bf16
// planes dst[p][rows][Kp], K-major, zero for k >= K.  One block: 32 rows x
// 64 k through shared memory, so both source layouts read coalesced.
template <int NP>
__global__ void __launch_bounds__(256) split_pieces_kernel(const float* __restrict__ src,
                                                           long long sr, long long sk, int rows,
                                                           int K, int Kp,
                                                           __nv_bfloat16* __restrict__ dst) {
  __shared__ float tile[32][65];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 64;
  const int t = threadIdx.x;
  if (sk == 1) {
    const int k = k0 + (t & 63);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int rr = (t >> 6) + 4 * i, r = r0 + rr;
      tile[rr][t & 63] = (r < rows && k < K) ? src[r * sr + k] : 0.f;
    }
  } else {
    const int rr = t & 31, r = r0 + rr;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int kk = (t >> 5) + 8 * i, k = k0 + kk;
      tile[rr][kk] = (r < rows && k < K) ? src[r * sr + k * sk] : 0.f;
    }
  }
  __syncthreads();
  const int kp = t & 31;  // k pair within the tile
  const int k = k0 + 2 * kp;
  if (k >= Kp) return;
  const size_t plane = static_cast<size_t>(rows) * Kp;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rr = (t >> 5) + 8 * i, r = r0 + rr;
    if (r >= rows) continue;
    float x[2] = {tile[rr][2 * kp], tile[rr][2 * kp + 1]};
    __nv_bfloat16 pc[3][2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      float rem = x[e];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        pc[p][e] = __float2bfloat16_rn(rem);
        rem = rem - __bfloat162float(pc[p][e]);
      }
    }
    const size_t off = static_cast<size_t>(r) * Kp + k;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      __nv_bfloat162 v;
      v.x = pc[p][0];
      v.y = pc[p][1];
      *reinterpret_cast<__nv_bfloat162*>(dst + p * plane + off) = v;
    }
  }
}

int kp_of(int K) { return static_cast<int>(align_up(std::max(K, 1), kKB)); }

template <int NP>
void launch_split(const float* src, long long sr, long long sk, int rows, int K, int Kp,
                  __nv_bfloat16* dst, cudaStream_t st) {
  dim3 grid(cdiv(Kp, 64), cdiv(rows, 32));
  prof_begin(st);
  split_pieces_kernel<NP><<<grid, 256, 0, st>>>(src, sr, sk, rows, K, Kp, dst);
  prof_end(st, kProfSplitPrep);
}

template <int NP, int BN>
ugemm_status launch_gemm(const Gemm& g, int nprod, const __nv_bfloat16* ap,
                         const __nv_bfloat16* bp, int Kp, int* dev_err, cudaStream_t st) {
  using S = TcShape<NP, BN>;
  CUtensorMap ta, tb;
  const uint64_t row = uint64_t(Kp) * 2;
  if (!encode_tmap_3d(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ap, Kp, g.M, NP, row, row * g.M,
                      kKB, kBM, NP, CU_TENSOR_MAP_SWIZZLE_64B))
    return UGEMM_ERR_CUDA;
  if (!encode_tmap_3d(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, bp, Kp, g.N, NP, row, row * g.N,
                      kKB, BN, NP, CU_TENSOR_MAP_SWIZZLE_64B))
    return UGEMM_ERR_CUDA;
  auto kern = split_tc_kernel<NP, BN>;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(S::SMEM)) != cudaSuccess)
      return UGEMM_ERR_CUDA;
    attr_set = true;
  }
  const int tiles_m = cdiv(g.M, kBM), tiles_n = cdiv(g.N, BN);
  prof_begin(st);
  kern<<<tiles_m * tiles_n, kThreads, S::SMEM, st>>>(ta, tb, g.C, g.M, g.N, g.ldc, g.alpha, g.beta,
                                                      Kp / kKB, nprod, tiles_m, tiles_n, dev_err);
  prof_end(st, kProfSplitGemm);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace

SplitPlan split_plan_for(int precision, const Gemm& g) {
  SplitPlan p;
  switch (precision) {
    case UGEMM_PREC_BF16X9: p.pieces = 3; p.products = 9; break;
    case UGEMM_PREC_BF16X3: p.pieces = 2; p.products = 3; break;
    default: p.pieces = 3; p.products = 6; break;
  }
  p.block_n = (g.N > 128) ? 256 : 128;
  return p;
}

size_t split_scratch_bytes(const Gemm& g, const SplitPlan& p) {
  const size_t kp = kp_of(g.K);
  return align_up(size_t(p.pieces) * g.M * kp * 2, 256) + align_up(size_t(p.pieces) * g.N * kp * 2, 256);
}

ugemm_status split_launch(const Gemm& g, const SplitPlan& p, Scratch ws, int* dev_err,
                          cudaStream_t st) {
  const int Kp = kp_of(g.K);
  const size_t a_bytes = align_up(size_t(p.pieces) * g.M * Kp * 2, 256);
  if (split_scratch_bytes(g, p) > ws.bytes) return UGEMM_ERR_ARENA_TOO_SMALL;
  auto* ap = static_cast<__nv_bfloat16*>(ws.ptr);
  auto* bp = reinterpret_cast<__nv_bfloat16*>(static_cast<uint8_t*>(ws.ptr) + a_bytes);
  // op(A)[m][k]:  'N' -> A[m*lda + k];  'T' -> A[k*lda + m]
  const long long a_sr = g.ta == 'N' ? g.lda : 1, a_sk = g.ta == 'N' ? 1 : g.lda;
  // op(B)^T[n][k]: 'N' -> B[k*ldb + n]; 'T' -> B[n*ldb + k]
  const long long b_sr = g.tb == 'N' ? 1 : g.ldb, b_sk = g.tb == 'N' ? g.ldb : 1;
  if (p.pieces == 3) {
    launch_split<3>(g.A, a_sr, a_sk, g.M, g.K, Kp, ap, st);
    launch_split<3>(g.B, b_sr, b_sk, g.N, g.K, Kp, bp, st);
    if (p.block_n == 256) return launch_gemm<3, 256>(g, p.products, ap, bp, Kp, dev_err, st);
    return launch_gemm<3, 128>(g, p.products, ap, bp, Kp, dev_err, st);
  }
  launch_split<2>(g.A, a_sr, a_sk, g.M, g.K, Kp, ap, st);
  launch_split<2>(g.B, b_sr, b_sk, g.N, g.K, Kp, bp, st);
  if (p.block_n == 256) return launch_gemm<2, 256>(g, p.products, ap, bp, Kp, dev_err, st);
  return launch_gemm<2, 128>(g, p.products, ap, bp, Kp, dev_err, st);
}

}  // namespace ugemm
