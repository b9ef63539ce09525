// simt.cu -- plain FP32 SIMT SGEMM for sm_103a (the "plain" form).
//
// Replaces the reference's OpenCL gemm_rnn (sgemm_ocl2.h:17-90: 16x16 tile,
// one output per work-item, two local-memory loads per FMA) and its separate
// transpose pass (sgemm_ocl2.h:95-128, :180-199).  Here:
//   * one CTA computes a BM x BN tile of C; 8 consumer warps (16 x 16 threads)
//     each hold a TM x TN register block; a ninth warp is the TMA producer;
//   * A and B k-slices (BK = 32) are staged by TMA into a 4-deep shared-memory
//     ring guarded by mbarriers; k-contiguous tiles use the 128-byte swizzle
//     so the float4 fragment reads are bank-conflict free;
//   * transposed operands are handled by the tile layout (an m- or
//     n-contiguous tile) -- no transpose kernel, no extra HBM pass;
//   * ragged edges: TMA zero-fills out-of-range rows/columns/k, the epilogue
//     guards its stores; alpha/beta are fused into the epilogue and C is not
//     read when beta == 0 (sgemm_ocl2.h:86-88).
// Operands whose base or leading dimension break TMA's 16-byte rules are
// first copied into an aligned scratch buffer (simt_scratch_bytes).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "internal.h"
#include "ptx.cuh"
#include "simt.cuh"

namespace ugemm {
namespace {

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Position of the 16-byte chunk `q` of row `r` in a 128-byte-row tile written
// by TMA with CU_TENSOR_MAP_SWIZZLE_128B (address bits [4,7) ^= bits [7,10)).
__device__ __forceinline__ int swz_chunk(int r, int q) { return q ^ (r & 7); }

// One BM x BN tile's k loop, consuming the TMA ring from stage counter `it`
// (which keeps running across the tiles of a persistent CTA).  AK: op(A) rows
// are k-contiguous (ta == 'N').  BKM: op(B) columns are k-contiguous (tb == 'T').
template <int TM, int TN, bool AK, bool BKM>
__device__ __forceinline__ bool simt_mainloop(const uint8_t* smem, uint64_t* full, uint64_t* empty,
                                              int nkt, uint32_t& it, float (&acc)[TM][TN],
                                              int* err) {
  using S = SimtShape<TM, TN>;
  constexpr int BM = S::BM, BN = S::BN;
  const int tid = threadIdx.x, lane = tid & 31;
  const int ty = tid >> 4, tx = tid & 15;
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
  for (int kt = 0; kt < nkt; ++kt, ++it) {
    const int s = it % kStages;
    const uint32_t ph = (it / kStages) & 1;
    if (!mbar_wait(&full[s], ph, err, kDevTimeoutFull)) return false;
    const float* As = reinterpret_cast<const float*>(smem + s * S::STAGE_BYTES);
    const float* Bs = reinterpret_cast<const float*>(smem + s * S::STAGE_BYTES + S::A_BYTES);
#pragma unroll
    for (int q = 0; q < kBK / 4; ++q) {
      float a[TM][4], bf[TN][4];
      if (AK) {  // As[BM][32], 128-byte swizzled rows; thread rows ty + 16 i
#pragma unroll
        for (int i = 0; i < TM; ++i) {
          const int r = ty + 16 * i;
          const float4 v = *reinterpret_cast<const float4*>(As + r * kBK + 4 * swz_chunk(r, q));
          a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; a[i][3] = v.w;
        }
      } else {   // As[32][BM]; thread rows 64 g + 4 ty + {0..3}
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int g = 0; g < TM / 4; ++g) {
            const float4 v =
                *reinterpret_cast<const float4*>(As + (4 * q + kk) * BM + 64 * g + 4 * ty);
            a[4 * g + 0][kk] = v.x; a[4 * g + 1][kk] = v.y;
            a[4 * g + 2][kk] = v.z; a[4 * g + 3][kk] = v.w;
          }
      }
      if (BKM) {  // Bs[BN][32], 128-byte swizzled rows; thread cols tx + 16 j
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          const int c = tx + 16 * j;
          const float4 v = *reinterpret_cast<const float4*>(Bs + c * kBK + 4 * swz_chunk(c, q));
          bf[j][0] = v.x; bf[j][1] = v.y; bf[j][2] = v.z; bf[j][3] = v.w;
        }
      } else {    // Bs[32][BN]; thread cols 64 g + 4 tx + {0..3}
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int g = 0; g < TN / 4; ++g) {
            const float4 v =
                *reinterpret_cast<const float4*>(Bs + (4 * q + kk) * BN + 64 * g + 4 * tx);
            bf[4 * g + 0][kk] = v.x; bf[4 * g + 1][kk] = v.y;
            bf[4 * g + 2][kk] = v.z; bf[4 * g + 3][kk] = v.w;
          }
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i][kk], bf[j][kk], acc[i][j]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  return true;
}

// One k-slice (kBK deep) of the register-blocked product, consumed from a
// staged tile pair.  k-contiguous operands are read as float4 of 4 k; the
// other layout is read per k so only TN (or TM) values are live at a time.
template <int TM, int TN, bool AK, bool BKM>
__device__ __forceinline__ void simt_consume(const float* As, const float* Bs, float (&acc)[TM][TN]) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
#pragma unroll
  for (int q = 0; q < kBK / 4; ++q) {
    float a[TM][4], bq[BKM ? TN : 1][4];
    if (AK) {
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int r = ty + 16 * i;
        const float4 v = *reinterpret_cast<const float4*>(As + r * kBK + 4 * swz_chunk(r, q));
        a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; a[i][3] = v.w;
      }
    }
    if (BKM) {
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int c = tx + 16 * j;
        const float4 v = *reinterpret_cast<const float4*>(Bs + c * kBK + 4 * swz_chunk(c, q));
        bq[j][0] = v.x; bq[j][1] = v.y; bq[j][2] = v.z; bq[j][3] = v.w;
      }
    }
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      float av[TM], bv[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) av[i] = AK ? a[i][kk] : 0.f;
      if (!AK) {
#pragma unroll
        for (int g = 0; g < TM / 4; ++g) {
          const float4 v = *reinterpret_cast<const float4*>(As + (4 * q + kk) * BM + 64 * g + 4 * ty);
          av[4 * g] = v.x; av[4 * g + 1] = v.y; av[4 * g + 2] = v.z; av[4 * g + 3] = v.w;
        }
      }
      if (BKM) {
#pragma unroll
        for (int j = 0; j < TN; ++j) bv[j] = bq[j][kk];
      } else {
#pragma unroll
        for (int g = 0; g < TN / 4; ++g) {
          const float4 v = *reinterpret_cast<const float4*>(Bs + (4 * q + kk) * BN + 64 * g + 4 * tx);
          bv[4 * g] = v.x; bv[4 * g + 1] = v.y; bv[4 * g + 2] = v.z; bv[4 * g + 3] = v.w;
        }
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
  }
}

// alpha/beta epilogue of one tile from registers; C is not read when beta == 0.
template <int TM, int TN, bool AK, bool BKM>
__device__ __forceinline__ void simt_store(const float (&acc)[TM][TN], float* C, int M, int N,
                                           int ldc, float alpha, float beta, int m0, int n0,
                                           const Epilogue& epi) {
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int row = m0 + (AK ? ty + 16 * i : 64 * (i / 4) + 4 * ty + (i % 4));
    if (row >= M) continue;
    float* crow = C + static_cast<size_t>(row) * ldc;
    if (BKM) {
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int col = n0 + tx + 16 * j;
        if (col < N) {
          float v = alpha * acc[i][j];
          if (beta != 0.f) v += beta * crow[col];
          crow[col] = epilogue_apply(v, epi, row);
        }
      }
    } else {
#pragma unroll
      for (int g = 0; g < TN / 4; ++g) {
        const int col = n0 + 64 * g + 4 * tx;
        if (vec && col + 3 < N) {
          float4 v = make_float4(alpha * acc[i][4 * g], alpha * acc[i][4 * g + 1],
                                 alpha * acc[i][4 * g + 2], alpha * acc[i][4 * g + 3]);
          if (beta != 0.f) {
            const float4 o = *reinterpret_cast<const float4*>(crow + col);
            v.x += beta * o.x; v.y += beta * o.y; v.z += beta * o.z; v.w += beta * o.w;
          }
          v.x = epilogue_apply(v.x, epi, row); v.y = epilogue_apply(v.y, epi, row);
          v.z = epilogue_apply(v.z, epi, row); v.w = epilogue_apply(v.w, epi, row);
          *reinterpret_cast<float4*>(crow + col) = v;
        } else {
#pragma unroll
          for (int jj = 0; jj < 4; ++jj)
            if (col + jj < N) {
              float v = alpha * acc[i][4 * g + jj];
              if (beta != 0.f) v += beta * crow[col + jj];
              crow[col + jj] = epilogue_apply(v, epi, row);
            }
        }
      }
    }
  }
}

__device__ __forceinline__ void raster_tile(int local, int tiles_m, int tiles_n, int& tile_m,
                                            int& tile_n) {
  const int per_group = kRaster * tiles_n;
  const int first_m = (local / per_group) * kRaster;
  const int group_rows = min(tiles_m - first_m, kRaster);
  tile_m = first_m + (local % per_group) % group_rows;
  tile_n = (local % per_group) / group_rows;
}

template <int TM, int TN, bool AK, bool BKM>
__global__ void __launch_bounds__(kThreads, 1)
    simt_sgemm_kernel(const __grid_constant__ CUtensorMap tmA,
                      const __grid_constant__ CUtensorMap tmB, float* __restrict__ C, int M,
                      int N, int K, int ldc, float alpha, float beta, Epilogue epi, int tiles_m,
                      int tiles_n, int* err) {
  using S = SimtShape<TM, TN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * S::STAGE_BYTES);
  uint64_t* empty = full + kStages;
  int tile_m, tile_n;
  raster_tile(blockIdx.x, tiles_m, tiles_n, tile_m, tile_n);
  const int m0 = tile_m * S::BM, n0 = tile_n * S::BN;
  const int nkt = (K + kBK - 1) / kBK;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    fence_barrier_init();
  }
  __syncthreads();

  if (warp == kConsumerWarps) {  // ---------------- TMA producer warp
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      for (int kt = 0; kt < nkt; ++kt) {
        const int s = kt % kStages;
        const uint32_t ph = (kt / kStages) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1, err, kDevTimeoutEmpty)) break;
        uint8_t* sa = smem + s * S::STAGE_BYTES;
        uint8_t* sb = sa + S::A_BYTES;
        mbar_arrive_expect_tx(&full[s], S::STAGE_BYTES);
        if (AK) tma_load_2d(sa, &tmA, &full[s], kt * kBK, m0);
        else    tma_load_2d(sa, &tmA, &full[s], m0, kt * kBK);
        if (BKM) tma_load_2d(sb, &tmB, &full[s], kt * kBK, n0);
        else     tma_load_2d(sb, &tmB, &full[s], n0, kt * kBK);
      }
    }
    return;
  }
  float acc[TM][TN];
  uint32_t it = 0;
  if (!simt_mainloop<TM, TN, AK, BKM>(smem, full, empty, nkt, it, acc, err)) return;
  simt_store<TM, TN, AK, BKM>(acc, C, M, N, ldc, alpha, beta, m0, n0, epi);
}

// Producer-less variant: 8 warps only.  With no ninth warp every thread may
// hold up to 255 registers (a ninth warp caps each scheduler's share at 168),
// room for the 8 x 16 register block that halves shared-memory wavefronts per
// FMA.  Thread 0 issues the TMA for stage kt + S - 1 once all warps released
// the stage they consumed at kt - 1.
template <int TM, int TN, bool AK, bool BKM>
__global__ void __launch_bounds__(kConsumerWarps * 32, 1)
    simt_sgemm_np_kernel(const __grid_constant__ CUtensorMap tmA,
                         const __grid_constant__ CUtensorMap tmB, float* __restrict__ C, int M,
                         int N, int K, int ldc, float alpha, float beta, Epilogue epi,
                         int tiles_m, int tiles_n, int* err) {
  using S = SimtShape<TM, TN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * S::STAGE_BYTES);
  uint64_t* empty = full + kStages;
  int tile_m, tile_n;
  raster_tile(blockIdx.x, tiles_m, tiles_n, tile_m, tile_n);
  const int m0 = tile_m * S::BM, n0 = tile_n * S::BN;
  const int nkt = (K + kBK - 1) / kBK;
  const int tid = threadIdx.x, lane = tid & 31;
  auto issue = [&](int kt) {
    const int s = kt % kStages;
    uint8_t* sa = smem + s * S::STAGE_BYTES;
    uint8_t* sb = sa + S::A_BYTES;
    mbar_arrive_expect_tx(&full[s], S::STAGE_BYTES);
    if (AK) tma_load_2d(sa, &tmA, &full[s], kt * kBK, m0);
    else    tma_load_2d(sa, &tmA, &full[s], m0, kt * kBK);
    if (BKM) tma_load_2d(sb, &tmB, &full[s], kt * kBK, n0);
    else     tma_load_2d(sb, &tmB, &full[s], n0, kt * kBK);
  };
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    fence_barrier_init();
    tma_prefetch_desc(&tmA);
    tma_prefetch_desc(&tmB);
    for (int kt = 0; kt < min(kStages - 1, nkt); ++kt) issue(kt);  // first use of each stage
  }
  __syncthreads();
  float acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
  for (int kt = 0; kt < nkt; ++kt) {
    if (tid == 0) {
      const int kn = kt + kStages - 1;
      if (kn < nkt) {
        if (!mbar_wait(&empty[kn % kStages], ((kn / kStages) & 1) ^ 1, err, kDevTimeoutEmpty))
          return;
        issue(kn);
      }
    }
    const int s = kt % kStages;
    if (!mbar_wait(&full[s], (kt / kStages) & 1, err, kDevTimeoutFull)) return;
    const float* As = reinterpret_cast<const float*>(smem + s * S::STAGE_BYTES);
    const float* Bs = reinterpret_cast<const float*>(smem + s * S::STAGE_BYTES + S::A_BYTES);
    simt_consume<TM, TN, AK, BKM>(As, Bs, acc);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  simt_store<TM, TN, AK, BKM>(acc, C, M, N, ldc, alpha, beta, m0, n0, epi);
}

// Persistent grouped SIMT GEMM: one CTA per SM walks the tiles of all
// problems.  The batched pre-pass packed every operand row-contiguous per k
// (A as K x M, B as K x N), the layout with 512-byte TMA rows that this kernel
// reads fastest, so all problems use the (!AK, !BKM) path.
template <int TM, int TN>
__global__ void __launch_bounds__(kThreads, 1)
    simt_grouped_kernel(const CUtensorMap* __restrict__ maps, const SimtProblem* __restrict__ probs,
                        int nprob, int total_tiles, int* err) {
  using S = SimtShape<TM, TN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * S::STAGE_BYTES);
  uint64_t* empty = full + kStages;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    fence_barrier_init();
  }
  __syncthreads();
  auto locate = [&](int t, SimtProblem& P, int& p, int& m0, int& n0) {
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (probs[mid].tile_start <= t) lo = mid; else hi = mid - 1;
    }
    p = lo;
    P = probs[lo];
    int tm, tn;
    raster_tile(t - P.tile_start, P.tiles_m, P.tiles_n, tm, tn);
    m0 = tm * S::BM;
    n0 = tn * S::BN;
  };
  if (warp == kConsumerWarps) {
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; ok && t < total_tiles; t += gridDim.x) {
        SimtProblem P;
        int p, m0, n0;
        locate(t, P, p, m0, n0);
        const CUtensorMap* ma = &maps[2 * p];
        const CUtensorMap* mb = &maps[2 * p + 1];
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                         reinterpret_cast<uint64_t>(ma)) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                         reinterpret_cast<uint64_t>(mb)) : "memory");
        for (int kt = 0; kt < P.nkt; ++kt, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (it / kStages) & 1;
          if (!mbar_wait(&empty[s], ph ^ 1, err, kDevTimeoutEmpty)) { ok = false; break; }
          uint8_t* sa = smem + s * S::STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], S::STAGE_BYTES);
          tma_load_2d(sa, ma, &full[s], m0, (P.kt0 + kt) * kBK);
          tma_load_2d(sa + S::A_BYTES, mb, &full[s], n0, (P.kt0 + kt) * kBK);
        }
      }
    }
    return;
  }
  uint32_t it = 0;
  for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
    SimtProblem P;
    int p, m0, n0;
    locate(t, P, p, m0, n0);
    float acc[TM][TN];
    if (!simt_mainloop<TM, TN, false, false>(smem, full, empty, P.nkt, it, acc, err)) return;
    simt_store<TM, TN, false, false>(acc, P.C, P.M, P.N, P.ldc, P.alpha, P.beta, m0, n0, P.epi);
  }
}

// Batched pre-pass of the grouped SIMT form: copy op(X) (element (r, k) at
// src[r*sr + k*sk]) to dst[k*ld + r] (rows contiguous per k), 32 x 64 tiles
// through shared memory so both source layouts read and write coalesced.
__global__ void __launch_bounds__(256) pack_kmajor_batched_kernel(const PackJob* __restrict__ jobs,
                                                                  int njobs, int total_tiles) {
  __shared__ float tile[32][65];
  __shared__ int starts[2048];
  const int cached = min(njobs, 2048);
  for (int i = threadIdx.x; i < cached; i += blockDim.x) starts[i] = jobs[i].tile_start;
  __syncthreads();
  for (int b = blockIdx.x; b < total_tiles; b += gridDim.x) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const int st = njobs <= 2048 ? starts[mid] : jobs[mid].tile_start;
    if (st <= b) lo = mid; else hi = mid - 1;
  }
  const PackJob j = jobs[lo];
  const int local = b - j.tile_start;
  const int tiles_k = (j.K + 63) / 64;
  const int r0 = (local / tiles_k) * 32, k0 = (local % tiles_k) * 64;
  const int t = threadIdx.x;
  if (j.gather) {  // implicit im2col: this thread's pixel is fixed, taps vary
    const int pix = j.gather == 2 ? k0 + (t & 63) : r0 + (t & 31);
    const Im2colPix px = im2col_pix(j.im, pix);
    const int npix = j.gather == 2 ? j.K : j.rows;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (j.gather == 2) {  // rows are taps
        const int rr = (t >> 6) + 4 * i, r = r0 + rr;
        tile[rr][t & 63] = (r < j.rows && pix < npix) ? im2col_load(j.im, im2col_tap(j.im, r), px)
                                                       : 0.f;
      } else {              // rows are pixels
        const int kk = (t >> 5) + 8 * i, k = k0 + kk;
        tile[t & 31][kk] = (k < j.K && pix < npix) ? im2col_load(j.im, im2col_tap(j.im, k), px)
                                                    : 0.f;
      }
    }
  } else if (j.sk == 1) {
    const int k = k0 + (t & 63);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int rr = (t >> 6) + 4 * i, r = r0 + rr;
      tile[rr][t & 63] = (r < j.rows && k < j.K) ? j.src[r * j.sr + k] : 0.f;
    }
  } else {
    const int rr = t & 31, r = r0 + rr;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int kk = (t >> 5) + 8 * i, k = k0 + kk;
      tile[rr][kk] = (r < j.rows && k < j.K) ? j.src[r * j.sr + k * j.sk] : 0.f;
    }
  }
  __syncthreads();
  {
    const int rr = t & 31, r = r0 + rr;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int kk = (t >> 5) + 8 * i, k = k0 + kk;
      if (r < j.rows && k < j.K) j.dst[static_cast<size_t>(k) * j.ld + r] = tile[rr][kk];
    }
  }
  __syncthreads();  // the tile buffer is refilled by the next iteration
  }
}

// Copy a rows x cols row-major matrix into a dense buffer whose rows are
// `ldd` floats (a multiple of 4) so that TMA can describe it.
__global__ void pack_rows_kernel(const float* __restrict__ src, int lds, float* __restrict__ dst,
                                 int ldd, int rows, int cols) {
  const size_t total = static_cast<size_t>(rows) * ldd;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i / ldd), c = static_cast<int>(i % ldd);
    dst[i] = (c < cols) ? src[static_cast<size_t>(r) * lds + c] : 0.f;
  }
}

__global__ void scale_kernel(float* __restrict__ C, int M, int N, int ldc, float beta) {
  const size_t total = static_cast<size_t>(M) * N;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    float* p = C + (i / N) * static_cast<size_t>(ldc) + (i % N);
    *p = (beta == 0.f) ? 0.f : beta * *p;
  }
}

bool tma_ok(const void* p, int ld) {
  return (reinterpret_cast<uintptr_t>(p) & 15) == 0 && (ld % 4) == 0;
}

// Stored shape (rows, cols) of an operand.
void stored_a(const Gemm& g, int& rows, int& cols) {
  if (g.ta == 'N') { rows = g.M; cols = g.K; } else { rows = g.K; cols = g.M; }
}
void stored_b(const Gemm& g, int& rows, int& cols) {
  if (g.tb == 'N') { rows = g.K; cols = g.N; } else { rows = g.N; cols = g.K; }
}

template <int TM, int TN, bool AK, bool BKM, bool NP>
ugemm_status launch_t(const Gemm& g, const float* A, int lda, const float* B, int ldb,
                      int* dev_err, cudaStream_t st) {
  using S = SimtShape<TM, TN>;
  CUtensorMap ta, tb;
  bool ok;
  if (AK) ok = encode_tmap_2d(&ta, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, A, g.K, g.M, lda * 4ull,
                              kBK, S::BM, CU_TENSOR_MAP_SWIZZLE_128B);
  else    ok = encode_tmap_2d(&ta, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, A, g.M, g.K, lda * 4ull,
                              S::BM, kBK, CU_TENSOR_MAP_SWIZZLE_NONE);
  if (!ok) return UGEMM_ERR_CUDA;
  if (BKM) ok = encode_tmap_2d(&tb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, B, g.K, g.N, ldb * 4ull,
                               kBK, S::BN, CU_TENSOR_MAP_SWIZZLE_128B);
  else     ok = encode_tmap_2d(&tb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, B, g.N, g.K, ldb * 4ull,
                               S::BN, kBK, CU_TENSOR_MAP_SWIZZLE_NONE);
  if (!ok) return UGEMM_ERR_CUDA;
  void (*kern)(const CUtensorMap, const CUtensorMap, float*, int, int, int, int, float, float,
               Epilogue, int, int, int*);
  if constexpr (NP) kern = simt_sgemm_np_kernel<TM, TN, AK, BKM>;
  else kern = simt_sgemm_kernel<TM, TN, AK, BKM>;
  const int threads = NP ? kConsumerWarps * 32 : kThreads;
  static std::atomic<uint64_t> attr_done{0};  // per instantiation and device
  if (!smem_attr_once(kern, S::SMEM, attr_done)) return UGEMM_ERR_CUDA;
  const int tiles_m = cdiv(g.M, S::BM), tiles_n = cdiv(g.N, S::BN);
  prof_begin(st);
  kern<<<tiles_m * tiles_n, threads, S::SMEM, st>>>(ta, tb, g.C, g.M, g.N, g.K, g.ldc, g.alpha,
                                                     g.beta, g.epi, tiles_m, tiles_n, dev_err);
  prof_end(st, kProfSimt);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

template <int TM, int TN, bool NP>
ugemm_status launch_tile(const Gemm& g, const float* A, int lda, const float* B, int ldb,
                         int* dev_err, cudaStream_t st) {
  const bool ak = g.ta == 'N', bk = g.tb == 'T';
  if (ak && !bk) return launch_t<TM, TN, true, false, NP>(g, A, lda, B, ldb, dev_err, st);
  if (ak && bk) return launch_t<TM, TN, true, true, NP>(g, A, lda, B, ldb, dev_err, st);
  if (!ak && !bk) return launch_t<TM, TN, false, false, NP>(g, A, lda, B, ldb, dev_err, st);
  return launch_t<TM, TN, false, true, NP>(g, A, lda, B, ldb, dev_err, st);
}

}  // namespace

size_t simt_scratch_bytes(const Gemm& g) {
  size_t bytes = 0;
  int r, c;
  if (!tma_ok(g.A, g.lda)) { stored_a(g, r, c); bytes += align_up(size_t(r) * align_up(c, 4) * 4, 256); }
  if (!tma_ok(g.B, g.ldb)) { stored_b(g, r, c); bytes += align_up(size_t(r) * align_up(c, 4) * 4, 256); }
  return bytes;
}

int simt_pick_tile(const Gemm& g) {
  int sms = 148;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  static int forced = -2;
  if (forced == -2) {
    const char* e = std::getenv("UGEMM_SIMT_TILE");
    forced = e ? std::atoi(e) : -1;
    if (forced >= kSimtTileCount) forced = -1;
  }
  if (forced >= 0) return forced;
  // Measured on GB300 at 8192^3: the producer-less 128x128 kernel is 3-18%
  // faster than the one with a producer warp in every transpose pair; 64x64
  // tiles win when 128x128 tiles cannot fill two waves.
  const long big = long(cdiv(g.M, 128)) * cdiv(g.N, 128);
  return big >= 2L * sms ? kSimt128x128np : kSimt64x64;
}

ugemm_status simt_launch(const Gemm& g, int tile, Scratch ws, int* dev_err, cudaStream_t st) {
  const float* A = g.A;
  const float* B = g.B;
  int lda = g.lda, ldb = g.ldb;
  uint8_t* wp = static_cast<uint8_t*>(ws.ptr);
  size_t used = 0;
  int r, c;
  if (!tma_ok(A, lda)) {
    stored_a(g, r, c);
    const int ld = static_cast<int>(align_up(c, 4));
    const size_t need = align_up(size_t(r) * ld * 4, 256);
    if (used + need > ws.bytes) return UGEMM_ERR_ARENA_TOO_SMALL;
    float* dst = reinterpret_cast<float*>(wp + used);
    prof_begin(st);
    pack_rows_kernel<<<std::min<size_t>(4096, (size_t(r) * ld + 255) / 256), 256, 0, st>>>(
        A, lda, dst, ld, r, c);
    prof_end(st, kProfAux);
    A = dst; lda = ld; used += need;
  }
  if (!tma_ok(B, ldb)) {
    stored_b(g, r, c);
    const int ld = static_cast<int>(align_up(c, 4));
    const size_t need = align_up(size_t(r) * ld * 4, 256);
    if (used + need > ws.bytes) return UGEMM_ERR_ARENA_TOO_SMALL;
    float* dst = reinterpret_cast<float*>(wp + used);
    prof_begin(st);
    pack_rows_kernel<<<std::min<size_t>(4096, (size_t(r) * ld + 255) / 256), 256, 0, st>>>(
        B, ldb, dst, ld, r, c);
    prof_end(st, kProfAux);
    B = dst; ldb = ld; used += need;
  }
  switch (tile) {
    case kSimt64x64: return launch_tile<4, 4, false>(g, A, lda, B, ldb, dev_err, st);
    case kSimt128x256: return launch_tile<8, 16, true>(g, A, lda, B, ldb, dev_err, st);
    case kSimt128x128np: return launch_tile<8, 8, true>(g, A, lda, B, ldb, dev_err, st);
    default: return launch_tile<8, 8, false>(g, A, lda, B, ldb, dev_err, st);
  }
}

ugemm_status scale_c_launch(const Gemm& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0 || g.beta == 1.f) return UGEMM_OK;
  const size_t total = size_t(g.M) * g.N;
  prof_begin(st);
  scale_kernel<<<std::min<size_t>(4096, (total + 255) / 256), 256, 0, st>>>(g.C, g.M, g.N, g.ldc,
                                                                            g.beta);
  prof_end(st, kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

int simt_block(int tile) { return tile == kSimt64x64 ? 64 : 128; }

bool simt_encode_grouped(int tile, const float* a, int M, const float* b, int N, int K, int ld_a,
                         int ld_b, CUtensorMap* ta, CUtensorMap* tb) {
  const int bm = simt_block(tile);
  return encode_tmap_2d(ta, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a, M, std::max(K, 1), ld_a * 4ull,
                        bm, kBK, CU_TENSOR_MAP_SWIZZLE_NONE) &&
         encode_tmap_2d(tb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b, N, std::max(K, 1), ld_b * 4ull,
                        bm, kBK, CU_TENSOR_MAP_SWIZZLE_NONE);
}

namespace {
template <int TM, int TN>
ugemm_status grouped_t(const CUtensorMap* maps, const SimtProblem* probs, int nprob, int total,
                       int max_ctas, int* dev_err, cudaStream_t st) {
  using S = SimtShape<TM, TN>;
  auto kern = simt_grouped_kernel<TM, TN>;
  static std::atomic<uint64_t> attr_done{0};  // per instantiation and device
  if (!smem_attr_once(kern, S::SMEM, attr_done)) return UGEMM_ERR_CUDA;
  int sms = 148, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::max(1, std::min(total, max_ctas > 0 ? max_ctas : sms));
  prof_begin(st);
  kern<<<grid, kThreads, S::SMEM, st>>>(maps, probs, nprob, total, dev_err);
  prof_end(st, kProfGrouped);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}
}  // namespace

ugemm_status simt_grouped_launch(int tile, const CUtensorMap* maps, const SimtProblem* probs,
                                 int nprob, int total_tiles, int max_ctas, int* dev_err,
                                 cudaStream_t st) {
  if (total_tiles <= 0) return UGEMM_OK;
  if (tile == kSimt64x64) return grouped_t<4, 4>(maps, probs, nprob, total_tiles, max_ctas, dev_err, st);
  return grouped_t<8, 8>(maps, probs, nprob, total_tiles, max_ctas, dev_err, st);
}

ugemm_status pack_batched_launch(const PackJob* jobs, int njobs, int total_tiles, cudaStream_t st) {
  if (total_tiles <= 0) return UGEMM_OK;
  int sms = 148, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  prof_begin(st);
  pack_kmajor_batched_kernel<<<std::min(total_tiles, sms * 8), 256, 0, st>>>(jobs, njobs,
                                                                             total_tiles);
  prof_end(st, kProfSplitPrep);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace ugemm
