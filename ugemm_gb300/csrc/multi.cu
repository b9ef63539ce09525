// multi.cu -- a few split-precision GEMMs, and split-K slices of them, in one
// persistent launch of the grouped tensor-core kernel, with all scratch in
// the caller's workspace: no plan, no allocation, nothing read from host
// memory at run time (the problem table travels as a kernel parameter), so
// it is usable inside stream capture.
//
// Used where one GEMM launch at a time leaves SMs idle:
//   * ugemm_sgemm_backward: dA = alpha dC op(B)^T and dB = alpha op(A)^T dC
//     share one launch, so the tiles of both fill the GPU together;
//   * single GEMMs whose output has fewer tiles than the GPU has SMs and
//     whose k is deep (a weight-gradient shape): cut into k slices whose
//     FP32 partial tiles one reduce launch sums in a fixed order.
// Each GEMM may also be computed transposed (C^T = op(B)^T op(A)^T) when
// that wastes less of the 128-row tiles, as in grouped plans.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>

#include "internal.h"
#include "split_tc.cuh"

namespace ugemm {
namespace {

constexpr int kMultiSubs = 24;  // kernel problems (slices) per launch
constexpr int kMinSlice = 16;   // shortest slice, in 32-deep k-blocks

// The shortest slice in stages of the kernel's k depth.
int min_slice(int pieces) { return kMinSlice * kTcKB / split_stage_k(pieces); }

// Everything the launch reads from device memory, filled by one small kernel
// from its by-value parameter (at most 4 KB of parameters).
struct MultiTable {
  CUtensorMap maps[2 * kMultiMax];
  TcProblem probs[kMultiSubs];
  ReduceJob red[kMultiMax];
};
static_assert(sizeof(MultiTable) <= 4000, "multi table must fit the kernel parameter space");
static_assert(sizeof(MultiTable) % 16 == 0, "multi table copies as 16-byte words");

// Block 0 copies the table; every thread also writes the tile table of a
// grid of `grid` CTAs: CTA c takes tiles c, c + grid, c + 2 grid, ... (in
// longest-k-first problem order), stored contiguously after the grid's
// {first, end} ranges, one {problem, m0, n0, 0} record per tile.
__global__ void multi_table_kernel(const __grid_constant__ MultiTable t, int nsub, int total_tiles,
                                   int block_n, int grid, MultiTable* dst, int4* table) {
  if (blockIdx.x == 0) {
    const uint4* s = reinterpret_cast<const uint4*>(&t);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int i = threadIdx.x; i < static_cast<int>(sizeof(MultiTable) / 16); i += blockDim.x)
      d[i] = s[i];
    // the GEMM kernel reads the tensor maps through the tensormap proxy
    asm volatile("fence.proxy.tensormap::generic.release.gpu;" ::: "memory");
  }
  const int per = total_tiles / grid, extra = total_tiles % grid;
  auto first = [&](int c) { return c * per + (c < extra ? c : extra); };
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < grid; c += gridDim.x * blockDim.x)
    table[c] = make_int4(first(c), first(c + 1), 0, 0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total_tiles; i += gridDim.x * blockDim.x) {
    int p = 0;
    while (p + 1 < nsub && t.probs[p + 1].tile_start <= i) ++p;
    const TcProblem& P = t.probs[p];
    int m0, n0;
    tc_raster(i - P.tile_start, P.tiles_m, P.tiles_n, block_n, m0, n0);
    table[grid + first(i % grid) + i / grid] = make_int4(p, m0, n0, 0);
  }
}

double padded(int rows, int cols, int bn) {
  return double(align_up(rows, 128)) * ((cols / bn) * bn + align_up(cols % bn, 16));
}

int sm_count() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

struct Geo {
  bool swap = false;
  int tiles = 0, nkb = 0, slices = 1, per = 0;
};

// Scratch layout: per GEMM [A pieces | B pieces], then the partial tiles of
// the sliced GEMMs, the table and the tile records.
struct Layout {
  Geo geo[kMultiMax];
  int block_n = 256;
  size_t a_off[kMultiMax], b_off[kMultiMax], part_off[kMultiMax];
  size_t table_off = 0, recs_off = 0, total = 0;
  int grid = 1;  // persistent CTAs of the launch
};

Layout layout_for(const Gemm* gs, int n, const SplitPlan& p, int sms) {
  Layout L;
  // 256-wide tiles unless every output is narrow in its better orientation
  int widest = 0;
  for (int i = 0; i < n; ++i) {
    const Gemm& g = gs[i];
    const bool swap = padded(g.N, g.M, 256) < padded(g.M, g.N, 256);
    widest = std::max(widest, swap ? g.M : g.N);
  }
  L.block_n = widest > 128 ? 256 : 128;
  double work = 0;
  for (int i = 0; i < n; ++i) {
    const Gemm& g = gs[i];
    Geo& o = L.geo[i];
    o.swap = padded(g.N, g.M, L.block_n) < padded(g.M, g.N, L.block_n);
    const int rows = o.swap ? g.N : g.M, cols = o.swap ? g.M : g.N;
    o.tiles = cdiv(rows, kTcBM) * cdiv(cols, L.block_n);
    o.nkb = split_nkb(p.pieces, g.K);
    o.per = o.nkb;
    work += double(o.tiles) * o.nkb;
  }
  // split-K: tiles no longer than about half an SM's fair share of the work
  const double fair = work / (2.0 * sms);
  int subs = n;
  for (int i = 0; i < n; ++i) {
    const Gemm& g = gs[i];
    Geo& o = L.geo[i];
    if (o.nkb < 2 * min_slice(p.pieces) || o.nkb <= fair) continue;
    const int len = std::max(min_slice(p.pieces), static_cast<int>(fair) + 1);
    const size_t tile_bytes = size_t(g.M) * g.N * 4;
    int sl = std::min(cdiv(o.nkb, len), kMultiSubs - (subs - 1));
    sl = static_cast<int>(std::min<size_t>(sl, (size_t(512) << 20) / tile_bytes));
    if (sl < 2) continue;
    o.per = cdiv(o.nkb, sl);
    o.slices = cdiv(o.nkb, o.per);
    subs += o.slices - 1;
  }
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    L.a_off[i] = off;
    off += split_operand_bytes(p.pieces, gs[i].M, gs[i].K);
    L.b_off[i] = off;
    off += split_operand_bytes(p.pieces, gs[i].N, gs[i].K);
  }
  for (int i = 0; i < n; ++i) {
    L.part_off[i] = off;
    if (L.geo[i].slices > 1) off += align_up(size_t(L.geo[i].slices) * gs[i].M * gs[i].N * 4, 256);
  }
  L.table_off = align_up(off, 256);
  int tiles = 0;
  for (int i = 0; i < n; ++i) tiles += L.geo[i].tiles * L.geo[i].slices;
  L.grid = std::max(1, std::min(tiles, sms));
  L.recs_off = L.table_off + align_up(sizeof(MultiTable), 256);
  L.total = L.recs_off + align_up(size_t(L.grid + tiles) * sizeof(int4), 256);
  return L;
}

}  // namespace

TailPlan tail_plan(const Gemm& g, const SplitPlan& p) {
  TailPlan t;
  if (g.M == 0 || g.N == 0 || g.K == 0 || g.alpha == 0.f) return t;
  const int sms = sm_count();
  const int tiles_m = cdiv(g.M, kTcBM), tiles_n = cdiv(g.N, p.block_n);
  const int tiles = tiles_m * tiles_n, rem = tiles % sms;
  if (tiles <= sms || rem == 0 || split_nkb(p.pieces, g.K) < 2 * min_slice(p.pieces)) return t;
  // the raster order ends with the last group of tile rows, column by column
  const int first_m = ((tiles_m - 1) / kTcRaster) * kTcRaster, rows = tiles_m - first_m;
  const int cols = cdiv(rem, rows);             // whole tile columns of that group
  if (cols >= tiles_n || 2 * cols * rows > sms) return t;
  t.use = true;
  t.main_tiles = tiles - cols * rows;
  t.r0 = first_m * kTcBM;
  t.c0 = (tiles_n - cols) * p.block_n;
  return t;
}

size_t tail_scratch_bytes(const Gemm& g, const SplitPlan& p) {
  const TailPlan t = tail_plan(g, p);
  if (!t.use) return 0;
  const int tiles = 2 * cdiv(g.M - t.r0, kTcBM) * cdiv(g.N - t.c0, p.block_n);
  return align_up(2 * size_t(g.M - t.r0) * (g.N - t.c0) * 4, 256) +
         align_up(sizeof(MultiTable), 256) + align_up(size_t(sm_count() + tiles) * sizeof(int4), 256);
}

ugemm_status tail_launch(const Gemm& g, const SplitPlan& p, const TailPlan& tail,
                         const void* a_pieces, const void* b_pieces, void* scratch, int* dev_err,
                         cudaStream_t st) {
  const int Mt = g.M - tail.r0, Nt = g.N - tail.c0, Kp = split_kp(g.K);
  const size_t mn = size_t(Mt) * Nt;
  uint8_t* base = static_cast<uint8_t*>(scratch);
  float* part = reinterpret_cast<float*>(base);
  uint8_t* tab = base + align_up(2 * mn * 4, 256);
  int4* recs = reinterpret_cast<int4*>(tab + align_up(sizeof(MultiTable), 256));
  MultiTable t;
  std::memset(&t, 0, sizeof t);
  const size_t row_bytes = size_t(Kp) * piece_bytes(p.pieces);
  const auto* ap = static_cast<const uint8_t*>(a_pieces) + size_t(tail.r0) * row_bytes;
  const auto* bp = static_cast<const uint8_t*>(b_pieces) + size_t(tail.c0) * row_bytes;
  if (!split_encode_view(p.pieces, kTcBM, ap, Mt, g.M, g.K, &t.maps[0]) ||
      !split_encode_view(p.pieces, p.block_n, bp, Nt, g.N, g.K, &t.maps[1]))
    return UGEMM_ERR_CUDA;
  const int nkb = split_nkb(p.pieces, g.K), per = cdiv(nkb, 2);
  int tiles = 0;
  for (int s = 0; s < 2; ++s) {
    TcProblem& tp = t.probs[s];
    tp.C = part + s * mn;
    tp.M = Mt;
    tp.N = Nt;
    tp.ldc = Nt;
    tp.alpha = g.alpha;
    tp.beta = 0.f;
    tp.kb0 = s * per;
    tp.nkb = std::min(per, nkb - tp.kb0);
    tp.tiles_m = cdiv(Mt, kTcBM);
    tp.tiles_n = cdiv(Nt, p.block_n);
    tp.tile_start = tiles;
    if (p.f16) {  // the views' rows and columns keep the whole operands' scales
      tp.fmax_a = split_fmax_word(a_pieces, p.pieces, g.M, g.K) + tail.r0;
      tp.fmax_b = split_fmax_word(b_pieces, p.pieces, g.N, g.K) + tail.c0;
    }
    tiles += tp.tiles_m * tp.tiles_n;
  }
  Epilogue epi = g.epi;
  if (epi.bias) epi.bias += tail.r0;
  t.red[0] = ReduceJob{part, g.C + size_t(tail.r0) * g.ldc + tail.c0, Mt, Nt, g.ldc, 2, g.beta, epi};
  const int grid = std::max(1, std::min(tiles, sm_count()));
  prof_begin(st);
  multi_table_kernel<<<std::max(1, std::min(cdiv(tiles, 256), 64)), 256, 0, st>>>(
      t, 2, tiles, p.block_n, grid, reinterpret_cast<MultiTable*>(tab), recs);
  prof_end(st, kProfControl);
  if (cudaPeekAtLastError() != cudaSuccess) return UGEMM_ERR_CUDA;
  SplitPlan q = p;
  q.epi = false;
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof dummy);
  TcProblem single{};
  const int chunk =
      split_chunk_stages(p.pieces, p.chunk_kb > 0 ? p.chunk_kb : split_default_chunk_kb(g.K));
  ugemm_status s = split_gemm_launch(
      q, dummy, dummy, single, reinterpret_cast<const CUtensorMap*>(tab + offsetof(MultiTable, maps)),
      reinterpret_cast<const TcProblem*>(tab + offsetof(MultiTable, probs)), recs, tiles, chunk,
      grid, dev_err, st);
  if (s != UGEMM_OK) return s;
  return splitk_reduce_launch(reinterpret_cast<const ReduceJob*>(tab + offsetof(MultiTable, red)),
                              1, static_cast<long long>(mn), st);
}

bool multi_wanted(const Gemm& g, const SplitPlan& p) {
  if (g.M == 0 || g.N == 0 || g.K == 0 || g.alpha == 0.f) return false;
  const int tiles = cdiv(g.M, kTcBM) * cdiv(g.N, p.block_n);
  return tiles < sm_count() && split_nkb(p.pieces, g.K) >= 2 * min_slice(p.pieces);
}

size_t multi_scratch_bytes(const Gemm* gs, int n, const SplitPlan& p) {
  if (n < 1 || n > kMultiMax) return 0;
  return layout_for(gs, n, p, sm_count()).total;
}

ugemm_status multi_launch(const Gemm* gs, int n, const SplitPlan& plan, Scratch ws, int* dev_err,
                          cudaStream_t st) {
  if (n < 1 || n > kMultiMax) return UGEMM_ERR_ARG;
  for (int i = 0; i < n; ++i)
    if (gs[i].M == 0 || gs[i].N == 0 || gs[i].K == 0 || gs[i].alpha == 0.f) return UGEMM_ERR_ARG;
  const Layout L = layout_for(gs, n, plan, sm_count());
  if (L.total > ws.bytes) return UGEMM_ERR_ARENA_TOO_SMALL;
  uint8_t* base = static_cast<uint8_t*>(ws.ptr);
  SplitPlan p = plan;
  p.block_n = L.block_n;
  p.epi = false;

  MultiTable t;
  std::memset(&t, 0, sizeof t);
  SplitJobTable jt{};
  static_assert(2 * kMultiMax <= kSplitTableJobs, "two operands per GEMM");
  int nj = 0, split_tiles = 0;
  int nsub = 0, nred = 0, tiles = 0;
  long long red_max = 0;
  for (int i = 0; i < n; ++i) {
    const Gemm& g = gs[i];
    const Geo& o = L.geo[i];
    void* ap = base + L.a_off[i];
    void* bp = base + L.b_off[i];
    long long a_sr, a_sk, b_sr, b_sk;
    split_operand_strides(g, &a_sr, &a_sk, &b_sr, &b_sk);
    if (p.f16) {  // the FP16x3 split needs each operand's row maxima first
      ugemm_status s = split_operand_launch(p.pieces, g.A, a_sr, a_sk, g.M, g.K, ap, st, true);
      if (s == UGEMM_OK) s = split_operand_launch(p.pieces, g.B, b_sr, b_sk, g.N, g.K, bp, st, true);
      if (s != UGEMM_OK) return s;
    } else {  // every operand in one split launch (below)
      const int kp = split_kp(g.K), tk = cdiv(kp, 64);
      jt.jobs[nj++] = SplitJob{g.A, a_sr, a_sk, static_cast<__nv_bfloat16*>(ap), g.M, g.K, kp,
                               split_tiles};
      split_tiles += cdiv(g.M, 32) * tk;
      jt.jobs[nj++] = SplitJob{g.B, b_sr, b_sk, static_cast<__nv_bfloat16*>(bp), g.N, g.K, kp,
                               split_tiles};
      split_tiles += cdiv(g.N, 32) * tk;
    }
    const bool ok = o.swap ? split_encode_maps(p.pieces, p.block_n, bp, g.N, ap, g.M, g.K,
                                               &t.maps[2 * i], &t.maps[2 * i + 1])
                           : split_encode_maps(p.pieces, p.block_n, ap, g.M, bp, g.N, g.K,
                                               &t.maps[2 * i], &t.maps[2 * i + 1]);
    if (!ok) return UGEMM_ERR_CUDA;
    const bool sliced = o.slices > 1;
    float* part = reinterpret_cast<float*>(base + L.part_off[i]);
    for (int sidx = 0; sidx < o.slices; ++sidx) {
      TcProblem& tp = t.probs[nsub++];
      tp.C = sliced ? part + size_t(sidx) * g.M * g.N : g.C;
      tp.M = o.swap ? g.N : g.M;
      tp.N = o.swap ? g.M : g.N;
      tp.ldc = sliced ? g.N : g.ldc;
      tp.alpha = g.alpha;
      tp.beta = sliced ? 0.f : g.beta;
      tp.kb0 = sidx * o.per;
      tp.nkb = std::min(o.per, o.nkb - tp.kb0);
      tp.tiles_m = cdiv(tp.M, kTcBM);
      tp.tiles_n = cdiv(tp.N, p.block_n);
      tp.swap = o.swap ? 1 : 0;
      tp.map = i;
      tp.epi = sliced ? Epilogue{} : g.epi;
      p.epi |= tp.epi.bias != nullptr || tp.epi.act != 0;
      if (p.f16) {  // kernel operand a is op(B)^T's pieces when swapped
        unsigned* wa = split_fmax_word(ap, p.pieces, g.M, g.K);
        unsigned* wb = split_fmax_word(bp, p.pieces, g.N, g.K);
        tp.fmax_a = o.swap ? wb : wa;
        tp.fmax_b = o.swap ? wa : wb;
      }
    }
    if (sliced) {
      t.red[nred++] = ReduceJob{part, g.C, g.M, g.N, g.ldc, o.slices, g.beta, g.epi};
      red_max = std::max(red_max, static_cast<long long>(g.M) * g.N);
    }
  }
  int min_k = gs[0].K;  // the chunk rule follows the shallowest GEMM (the most accurate choice)
  for (int i = 1; i < n; ++i) min_k = std::min(min_k, gs[i].K);
  // longest k first; tile offsets in that order
  std::stable_sort(t.probs, t.probs + nsub,
                   [](const TcProblem& a, const TcProblem& b) { return a.nkb > b.nkb; });
  for (int j = 0; j < nsub; ++j) {
    t.probs[j].tile_start = tiles;
    tiles += t.probs[j].tiles_m * t.probs[j].tiles_n;
  }
  // the operands' bf16 / TF32 pieces: one launch for all of them (four
  // launches of one operand each left a ramp and a tail apiece)
  if (nj > 0) {
    const ugemm_status s = split_param_launch(p.pieces, jt, nj, split_tiles, st);
    if (s != UGEMM_OK) return s;
  }
  uint8_t* tab = base + L.table_off;
  int4* recs = reinterpret_cast<int4*>(base + L.recs_off);
  prof_begin(st);
  multi_table_kernel<<<std::max(1, std::min(cdiv(tiles, 256), 64)), 256, 0, st>>>(
      t, nsub, tiles, p.block_n, L.grid, reinterpret_cast<MultiTable*>(tab), recs);
  prof_end(st, kProfControl);
  if (cudaPeekAtLastError() != cudaSuccess) return UGEMM_ERR_CUDA;
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof dummy);
  TcProblem single{};
  const int chunk =
      split_chunk_stages(p.pieces, p.chunk_kb > 0 ? p.chunk_kb : split_default_chunk_kb(min_k));
  ugemm_status s = split_gemm_launch(
      p, dummy, dummy, single, reinterpret_cast<const CUtensorMap*>(tab + offsetof(MultiTable, maps)),
      reinterpret_cast<const TcProblem*>(tab + offsetof(MultiTable, probs)), recs, tiles, chunk,
      L.grid, dev_err, st);
  if (s != UGEMM_OK || nred == 0) return s;
  return splitk_reduce_launch(reinterpret_cast<const ReduceJob*>(tab + offsetof(MultiTable, red)),
                              nred, red_max, st);
}

}  // namespace ugemm
