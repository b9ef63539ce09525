// grouped.cu -- grouped GEMM: many independent, unevenly sized SGEMMs in one
// persistent launch (spec batching form; no reference counterpart --
// the reference runs one GEMM per OpenCL NDRange, sgemm_ocl2.h:201-215).
//
// A plan is built once on the host and replayed any number of times:
//   * problems are validated and ordered by decreasing k depth, so the
//     persistent CTAs, which take tiles in round-robin order, meet the
//     longest tiles first;
//   * every operand gets a slot in one scratch buffer: bf16 pieces for the
//     split-precision form, K x rows FP32 copies for the SIMT form;
//   * one batched pre-pass launch writes all the slots, one persistent GEMM
//     launch walks all output tiles of all problems; per-problem TMA
//     descriptors and tile offsets live in one device table;
//   * with UGEMM_PLAN_GRAPH the two launches are captured once into a CUDA
//     graph, and ugemm_grouped_run replays the graph on the caller's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "internal.h"
#include "simt.cuh"
#include "split_tc.cuh"

namespace ugemm {
namespace {

// Split-K reduction: C = sum_s part_s + beta*C (C not read when beta == 0),
// then the optional bias / activation; slices summed in a fixed order.
__global__ void __launch_bounds__(256) splitk_reduce_kernel(const ReduceJob* __restrict__ jobs) {
  const ReduceJob J = jobs[blockIdx.y];
  const long long mn = static_cast<long long>(J.M) * J.N;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < mn; i += 256LL * gridDim.x) {
    float v = 0.f;
    for (int s = 0; s < J.slices; ++s) v += J.part[s * mn + i];
    const int m = static_cast<int>(i / J.N), n = static_cast<int>(i % J.N);
    float* cp = J.C + static_cast<long long>(m) * J.ldc + n;
    if (J.beta != 0.f) v += J.beta * *cp;
    *cp = epilogue_apply(v, J.epi, m);
  }
}

}  // namespace

ugemm_status splitk_reduce_launch(const ReduceJob* jobs, int njobs, long long max_mn,
                                  cudaStream_t st) {
  if (njobs <= 0) return UGEMM_OK;
  const long long blocks = std::min<long long>((max_mn + 255) / 256, 152LL * 8);
  prof_begin(st);
  splitk_reduce_kernel<<<dim3(static_cast<unsigned>(blocks), njobs), 256, 0, st>>>(jobs);
  prof_end(st, kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace ugemm

struct ugemm_grouped_plan_s {
  int count = 0;
  int form = UGEMM_PREC_SIMT;
  ugemm_tile_config cfg{};
  int device = 0;
  double flops = 0;
  // device memory
  void* table = nullptr;    // maps | problems | jobs | reduce jobs | tile records | max words
  void* scratch = nullptr;  // operand slots
  int* dev_err = nullptr;
  const CUtensorMap* maps = nullptr;
  const void* probs = nullptr;
  const void* jobs = nullptr;
  int njobs = 0, prep_tiles = 0, gemm_tiles = 0;
  int nsub = 0;                   // kernel problems (split-K slices count one each)
  const void* reduce = nullptr;   // split-K reduce jobs
  const int4* tiles = nullptr;    // split form: per-CTA ranges, then one record per tile
  float* chunk_sums = nullptr;    // fused 256-wide launches: kTcFusedSumBytes per CTA
  unsigned* fmax = nullptr;       // FP16x3: the largest magnitude of every operand row
  int nfmax = 0;                  // words at fmax
  int grid = 0;                   // split form: persistent CTAs the tile table is dealt to
  int nreduce = 0;
  long long reduce_max = 0;       // largest M x N among them
  ugemm::SplitPlan split{};
  // optional graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace ugemm {
namespace {

ugemm_status plan_fail(ugemm_status s, const char* msg) {
  set_last_error(s, msg);
  return s;
}

ugemm_status reduce_launch(const ugemm_grouped_plan_s* p, cudaStream_t st) {
  if (p->nreduce == 0) return UGEMM_OK;
  return splitk_reduce_launch(static_cast<const ReduceJob*>(p->reduce), p->nreduce, p->reduce_max,
                              st);
}

ugemm_status launch_plan(ugemm_grouped_plan_s* p, cudaStream_t st) {
  ugemm_status s;
  if (p->form == UGEMM_PREC_SIMT) {
    s = pack_batched_launch(static_cast<const PackJob*>(p->jobs), p->njobs, p->prep_tiles, st);
    if (s != UGEMM_OK) return s;
    const int tile = p->cfg.block_n == 64 ? kSimt64x64 : kSimt128x128;
    s = simt_grouped_launch(tile, p->maps, static_cast<const SimtProblem*>(p->probs), p->nsub,
                            p->gemm_tiles, p->cfg.max_ctas, p->dev_err, st);
    return s == UGEMM_OK ? reduce_launch(p, st) : s;
  }
  if (!p->split.fused) {
    s = split_batched_launch(p->split.pieces, static_cast<const SplitJob*>(p->jobs), p->njobs,
                             p->prep_tiles, st, p->fmax, p->nfmax);
    if (s != UGEMM_OK) return s;
  }
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof dummy);
  TcProblem single{};
  single.chunk_sums = p->chunk_sums;
  s = split_gemm_launch(p->split, dummy, dummy, single, p->maps,
                        static_cast<const TcProblem*>(p->probs), p->tiles, p->gemm_tiles,
                        split_chunk_stages(p->split.pieces, std::max(1, p->cfg.chunk_k / kTcKB)),
                        p->grid, p->dev_err, st);
  return s == UGEMM_OK ? reduce_launch(p, st) : s;
}

// The FP32 source of one kernel operand of a fused launch (rows of op(A),
// or of op(B)^T, by k) as a 2-D tensor map: k contiguous (row stride sr) or
// rows contiguous (k stride sk).  *kc says which.
bool fused_operand_map(const float* base, long long sr, long long sk, int rows, int K,
                       int box_rows, int box_k, CUtensorMap* map, int* kc) {
  if (sk == 1) {
    *kc = 1;
    return fused_encode_map(base, sr, rows, K, true, box_rows, box_k, map);
  }
  *kc = 0;
  return sr == 1 && fused_encode_map(base, sk, K, rows, false, box_rows, box_k, map);
}

// A fused launch copies the FP32 operands with TMA: each needs a unit
// stride, a 16-byte aligned base and leading dimension, and k > 0 (a K == 0
// problem's operands may be empty); implicit im2col gathers take the
// pre-pass.
bool fusable(const Gemm& x) {
  if (x.K == 0 || x.b_im2col) return false;
  long long a_sr, a_sk, b_sr, b_sk;
  split_operand_strides(x, &a_sr, &a_sk, &b_sr, &b_sk);
  auto ok = [](const float* p, long long sr, long long sk) {
    const long long ld = sk == 1 ? sr : sk;
    return (sr == 1 || sk == 1) && (reinterpret_cast<uintptr_t>(p) & 15) == 0 && ld % 4 == 0;
  };
  return ok(x.A, a_sr, a_sk) && ok(x.B, b_sr, b_sk);
}

// Padded tile area of an R x C output in 128 x bn tiles whose right-edge
// tile is only as wide as its columns rounded to 16 (the split kernel's
// narrow-N MMAs).
double padded_area(int rows, int cols, int bn) {
  return double(align_up(rows, 128)) * ((cols / bn) * bn + align_up(cols % bn, 16));
}

void free_plan(ugemm_grouped_plan_s* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->table) cudaFree(p->table);
  if (p->scratch) cudaFree(p->scratch);
  if (p->dev_err) cudaFree(p->dev_err);
  delete p;
}

}  // namespace

ugemm_tile_config default_grouped_config(int form) {
  ugemm_tile_config c{};
  if (form == UGEMM_PREC_SIMT) {
    c.block_n = 128;
  } else {
    c.block_n = 256;
    c.chunk_k = split_default_chunk_kb(1 << 30) * kTcKB;
  }
  c.max_ctas = 0;
  return c;
}

}  // namespace ugemm

using namespace ugemm;

extern "C" {

UGEMM_API int ugemm_grouped_plan_create(int count, const ugemm_problem* problems, int precision,
                                        const ugemm_tile_config* config, int flags,
                                        ugemm_grouped_plan** out) {
  if (!out) return plan_fail(UGEMM_ERR_ARG, "plan output pointer is NULL");
  *out = nullptr;
  if (count <= 0 || !problems) return plan_fail(UGEMM_ERR_ARG, "empty problem list");
  int form = precision;
  if (form == UGEMM_PREC_AUTO) form = UGEMM_PREC_BF16X6;
  if (form < UGEMM_PREC_SIMT || form > UGEMM_PREC_TF32X3)
    return plan_fail(UGEMM_ERR_ARG, "unknown precision");
  // validate and normalise
  std::vector<Gemm> g(count);
  for (int i = 0; i < count; ++i) {
    const ugemm_problem& q = problems[i];
    const char ta = (q.transa == 'T' || q.transa == 't') ? 'T' : ((q.transa == 'N' || q.transa == 'n') ? 'N' : 0);
    const char tb = (q.transb == 'T' || q.transb == 't') ? 'T' : ((q.transb == 'N' || q.transb == 'n') ? 'N' : 0);
    if (!ta || !tb) return plan_fail(UGEMM_ERR_ARG, "transpose flags must be 'N' or 'T'");
    if (q.M <= 0 || q.N <= 0 || q.K < 0) return plan_fail(UGEMM_ERR_ARG, "bad problem size");
    const int a_cols = ta == 'N' ? q.K : q.M, b_cols = tb == 'N' ? q.N : q.K;
    if (q.lda < std::max(1, a_cols) || q.ldb < std::max(1, b_cols) || q.ldc < q.N)
      return plan_fail(UGEMM_ERR_ARG, "leading dimension smaller than the matrix width");
    if (!q.C || (q.K > 0 && (!q.A || !q.B))) return plan_fail(UGEMM_ERR_ARG, "NULL operand");
    g[i] = Gemm{ta, tb, q.M, q.N, q.K, q.alpha, q.beta, q.A, q.lda, q.B, q.ldb, q.C, q.ldc};
    g[i].epi.bias = q.bias;
    g[i].epi.act = q.act;
    g[i].epi.slope = q.slope;
  }
  ugemm_tile_config tuned{};
  const ugemm_tile_config* cfg = config;
  if (!cfg && tuned_config(count, problems, form, &tuned)) cfg = &tuned;
  return grouped_plan_build(g.data(), count, form, cfg, flags, out);
}

}  // extern "C"

namespace ugemm {

ugemm_status grouped_plan_build(const Gemm* gs, int count, int form,
                                const ugemm_tile_config* config, int flags,
                                ugemm_grouped_plan** out) {
  *out = nullptr;
  std::vector<Gemm> g(gs, gs + count);
  // longest k first (round-robin tile order then balances better)
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g[a].K > g[b].K; });

  auto* p = new ugemm_grouped_plan_s;
  p->count = count;
  p->form = form;
  if (config) {
    p->cfg = *config;
  } else {
    p->cfg = default_grouped_config(form);
    // Untuned split plans: 128-wide tiles only when no problem is wider than
    // 128 columns in the orientation the kernel computes it (a transposed
    // problem's width is its M); measured on the 256-problem set, 256-wide
    // tiles with the staged epilogue and narrow-N MMAs win (144 vs 162 us).
    if (form != UGEMM_PREC_SIMT) {
      int widest = 0;
      for (const Gemm& x : g)
        widest = std::max(widest,
                          padded_area(x.N, x.M, 128) < padded_area(x.M, x.N, 128) ? x.M : x.N);
      if (widest <= 128) p->cfg.block_n = 128;
    }
  }
  if (form != UGEMM_PREC_SIMT) {
    // fused launches split three bf16 pieces inside the GEMM kernel (128-
    // or 256-wide tiles); other forms ignore the knob
    const bool can_fuse = split_plan_for(form, g[0]).pieces == 3 &&
                          std::all_of(g.begin(), g.end(), fusable);
    if (!(p->cfg.fused && can_fuse)) p->cfg.fused = 0;
    if (p->cfg.block_n != 128 && p->cfg.block_n != 256) p->cfg.block_n = 256;
    if (p->cfg.chunk_k < kTcKB) p->cfg.chunk_k = split_default_chunk_kb(1 << 30) * kTcKB;
  } else {
    p->cfg.fused = 0;
    if (p->cfg.block_n != 64 && p->cfg.block_n != 128) p->cfg.block_n = 128;
  }
  cudaGetDevice(&p->device);
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
  for (const Gemm& x : g) p->flops += 2.0 * x.M * x.N * x.K;

  const bool simt = form == UGEMM_PREC_SIMT;
  const int bn = p->cfg.block_n;
  int pieces = 3;
  if (!simt) {
    p->split = split_plan_for(form, g[0]);
    p->split.block_n = bn;
    p->split.fused = p->cfg.fused != 0;
    pieces = p->split.pieces;
  }
  // Kernel geometry of each problem (in k-depth order j).  The split form
  // computes C^T = op(B)^T op(A)^T when that wastes less of its 128-row
  // tiles (a problem with few rows and many columns); both operands are
  // K-major pieces either way, so only the roles of the maps swap.
  struct Geo {
    bool swap = false;
    int tiles = 0, nkb = 0;  // output tiles, k-blocks (32 deep)
    int slices = 1, per = 0; // split-K slices and their length in k-blocks
  };
  std::vector<Geo> geo(count);
  double work = 0;
  for (int j = 0; j < count; ++j) {
    const Gemm& x = g[order[j]];
    Geo& o = geo[j];
    if (simt) {
      o.tiles = cdiv(x.M, bn) * cdiv(x.N, bn);
      o.nkb = std::max(1, cdiv(x.K, kBK));
    } else {
      o.swap = p->cfg.transpose == 0 && padded_area(x.N, x.M, bn) < padded_area(x.M, x.N, bn);
      const int rows = o.swap ? x.N : x.M, cols = o.swap ? x.M : x.N;
      o.tiles = cdiv(rows, kTcBM) * cdiv(cols, bn);
      o.nkb = split_nkb(pieces, x.K);
    }
    o.per = o.nkb;
    work += double(o.tiles) * o.nkb;
  }
  // Split-K.  The persistent CTAs share the group's tile k-blocks; a problem
  // whose tiles are each longer than half an SM's fair share (a weight
  // gradient: small output, k = batch x pixels) would leave most SMs idle,
  // so it is cut into slices of about that length, at least min_slice
  // k-blocks, and at most 1 GiB of partial tiles.
  // (stages: 16 k-blocks of 32 in the SIMT form and the three-piece split
  // form, 8 of 64 for two-piece operands)
  const int min_slice = 16 * kTcKB / (simt ? kTcKB : split_stage_k(pieces));
  // (the threshold divisor is the configuration's split_k: 0 means 2,
  // negative disables split-K)
  const double fair = p->cfg.split_k < 0 ? 1e300
                                          : work / ((p->cfg.split_k > 0 ? p->cfg.split_k : 2) * sms);
  std::vector<size_t> part_off(count, 0);
  size_t part_bytes = 0;
  for (int j = 0; j < count; ++j) {
    const Gemm& x = g[order[j]];
    Geo& o = geo[j];
    if (x.K == 0 || o.nkb < 2 * min_slice || o.nkb <= fair) continue;
    const int len = std::max(min_slice, static_cast<int>(fair) + 1);
    const size_t tile_bytes = size_t(x.M) * x.N * 4;
    int sl = std::min(cdiv(o.nkb, len), 256);
    sl = static_cast<int>(std::min<size_t>(sl, (size_t(1) << 30) / tile_bytes));
    if (sl < 2) continue;
    o.per = cdiv(o.nkb, sl);
    o.slices = cdiv(o.nkb, o.per);
    part_off[j] = part_bytes;
    part_bytes += align_up(size_t(o.slices) * tile_bytes, 256);
  }

  // scratch: operand slots, then the split-K partial tiles
  std::vector<size_t> a_off(count), b_off(count);
  std::vector<int> ld_a(count), ld_b(count);
  size_t scratch = 0;
  for (int j = 0; j < count; ++j) {
    const Gemm& x = g[order[j]];
    a_off[j] = scratch;
    if (simt) {
      // packed K x M and K x N, rows padded to 16 bytes for TMA
      ld_a[j] = static_cast<int>(align_up(x.M, 4));
      ld_b[j] = static_cast<int>(align_up(x.N, 4));
      scratch += align_up(size_t(std::max(x.K, 1)) * ld_a[j] * 4, 256);
      b_off[j] = scratch;
      scratch += align_up(size_t(std::max(x.K, 1)) * ld_b[j] * 4, 256);
    } else if (p->split.fused) {
      b_off[j] = scratch;  // no pieces in memory: the kernel splits the operands
    } else {
      scratch += split_operand_bytes(pieces, x.M, x.K);
      b_off[j] = scratch;
      scratch += split_operand_bytes(pieces, x.N, x.K);
    }
  }
  const size_t part_base = scratch;
  scratch += part_bytes;
  // fused 256-wide launches: the chunk sums of every persistent CTA
  const size_t sums_base = scratch;
  if (!simt && p->split.fused && bn == 256)
    scratch += size_t(std::max(1, p->cfg.max_ctas > 0 ? p->cfg.max_ctas : sms)) * kTcFusedSumBytes;
  cudaError_t e = cudaMalloc(&p->scratch, std::max<size_t>(scratch, 256));
  // zeroed once: a K == 0 problem's slot is read as one zero k tile
  if (e == cudaSuccess) e = cudaMemset(p->scratch, 0, std::max<size_t>(scratch, 256));
  if (e == cudaSuccess) e = cudaMalloc(&p->dev_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->dev_err, 0, sizeof(int));
  if (e != cudaSuccess) {
    free_plan(p);
    return plan_fail(UGEMM_ERR_ALLOC, "cudaMalloc for the grouped plan failed");
  }
  uint8_t* base = static_cast<uint8_t*>(p->scratch);
  if (!simt && p->split.fused && bn == 256) p->chunk_sums = reinterpret_cast<float*>(base + sums_base);

  // pre-pass jobs: one per operand of every problem
  std::vector<SplitJob> sjobs;
  std::vector<PackJob> pjobs;
  int prep = 0;
  for (int j = 0; j < count; ++j) {
    const Gemm& x = g[order[j]];
    long long a_sr, a_sk, b_sr, b_sk;
    split_operand_strides(x, &a_sr, &a_sk, &b_sr, &b_sk);
    // an implicit im2col B: rows of op(B)^T are pixels ('N') or taps ('T');
    // the thread layout of the rows-of-taps gather is the k-contiguous one
    const int gather = x.b_im2col ? (x.tb == 'N' ? 1 : 2) : 0;
    if (gather) b_sk = gather == 2 ? 1 : 0;
    if (simt) {
      const int tk = cdiv(std::max(x.K, 1), 64);
      pjobs.push_back(PackJob{x.A, a_sr, a_sk, reinterpret_cast<float*>(base + a_off[j]), x.M,
                              x.K, ld_a[j], prep});
      prep += cdiv(x.M, 32) * tk;
      PackJob bj{x.B, b_sr, b_sk, reinterpret_cast<float*>(base + b_off[j]), x.N, x.K, ld_b[j],
                 prep};
      if (gather) { bj.gather = gather; bj.im = *x.b_im2col; }
      pjobs.push_back(bj);
      prep += cdiv(x.N, 32) * tk;
    } else {
      const int kp = split_kp(x.K);
      const int tk = cdiv(kp, 64);
      sjobs.push_back(SplitJob{x.A, a_sr, a_sk, reinterpret_cast<__nv_bfloat16*>(base + a_off[j]),
                               x.M, x.K, kp, prep});
      prep += cdiv(x.M, 32) * tk;
      SplitJob bj{x.B, b_sr, b_sk, reinterpret_cast<__nv_bfloat16*>(base + b_off[j]), x.N, x.K, kp,
                  prep};
      if (gather) { bj.gather = gather; bj.im = *x.b_im2col; }
      sjobs.push_back(bj);  // FP16x3: fmax words are set once the table exists
      prep += cdiv(x.N, 32) * tk;
    }
  }

  // kernel problems: every slice of every problem, longest k first
  struct Sub { int j, kb0, nkb, slice; };
  std::vector<Sub> subs;
  for (int j = 0; j < count; ++j)
    for (int sidx = 0; sidx < geo[j].slices; ++sidx) {
      const int kb0 = sidx * geo[j].per;
      subs.push_back(Sub{j, kb0, std::min(geo[j].per, geo[j].nkb - kb0), sidx});
    }
  std::stable_sort(subs.begin(), subs.end(), [](const Sub& a, const Sub& b) { return a.nkb > b.nkb; });

  std::vector<CUtensorMap> maps(2 * subs.size());
  std::vector<TcProblem> tprobs;
  std::vector<SimtProblem> sprobs;
  std::vector<ReduceJob> rjobs;
  int tiles = 0;
  bool any_epi = false;
  for (size_t i = 0; i < subs.size(); ++i) {
    const Sub& u = subs[i];
    const Gemm& x = g[order[u.j]];
    const Geo& o = geo[u.j];
    // a slice writes alpha * (its partial product) to its partial tile set
    const bool sliced = o.slices > 1;
    float* target = sliced ? reinterpret_cast<float*>(base + part_base + part_off[u.j]) +
                                 size_t(u.slice) * x.M * x.N
                           : x.C;
    const int ldt = sliced ? x.N : x.ldc;
    const float beta = sliced ? 0.f : x.beta;
    const Epilogue epi = sliced ? Epilogue{} : x.epi;
    any_epi |= epi.bias != nullptr || epi.act != 0;
    bool ok;
    if (simt) {
      const float* da = reinterpret_cast<const float*>(base + a_off[u.j]);
      const float* db = reinterpret_cast<const float*>(base + b_off[u.j]);
      ok = simt_encode_grouped(bn == 64 ? kSimt64x64 : kSimt128x128, da, x.M, db, x.N, x.K,
                               ld_a[u.j], ld_b[u.j], &maps[2 * i], &maps[2 * i + 1]);
      SimtProblem sp{target, x.M, x.N, ldt, x.alpha, beta, u.nkb, cdiv(x.M, bn), cdiv(x.N, bn),
                     tiles, epi};
      sp.kt0 = u.kb0;
      tiles += sp.tiles_m * sp.tiles_n;
      sprobs.push_back(sp);
    } else {
      TcProblem tp{};
      if (p->split.fused) {
        // the kernel copies the FP32 operands; its operand a is op(B)^T
        // when the problem is computed transposed
        long long a_sr, a_sk, b_sr, b_sk;
        split_operand_strides(x, &a_sr, &a_sk, &b_sr, &b_sk);
        const int bk = fused_raw_k(bn);
        ok = o.swap ? fused_operand_map(x.B, b_sr, b_sk, x.N, x.K, kTcBM, bk, &maps[2 * i],
                                        &tp.kc_a) &&
                          fused_operand_map(x.A, a_sr, a_sk, x.M, x.K, bn, bk, &maps[2 * i + 1],
                                            &tp.kc_b)
                    : fused_operand_map(x.A, a_sr, a_sk, x.M, x.K, kTcBM, bk, &maps[2 * i],
                                        &tp.kc_a) &&
                          fused_operand_map(x.B, b_sr, b_sk, x.N, x.K, bn, bk, &maps[2 * i + 1],
                                            &tp.kc_b);
      } else {
        const void* da = base + a_off[u.j];
        const void* db = base + b_off[u.j];
        ok = o.swap ? split_encode_maps(pieces, bn, db, x.N, da, x.M, x.K, &maps[2 * i],
                                        &maps[2 * i + 1])
                    : split_encode_maps(pieces, bn, da, x.M, db, x.N, x.K, &maps[2 * i],
                                        &maps[2 * i + 1]);
      }
      tp.C = target;
      tp.M = o.swap ? x.N : x.M;
      tp.N = o.swap ? x.M : x.N;
      tp.ldc = ldt;
      tp.alpha = x.alpha;
      tp.beta = beta;
      tp.nkb = u.nkb;
      tp.tiles_m = cdiv(tp.M, kTcBM);
      tp.tiles_n = cdiv(tp.N, bn);
      tp.tile_start = tiles;
      tp.kb0 = u.kb0;
      tp.swap = o.swap ? 1 : 0;
      tp.map = static_cast<int>(i);
      tp.epi = epi;
      tiles += tp.tiles_m * tp.tiles_n;
      tprobs.push_back(tp);
    }
    if (!ok) {
      free_plan(p);
      return plan_fail(UGEMM_ERR_CUDA, "tensor map encoding failed");
    }
    if (sliced && u.slice == 0) {
      rjobs.push_back(ReduceJob{target, x.C, x.M, x.N, x.ldc, o.slices, x.beta, x.epi});
      p->reduce_max = std::max(p->reduce_max, static_cast<long long>(x.M) * x.N);
    }
  }
  if (!simt) p->split.epi = any_epi;
  p->gemm_tiles = tiles;
  p->prep_tiles = prep;
  p->njobs = 2 * count;
  p->nsub = static_cast<int>(subs.size());
  p->nreduce = static_cast<int>(rjobs.size());

  // one device table: maps (64-byte aligned) | problems | jobs | reduce jobs
  const size_t maps_bytes = maps.size() * sizeof(CUtensorMap);
  const size_t prob_bytes = simt ? sprobs.size() * sizeof(SimtProblem) : tprobs.size() * sizeof(TcProblem);
  const size_t job_bytes = simt ? pjobs.size() * sizeof(PackJob) : sjobs.size() * sizeof(SplitJob);
  const size_t red_bytes = rjobs.size() * sizeof(ReduceJob);
  const size_t off_p = align_up(maps_bytes, 256), off_j = off_p + align_up(prob_bytes, 256);
  const size_t off_r = off_j + align_up(job_bytes, 256);
  // split form: the tile table, dealt to exactly p->grid persistent CTAs
  std::vector<int4> recs;
  if (!simt) {
    p->grid = std::max(1, std::min(tiles, p->cfg.max_ctas > 0 ? p->cfg.max_ctas : sms));
    recs = split_tile_table(tprobs.data(), static_cast<int>(tprobs.size()), bn, p->grid,
                            p->cfg.deal == 1);
  }
  const size_t rec_bytes = recs.size() * sizeof(int4);
  const size_t off_t = off_r + align_up(std::max<size_t>(red_bytes, 1), 256);
  // FP16x3: the largest magnitude of every row of every operand (job q's
  // rows from word_off[q] on), cleared on every run
  const bool f16 = !simt && p->split.f16;
  std::vector<size_t> word_off(sjobs.size() + 1, 0);
  for (size_t q = 0; q < sjobs.size(); ++q) word_off[q + 1] = word_off[q] + sjobs[q].rows;
  const size_t off_w = off_t + align_up(std::max<size_t>(rec_bytes, 1), 256);
  const size_t total =
      off_w + (f16 ? align_up(std::max<size_t>(word_off.back(), 1) * sizeof(unsigned), 256) : 0);
  e = cudaMalloc(&p->table, total);
  if (e != cudaSuccess) {
    free_plan(p);
    return plan_fail(UGEMM_ERR_ALLOC, "grouped plan table allocation failed");
  }
  uint8_t* tb = static_cast<uint8_t*>(p->table);
  if (f16) {  // problem j's row words: job 2j (A) and 2j + 1 (B) fill them, its slices read them
    unsigned* words = reinterpret_cast<unsigned*>(tb + off_w);
    p->fmax = words;
    p->nfmax = static_cast<int>(word_off.back());
    for (size_t q = 0; q < sjobs.size(); ++q) sjobs[q].fmax = words + word_off[q];
    for (size_t i = 0; i < tprobs.size(); ++i) {
      const int j = subs[i].j;
      const bool sw = geo[j].swap;  // kernel operand a is op(B)^T's pieces when swapped
      tprobs[i].fmax_a = words + word_off[2 * j + (sw ? 1 : 0)];
      tprobs[i].fmax_b = words + word_off[2 * j + (sw ? 0 : 1)];
    }
  }
  std::vector<uint8_t> host(total, 0);
  std::memcpy(host.data(), maps.data(), maps_bytes);
  std::memcpy(host.data() + off_p, simt ? static_cast<const void*>(sprobs.data()) : tprobs.data(),
              prob_bytes);
  std::memcpy(host.data() + off_j, simt ? static_cast<const void*>(pjobs.data()) : sjobs.data(),
              job_bytes);
  if (red_bytes) std::memcpy(host.data() + off_r, rjobs.data(), red_bytes);
  if (rec_bytes) std::memcpy(host.data() + off_t, recs.data(), rec_bytes);
  e = cudaMemcpy(p->table, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_plan(p);
    return plan_fail(UGEMM_ERR_ALLOC, "grouped plan table upload failed");
  }
  p->maps = reinterpret_cast<const CUtensorMap*>(tb);
  p->probs = tb + off_p;
  p->jobs = tb + off_j;
  p->reduce = tb + off_r;
  p->tiles = reinterpret_cast<const int4*>(tb + off_t);

  if (flags & UGEMM_PLAN_GRAPH) {
    cudaStream_t cs;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    ugemm_status ls = UGEMM_OK;
    if (e == cudaSuccess) {
      ls = launch_plan(p, cs);
      e = cudaStreamEndCapture(cs, &p->graph);
    }
    if (e == cudaSuccess && ls == UGEMM_OK) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess || ls != UGEMM_OK) {
      free_plan(p);
      return plan_fail(UGEMM_ERR_CUDA, "CUDA graph capture of the grouped plan failed");
    }
  }
  *out = p;
  return UGEMM_OK;
}

}  // namespace ugemm

extern "C" {

UGEMM_API int ugemm_grouped_run(ugemm_grouped_plan* p, void* stream) {
  if (!p) return plan_fail(UGEMM_ERR_ARG, "NULL plan");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (p->exec) {
    cudaError_t e = cudaGraphLaunch(p->exec, st);
    if (e != cudaSuccess) return plan_fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
    return UGEMM_OK;
  }
  ugemm_status s = launch_plan(p, st);
  if (s != UGEMM_OK) return plan_fail(s, "grouped launch failed");
  return UGEMM_OK;
}

UGEMM_API int ugemm_grouped_check(ugemm_grouped_plan* p, void* stream) {
  if (!p) return plan_fail(UGEMM_ERR_ARG, "NULL plan");
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return plan_fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
  int code = 0;
  e = cudaMemcpy(&code, p->dev_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return plan_fail(UGEMM_ERR_CUDA, cudaGetErrorString(e));
  if (code) {
    cudaMemset(p->dev_err, 0, sizeof(int));
    return plan_fail(UGEMM_ERR_TIMEOUT, "grouped kernel wait timed out");
  }
  return UGEMM_OK;
}

UGEMM_API int ugemm_grouped_plan_destroy(ugemm_grouped_plan* p) {
  if (!p) return UGEMM_OK;
  cudaDeviceSynchronize();
  free_plan(p);
  return UGEMM_OK;
}

UGEMM_API double ugemm_grouped_flops(const ugemm_grouped_plan* p) { return p ? p->flops : 0.0; }

UGEMM_API int ugemm_grouped_config(const ugemm_grouped_plan* p, ugemm_tile_config* cfg) {
  if (!p || !cfg) return UGEMM_ERR_ARG;
  *cfg = p->cfg;
  return UGEMM_OK;
}

UGEMM_API int ugemm_sgemm_grouped(int count, const ugemm_problem* problems, int precision,
                                  void* stream) {
  ugemm_grouped_plan* p = nullptr;
  int s = ugemm_grouped_plan_create(count, problems, precision, nullptr, 0, &p);
  if (s != UGEMM_OK) return s;
  s = ugemm_grouped_run(p, stream);
  if (s == UGEMM_OK) s = ugemm_grouped_check(p, stream);
  ugemm_grouped_plan_destroy(p);
  return s;
}

}  // extern "C"
