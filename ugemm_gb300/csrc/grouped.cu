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

struct ugemm_grouped_plan_s {
  int count = 0;
  int form = UGEMM_PREC_SIMT;
  ugemm_tile_config cfg{};
  int device = 0;
  double flops = 0;
  // device memory
  void* table = nullptr;    // maps | problems | jobs
  void* scratch = nullptr;  // operand slots
  int* dev_err = nullptr;
  const CUtensorMap* maps = nullptr;
  const void* probs = nullptr;
  const void* jobs = nullptr;
  int njobs = 0, prep_tiles = 0, gemm_tiles = 0;
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

ugemm_status launch_plan(ugemm_grouped_plan_s* p, cudaStream_t st) {
  ugemm_status s;
  if (p->form == UGEMM_PREC_SIMT) {
    s = pack_batched_launch(static_cast<const PackJob*>(p->jobs), p->njobs, p->prep_tiles, st);
    if (s != UGEMM_OK) return s;
    const int tile = p->cfg.block_n == 64 ? kSimt64x64 : kSimt128x128;
    return simt_grouped_launch(tile, p->maps, static_cast<const SimtProblem*>(p->probs), p->count,
                               p->gemm_tiles, p->cfg.max_ctas, p->dev_err, st);
  }
  s = split_batched_launch(p->split.pieces, static_cast<const SplitJob*>(p->jobs), p->njobs,
                           p->prep_tiles, st);
  if (s != UGEMM_OK) return s;
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof dummy);
  TcProblem single{};
  return split_gemm_launch(p->split, dummy, dummy, single, p->maps,
                           static_cast<const TcProblem*>(p->probs), p->count, p->gemm_tiles,
                           std::max(1, p->cfg.chunk_k / kTcKB), p->cfg.max_ctas, p->dev_err, st);
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
    c.chunk_k = split_default_chunk_kb() * kTcKB;
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
  if (form < UGEMM_PREC_SIMT || form > UGEMM_PREC_BF16X3)
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
  // longest k first (round-robin tile order then balances better)
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g[a].K > g[b].K; });

  auto* p = new ugemm_grouped_plan_s;
  p->count = count;
  p->form = form;
  if (config) {
    p->cfg = *config;
  } else if (!tuned_config(count, problems, form, &p->cfg)) {
    p->cfg = default_grouped_config(form);
    // Untuned split plans: 256-wide tiles only pay when the problems are wide
    // (measured: 128 wins on the 256-problem set with N in [32, 1024]).
    if (form != UGEMM_PREC_SIMT) {
      double n_sum = 0;
      for (const Gemm& x : g) n_sum += x.N;
      if (n_sum / count < 512) p->cfg.block_n = 128;
    }
  }
  if (form != UGEMM_PREC_SIMT) {
    if (p->cfg.block_n != 128 && p->cfg.block_n != 256) p->cfg.block_n = 256;
    if (p->cfg.chunk_k < kTcKB) p->cfg.chunk_k = split_default_chunk_kb() * kTcKB;
  } else if (p->cfg.block_n != 64 && p->cfg.block_n != 128) {
    p->cfg.block_n = 128;
  }
  cudaGetDevice(&p->device);
  for (const Gemm& x : g) p->flops += 2.0 * x.M * x.N * x.K;

  const bool simt = form == UGEMM_PREC_SIMT;
  // scratch slots
  std::vector<size_t> a_off(count), b_off(count);
  size_t scratch = 0;
  int pieces = 3;
  if (!simt) {
    p->split = split_plan_for(form, g[0]);
    p->split.block_n = p->cfg.block_n;
    p->split.epi = false;
    for (const Gemm& x : g) p->split.epi |= x.epi.bias != nullptr || x.epi.act != 0;
    pieces = p->split.pieces;
  }
  std::vector<int> ld_a(count), ld_b(count);
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
    } else {
      scratch += split_operand_bytes(pieces, x.M, x.K);
      b_off[j] = scratch;
      scratch += split_operand_bytes(pieces, x.N, x.K);
    }
  }
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

  // host tables
  std::vector<CUtensorMap> maps(2 * count);
  std::vector<TcProblem> tprobs;
  std::vector<SimtProblem> sprobs;
  std::vector<SplitJob> sjobs;
  std::vector<PackJob> pjobs;
  int tiles = 0, prep = 0;
  for (int j = 0; j < count; ++j) {
    const Gemm& x = g[order[j]];
    long long a_sr, a_sk, b_sr, b_sk;
    split_operand_strides(x, &a_sr, &a_sk, &b_sr, &b_sk);
    bool ok;
    if (simt) {
      float* da = reinterpret_cast<float*>(base + a_off[j]);
      float* db = reinterpret_cast<float*>(base + b_off[j]);
      const int tk = cdiv(std::max(x.K, 1), 64);
      pjobs.push_back(PackJob{x.A, a_sr, a_sk, da, x.M, x.K, ld_a[j], prep});
      prep += cdiv(x.M, 32) * tk;
      pjobs.push_back(PackJob{x.B, b_sr, b_sk, db, x.N, x.K, ld_b[j], prep});
      prep += cdiv(x.N, 32) * tk;
      ok = simt_encode_grouped(p->cfg.block_n == 64 ? kSimt64x64 : kSimt128x128, da, x.M, db,
                               x.N, x.K, ld_a[j], ld_b[j], &maps[2 * j], &maps[2 * j + 1]);
      const int bm = p->cfg.block_n;
      SimtProblem sp{x.C, x.M, x.N, x.ldc, x.alpha, x.beta, cdiv(x.K, kBK), cdiv(x.M, bm),
                     cdiv(x.N, bm), tiles, x.epi};
      if (x.K == 0) sp.nkt = 1;  // one zero-filled k tile keeps the pipeline uniform
      tiles += sp.tiles_m * sp.tiles_n;
      sprobs.push_back(sp);
    } else {
      auto* da = reinterpret_cast<__nv_bfloat16*>(base + a_off[j]);
      auto* db = reinterpret_cast<__nv_bfloat16*>(base + b_off[j]);
      const int kp = split_kp(x.K);
      const int tk = cdiv(kp, 64);
      sjobs.push_back(SplitJob{x.A, a_sr, a_sk, da, x.M, x.K, kp, prep});
      prep += cdiv(x.M, 32) * tk;
      sjobs.push_back(SplitJob{x.B, b_sr, b_sk, db, x.N, x.K, kp, prep});
      prep += cdiv(x.N, 32) * tk;
      ok = split_encode_maps(pieces, p->cfg.block_n, da, x.M, db, x.N, x.K, &maps[2 * j],
                             &maps[2 * j + 1]);
      TcProblem tp = split_problem(x, p->cfg.block_n, tiles);
      tiles += tp.tiles_m * tp.tiles_n;
      tprobs.push_back(tp);
    }
    if (!ok) {
      free_plan(p);
      return plan_fail(UGEMM_ERR_CUDA, "tensor map encoding failed");
    }
  }
  p->gemm_tiles = tiles;
  p->prep_tiles = prep;
  p->njobs = 2 * count;

  // one device table: maps (64-byte aligned) | problems | jobs
  const size_t maps_bytes = maps.size() * sizeof(CUtensorMap);
  const size_t prob_bytes = simt ? sprobs.size() * sizeof(SimtProblem) : tprobs.size() * sizeof(TcProblem);
  const size_t job_bytes = simt ? pjobs.size() * sizeof(PackJob) : sjobs.size() * sizeof(SplitJob);
  const size_t off_p = align_up(maps_bytes, 256), off_j = off_p + align_up(prob_bytes, 256);
  const size_t total = off_j + align_up(job_bytes, 256);
  std::vector<uint8_t> host(total, 0);
  std::memcpy(host.data(), maps.data(), maps_bytes);
  std::memcpy(host.data() + off_p, simt ? static_cast<const void*>(sprobs.data()) : tprobs.data(),
              prob_bytes);
  std::memcpy(host.data() + off_j, simt ? static_cast<const void*>(pjobs.data()) : sjobs.data(),
              job_bytes);
  e = cudaMalloc(&p->table, total);
  if (e == cudaSuccess) e = cudaMemcpy(p->table, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_plan(p);
    return plan_fail(UGEMM_ERR_ALLOC, "grouped plan table upload failed");
  }
  uint8_t* tb = static_cast<uint8_t*>(p->table);
  p->maps = reinterpret_cast<const CUtensorMap*>(tb);
  p->probs = tb + off_p;
  p->jobs = tb + off_j;

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
