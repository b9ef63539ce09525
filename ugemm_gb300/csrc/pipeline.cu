// pipeline.cu -- overlapped host <-> device copies for the host-pointer API.
//
// The reference's sgemm_ocl (sgemm_ocl2.h:166-219) writes A, B (and C) to the
// device, runs the kernel and reads C back, one blocking step after another,
// and the reference's benchmarks time all of it (sgemm_test.c:229-232).
// Here a large host-pointer GEMM is cut into blocks of C: row bands of op(A)
// times column parts of op(B).  Every block is an independent GEMM of the
// same operands, so the result equals the unblocked call.
//   * copies go out, on one stream, in the order the blocks need them:
//     band s of A, part s of B, each followed by the C blocks (when
//     beta != 0) of the blocks it completes; so the first GEMM starts after
//     one band of A and one part of B have crossed the host link, not after
//     all of B, and after 2s operand copies s^2 blocks can run;
//   * each band of A and each part of B is split into bf16 pieces once
//     (tensor-core form) by the first block that uses it;
//   * blocks run on two compute streams, so one block's first tiles start
//     while the previous block's last tiles are still running, and each
//     finished block of C goes back on its own stream while later blocks
//     compute.
// Device staging: all bands of A and parts of B (and their pieces), four
// block slots of C, all with 16-byte pitches so that TMA can describe them
// whatever the host leading dimensions are.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "internal.h"
#include "split_tc.cuh"

namespace ugemm {
namespace {

constexpr int kMaxBands = 8, kMaxParts = 8, kMaxBlocks = kMaxBands * kMaxParts;
constexpr int kCSlots = 4;

struct PipeState {
  bool ready = false;
  cudaStream_t h2d = nullptr, d2h = nullptr, comp[2] = {nullptr, nullptr};
  // per band: A copied, A split, all blocks computed; per part: B copied, B
  // split; per block: C copied, computed, copied back; plus one entry event
  cudaEvent_t a_in[kMaxBands], a_split[kMaxBands], b_in[kMaxParts], b_split[kMaxParts];
  cudaEvent_t c_in[kMaxBlocks], comp_done[kMaxBlocks], c_out[kMaxBlocks], entry;
};

std::mutex g_pmu;
PipeState g_pipe[64];

ugemm_status pipe_state(PipeState** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return UGEMM_ERR_CUDA;
  PipeState& p = g_pipe[dev];
  if (!p.ready) {
    const unsigned fl = cudaStreamNonBlocking;
    if (cudaStreamCreateWithFlags(&p.h2d, fl) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p.d2h, fl) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p.comp[0], fl) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p.comp[1], fl) != cudaSuccess)
      return UGEMM_ERR_CUDA;
    std::vector<cudaEvent_t*> all = {&p.entry};
    for (int i = 0; i < kMaxBands; ++i) { all.push_back(&p.a_in[i]); all.push_back(&p.a_split[i]); }
    for (int j = 0; j < kMaxParts; ++j) { all.push_back(&p.b_in[j]); all.push_back(&p.b_split[j]); }
    for (int b = 0; b < kMaxBlocks; ++b) {
      all.push_back(&p.c_in[b]);
      all.push_back(&p.comp_done[b]);
      all.push_back(&p.c_out[b]);
    }
    for (cudaEvent_t* e : all)
      if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return UGEMM_ERR_CUDA;
    p.ready = true;
  }
  *out = &p;
  return UGEMM_OK;
}

bool is_split(int form) {
  return form == UGEMM_PREC_BF16X6 || form == UGEMM_PREC_BF16X9 || form == UGEMM_PREC_BF16X3;
}

int pitch4(int n) { return static_cast<int>(align_up(n, 4)); }

}  // namespace

ugemm_status host_gemm_pipelined(const Gemm& g, int form, void* arena, size_t arena_bytes,
                                 int* dev_err, cudaStream_t caller) {
  const bool split = is_split(form);
  if (!split && form != UGEMM_PREC_SIMT) return UGEMM_ERR_UNSUPPORTED;
  if (g.K == 0 || g.alpha == 0.f || g.M < 1024) return UGEMM_ERR_UNSUPPORTED;
  const size_t a_rows = g.ta == 'N' ? g.M : g.K, a_cols = g.ta == 'N' ? g.K : g.M;
  const size_t b_rows = g.tb == 'N' ? g.K : g.N, b_cols = g.tb == 'N' ? g.N : g.K;
  const size_t bytes = 4 * (a_rows * a_cols + b_rows * b_cols + size_t(g.M) * g.N);
  if (bytes < (size_t(64) << 20)) return UGEMM_ERR_UNSUPPORTED;

  // blocks: about four bands of whole 128-row tiles times about four parts
  // of whole 256-column tiles
  int band = static_cast<int>(align_up(std::max(512, cdiv(g.M, 4)), 128));
  while (cdiv(g.M, band) > kMaxBands) band += 128;
  int part = static_cast<int>(align_up(std::max(1024, cdiv(g.N, 4)), 256));
  while (cdiv(g.N, part) > kMaxParts) part += 256;
  const int nb = cdiv(g.M, band), npart = cdiv(g.N, part);
  if (nb < 2) return UGEMM_ERR_UNSUPPORTED;

  SplitPlan plan{};
  if (split) plan = split_plan_for(form, g);
  // device pitches (floats) and slot sizes
  const int lda_d = g.ta == 'N' ? pitch4(g.K) : pitch4(band);   // band: band x K or K x band
  const int ldb_d = g.tb == 'N' ? pitch4(part) : pitch4(g.K);   // part: K x part or part x K
  const int ldc_d = pitch4(part);
  const size_t a_slot = align_up(size_t(g.ta == 'N' ? band : g.K) * lda_d * 4, 256);
  const size_t b_slot = align_up(size_t(g.tb == 'N' ? g.K : part) * ldb_d * 4, 256);
  const size_t c_slot = align_up(size_t(band) * ldc_d * 4, 256);
  const size_t ap_slot = split ? split_operand_bytes(plan.pieces, band, g.K) : 0;
  const size_t bp_slot = split ? split_operand_bytes(plan.pieces, part, g.K) : 0;
  const size_t need = npart * (b_slot + bp_slot) + nb * (a_slot + ap_slot) + kCSlots * c_slot;
  if (need > arena_bytes) return UGEMM_ERR_UNSUPPORTED;

  std::lock_guard<std::mutex> lock(g_pmu);
  PipeState* ps = nullptr;
  if (pipe_state(&ps) != UGEMM_OK) return UGEMM_ERR_CUDA;
  uint8_t* base = static_cast<uint8_t*>(arena);
  size_t off = 0;
  auto take = [&](size_t n) { uint8_t* p = base + off; off += n; return p; };
  float* dB[kMaxParts];
  void* dBp[kMaxParts] = {};
  for (int j = 0; j < npart; ++j) {
    dB[j] = reinterpret_cast<float*>(take(b_slot));
    if (split) dBp[j] = take(bp_slot);
  }
  float* dA[kMaxBands];
  void* dAp[kMaxBands] = {};
  for (int s = 0; s < nb; ++s) {
    dA[s] = reinterpret_cast<float*>(take(a_slot));
    if (split) dAp[s] = take(ap_slot);
  }
  float* dC[kCSlots];
  for (int s = 0; s < kCSlots; ++s) dC[s] = reinterpret_cast<float*>(take(c_slot));
  auto ck = [](cudaError_t e) { return e == cudaSuccess; };

  // work queued earlier on the caller's stream comes first
  if (!ck(cudaEventRecord(ps->entry, caller))) return UGEMM_ERR_CUDA;
  for (cudaStream_t s : {ps->h2d, ps->d2h, ps->comp[0], ps->comp[1]})
    if (!ck(cudaStreamWaitEvent(s, ps->entry, 0))) return UGEMM_ERR_CUDA;

  bool a_split_done[kMaxBands] = {}, b_split_done[kMaxParts] = {};
  auto copy_a = [&](int i) {
    const int m0 = i * band, mb = std::min(band, g.M - m0);
    bool ok;
    if (g.ta == 'N')  // rows m0 .. m0+mb of the M x K operand
      ok = ck(cudaMemcpy2DAsync(dA[i], size_t(lda_d) * 4, g.A + size_t(m0) * g.lda,
                                size_t(g.lda) * 4, size_t(g.K) * 4, mb, cudaMemcpyHostToDevice,
                                ps->h2d));
    else              // columns m0 .. m0+mb of the K x M operand
      ok = ck(cudaMemcpy2DAsync(dA[i], size_t(lda_d) * 4, g.A + m0, size_t(g.lda) * 4,
                                size_t(mb) * 4, g.K, cudaMemcpyHostToDevice, ps->h2d));
    return ok && ck(cudaEventRecord(ps->a_in[i], ps->h2d));
  };
  auto copy_b = [&](int j) {
    const int n0 = j * part, nw = std::min(part, g.N - n0);
    bool ok;
    if (g.tb == 'N')  // columns n0 .. n0+nw of the K x N operand
      ok = ck(cudaMemcpy2DAsync(dB[j], size_t(ldb_d) * 4, g.B + n0, size_t(g.ldb) * 4,
                                size_t(nw) * 4, g.K, cudaMemcpyHostToDevice, ps->h2d));
    else              // rows n0 .. n0+nw of the N x K operand
      ok = ck(cudaMemcpy2DAsync(dB[j], size_t(ldb_d) * 4, g.B + size_t(n0) * g.ldb,
                                size_t(g.ldb) * 4, size_t(g.K) * 4, nw, cudaMemcpyHostToDevice,
                                ps->h2d));
    return ok && ck(cudaEventRecord(ps->b_in[j], ps->h2d));
  };
  int blk = 0;
  auto run_block = [&](int i, int j) -> ugemm_status {
    const int m0 = i * band, mb = std::min(band, g.M - m0);
    const int n0 = j * part, nw = std::min(part, g.N - n0), cs_slot = blk % kCSlots;
    cudaStream_t cs = ps->comp[blk & 1];
    // block (i, j) of C into its slot once the slot's previous block is home
    if (blk >= kCSlots) cudaStreamWaitEvent(ps->h2d, ps->c_out[blk - kCSlots], 0);
    if (g.beta != 0.f &&  // beta == 0: C is not read (sgemm_ocl2.h:177)
        !ck(cudaMemcpy2DAsync(dC[cs_slot], size_t(ldc_d) * 4, g.C + size_t(m0) * g.ldc + n0,
                              size_t(g.ldc) * 4, size_t(nw) * 4, mb, cudaMemcpyHostToDevice,
                              ps->h2d)))
      return UGEMM_ERR_CUDA;
    if (!ck(cudaEventRecord(ps->c_in[blk], ps->h2d))) return UGEMM_ERR_CUDA;
    // operands: the band's and the part's pieces, split by their first user
    if (!a_split_done[i]) {
      cudaStreamWaitEvent(cs, ps->a_in[i], 0);
      if (split) {
        const long long sr = g.ta == 'N' ? lda_d : 1, sk = g.ta == 'N' ? 1 : lda_d;
        if (split_operand_launch(plan.pieces, dA[i], sr, sk, mb, g.K, dAp[i], cs) != UGEMM_OK)
          return UGEMM_ERR_CUDA;
      }
      cudaEventRecord(ps->a_split[i], cs);
      a_split_done[i] = true;
    } else {
      cudaStreamWaitEvent(cs, ps->a_split[i], 0);
    }
    if (!b_split_done[j]) {
      cudaStreamWaitEvent(cs, ps->b_in[j], 0);
      if (split) {
        const long long sr = g.tb == 'N' ? 1 : ldb_d, sk = g.tb == 'N' ? ldb_d : 1;
        if (split_operand_launch(plan.pieces, dB[j], sr, sk, nw, g.K, dBp[j], cs) != UGEMM_OK)
          return UGEMM_ERR_CUDA;
      }
      cudaEventRecord(ps->b_split[j], cs);
      b_split_done[j] = true;
    } else {
      cudaStreamWaitEvent(cs, ps->b_split[j], 0);
    }
    cudaStreamWaitEvent(cs, ps->c_in[blk], 0);
    Gemm gb = g;
    gb.M = mb;
    gb.N = nw;
    gb.A = dA[i];
    gb.lda = lda_d;
    gb.B = dB[j];
    gb.ldb = ldb_d;
    gb.C = dC[cs_slot];
    gb.ldc = ldc_d;
    if (gb.epi.bias) gb.epi.bias += m0;  // per-row bias follows the band
    ugemm_status st;
    if (split) st = split_gemm_on_pieces(gb, plan, dAp[i], dBp[j], dev_err, cs);
    else st = simt_launch(gb, simt_pick_tile(gb), Scratch{nullptr, 0}, dev_err, cs);
    if (st != UGEMM_OK || !ck(cudaEventRecord(ps->comp_done[blk], cs))) return UGEMM_ERR_CUDA;
    cudaStreamWaitEvent(ps->d2h, ps->comp_done[blk], 0);
    if (!ck(cudaMemcpy2DAsync(g.C + size_t(m0) * g.ldc + n0, size_t(g.ldc) * 4, dC[cs_slot],
                              size_t(ldc_d) * 4, size_t(nw) * 4, mb, cudaMemcpyDeviceToHost,
                              ps->d2h)) ||
        !ck(cudaEventRecord(ps->c_out[blk], ps->d2h)))
      return UGEMM_ERR_CUDA;
    ++blk;
    return UGEMM_OK;
  };
  // shells: band s of A, the blocks it completes with the parts already in,
  // then part s of B and the blocks it completes -- after 2s copies of
  // operands, s^2 blocks can run
  for (int s = 0; s < std::max(nb, npart); ++s) {
    if (s < nb) {
      if (!copy_a(s)) return UGEMM_ERR_CUDA;
      for (int j = 0; j < std::min(s, npart); ++j)
        if (run_block(s, j) != UGEMM_OK) return UGEMM_ERR_CUDA;
    }
    if (s < npart) {
      if (!copy_b(s)) return UGEMM_ERR_CUDA;
      for (int i = 0; i <= std::min(s, nb - 1); ++i)
        if (run_block(i, s) != UGEMM_OK) return UGEMM_ERR_CUDA;
    }
  }
  // the caller's stream resumes after the last copy back
  cudaStreamWaitEvent(caller, ps->c_out[blk - 1], 0);
  return cudaStreamSynchronize(ps->d2h) == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace ugemm
