// pipeline.cu -- overlapped host <-> device copies for the host-pointer API.
//
// The reference's sgemm_ocl (sgemm_ocl2.h:166-219) writes A, B (and C) to the
// device, runs the kernel and reads C back, one blocking step after another,
// and the reference's benchmarks time all of it (sgemm_test.c:229-232).
// Here a large host-pointer GEMM is cut into row bands of C:
//   * B is copied once, and split once into bf16 pieces for the tensor-core
//     form;
//   * band i's rows of op(A) (and of C when beta != 0) travel on a copy
//     stream while band i-1 is computed and band i-2 is copied back, through
//     two device slots per operand;
//   * consecutive bands run on two compute streams, so a band's first CTAs
//     start while the previous band's last wave is still running.
// The result equals the unbanded call: every C row band is an independent
// GEMM of the same operands.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "internal.h"
#include "split_tc.cuh"

namespace ugemm {
namespace {

struct PipeState {
  bool ready = false;
  cudaStream_t h2d = nullptr, d2h = nullptr, comp[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> events;
};

constexpr int kMaxBands = 64;
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
    p.events.resize(3 * kMaxBands + 2);
    for (auto& e : p.events)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return UGEMM_ERR_CUDA;
    p.ready = true;
  }
  *out = &p;
  return UGEMM_OK;
}

bool is_split(int form) {
  return form == UGEMM_PREC_BF16X6 || form == UGEMM_PREC_BF16X9 || form == UGEMM_PREC_BF16X3;
}

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
  // SIMT bands read the device copies through TMA: they need 16-byte pitches.
  if (!split && ((g.ldb & 3) != 0 || (g.ta == 'N' && (g.lda & 3) != 0)))
    return UGEMM_ERR_UNSUPPORTED;

  // bands of C rows: about eight, whole 128-row tiles
  const int band = static_cast<int>(align_up(std::max(512, cdiv(g.M, 8)), 128));
  const int nb = cdiv(g.M, band);
  if (nb < 2 || nb > kMaxBands) return UGEMM_ERR_UNSUPPORTED;

  SplitPlan plan{};
  if (split) plan = split_plan_for(form, g);
  // device layout: B | 2 x (A band | C band) | [B pieces | 2 x A band pieces]
  const int band_p = static_cast<int>(align_up(band, 4));        // pitch of a 'T' A band
  const size_t a_band_elems = g.ta == 'N' ? size_t(band) * g.lda : size_t(g.K) * band_p;
  const int ldc_d = static_cast<int>(align_up(g.N, 4));
  const size_t b_bytes = align_up(b_rows * g.ldb * 4, 256);
  const size_t a_slot = align_up(a_band_elems * 4, 256);
  const size_t c_slot = align_up(size_t(band) * ldc_d * 4, 256);
  const size_t bp_bytes = split ? split_operand_bytes(plan.pieces, g.N, g.K) : 0;
  const size_t ap_slot = split ? split_operand_bytes(plan.pieces, band, g.K) : 0;
  const size_t need = b_bytes + 2 * (a_slot + c_slot) + bp_bytes + 2 * ap_slot;
  if (need > arena_bytes) return UGEMM_ERR_UNSUPPORTED;

  std::lock_guard<std::mutex> lock(g_pmu);
  PipeState* ps = nullptr;
  if (pipe_state(&ps) != UGEMM_OK) return UGEMM_ERR_CUDA;
  uint8_t* base = static_cast<uint8_t*>(arena);
  float* dB = reinterpret_cast<float*>(base);
  float* dA[2];
  float* dC[2];
  void* dAp[2] = {nullptr, nullptr};
  size_t off = b_bytes;
  for (int s = 0; s < 2; ++s) {
    dA[s] = reinterpret_cast<float*>(base + off);
    off += a_slot;
    dC[s] = reinterpret_cast<float*>(base + off);
    off += c_slot;
  }
  void* dBp = base + off;
  off += bp_bytes;
  for (int s = 0; s < 2; ++s) {
    dAp[s] = base + off;
    off += ap_slot;
  }
  cudaEvent_t* ev_h2d = &ps->events[0];
  cudaEvent_t* ev_comp = &ps->events[kMaxBands];
  cudaEvent_t* ev_d2h = &ps->events[2 * kMaxBands];
  cudaEvent_t ev_b = ps->events[3 * kMaxBands], ev_bsplit = ps->events[3 * kMaxBands + 1];
  auto ck = [](cudaError_t e) { return e == cudaSuccess; };

  // work queued earlier on the caller's stream comes first
  if (!ck(cudaEventRecord(ev_b, caller)) || !ck(cudaStreamWaitEvent(ps->h2d, ev_b, 0)))
    return UGEMM_ERR_CUDA;
  if (!ck(cudaMemcpyAsync(dB, g.B, ((b_rows - 1) * g.ldb + b_cols) * 4, cudaMemcpyHostToDevice,
                          ps->h2d)) ||
      !ck(cudaEventRecord(ev_b, ps->h2d)))
    return UGEMM_ERR_CUDA;
  cudaStreamWaitEvent(ps->comp[0], ev_b, 0);
  if (split) {
    const long long b_sr = g.tb == 'N' ? 1 : g.ldb, b_sk = g.tb == 'N' ? g.ldb : 1;
    if (split_operand_launch(plan.pieces, dB, b_sr, b_sk, g.N, g.K, dBp, ps->comp[0]) != UGEMM_OK)
      return UGEMM_ERR_CUDA;
  }
  cudaEventRecord(ev_bsplit, ps->comp[0]);
  cudaStreamWaitEvent(ps->comp[1], ev_bsplit, 0);

  for (int i = 0; i < nb; ++i) {
    const int s = i & 1;
    const int m0 = i * band, mb = std::min(band, g.M - m0);
    cudaStream_t cs = ps->comp[s];
    if (i >= 2) cudaStreamWaitEvent(ps->h2d, ev_d2h[i - 2], 0);  // both slots free again
    bool ok;
    if (g.ta == 'N') {
      ok = ck(cudaMemcpyAsync(dA[s], g.A + size_t(m0) * g.lda,
                              ((size_t(mb) - 1) * g.lda + g.K) * 4, cudaMemcpyHostToDevice,
                              ps->h2d));
    } else {  // columns m0 .. m0+mb of the K x M operand
      ok = ck(cudaMemcpy2DAsync(dA[s], size_t(band_p) * 4, g.A + m0, size_t(g.lda) * 4,
                                size_t(mb) * 4, g.K, cudaMemcpyHostToDevice, ps->h2d));
    }
    if (ok && g.beta != 0.f)  // beta == 0: C is not read (sgemm_ocl2.h:177)
      ok = ck(cudaMemcpy2DAsync(dC[s], size_t(ldc_d) * 4, g.C + size_t(m0) * g.ldc,
                                size_t(g.ldc) * 4, size_t(g.N) * 4, mb, cudaMemcpyHostToDevice,
                                ps->h2d));
    if (!ok || !ck(cudaEventRecord(ev_h2d[i], ps->h2d))) return UGEMM_ERR_CUDA;

    cudaStreamWaitEvent(cs, ev_h2d[i], 0);
    Gemm gb = g;
    gb.M = mb;
    gb.A = dA[s];
    gb.lda = g.ta == 'N' ? g.lda : band_p;
    gb.B = dB;
    gb.C = dC[s];
    if (gb.epi.bias) gb.epi.bias += m0;  // per-row bias follows the band
    gb.ldc = ldc_d;
    ugemm_status st;
    if (split) {
      const long long a_sr = gb.ta == 'N' ? gb.lda : 1, a_sk = gb.ta == 'N' ? 1 : gb.lda;
      st = split_operand_launch(plan.pieces, gb.A, a_sr, a_sk, mb, g.K, dAp[s], cs);
      if (st == UGEMM_OK) st = split_gemm_on_pieces(gb, plan, dAp[s], dBp, dev_err, cs);
    } else {
      st = simt_launch(gb, simt_pick_tile(gb), Scratch{nullptr, 0}, dev_err, cs);
    }
    if (st != UGEMM_OK || !ck(cudaEventRecord(ev_comp[i], cs))) return UGEMM_ERR_CUDA;

    cudaStreamWaitEvent(ps->d2h, ev_comp[i], 0);
    if (!ck(cudaMemcpy2DAsync(g.C + size_t(m0) * g.ldc, size_t(g.ldc) * 4, dC[s],
                              size_t(ldc_d) * 4, size_t(g.N) * 4, mb, cudaMemcpyDeviceToHost,
                              ps->d2h)) ||
        !ck(cudaEventRecord(ev_d2h[i], ps->d2h)))
      return UGEMM_ERR_CUDA;
  }
  // the caller's stream resumes after the last copy back
  cudaStreamWaitEvent(caller, ev_d2h[nb - 1], 0);
  return cudaStreamSynchronize(ps->d2h) == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace ugemm
