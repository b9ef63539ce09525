// tune.cu -- autotuner for grouped GEMM plans (the reference has none: its
// tile parameters were pasted from an offline CLTune run, sgemm_ocl.h:14-31).
//
// Candidates are timed on the current device with CUDA events after a
// warm-up, the fastest wins, and the choice is appended to a JSON-lines
// cache keyed by device, form and a signature of the problem list, so a
// later ugemm_grouped_plan_create(config = NULL) for the same problem set
// picks it up without timing.
#include <cuda_runtime.h>

#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace ugemm {
namespace {

std::mutex g_tmu;

std::string cache_path() {
  const char* e = std::getenv("UGEMM_TUNE_CACHE");
  return e && *e ? std::string(e) : std::string("ugemm_tune_cache.jsonl");
}

std::string device_key() {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string name(prop.name);
  for (char& c : name)
    if (c == '"' || c == ' ') c = '_';
  return name + "_sm" + std::to_string(prop.multiProcessorCount);
}

uint64_t signature(int count, const ugemm_problem* q, int form) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xff;
      h *= 1099511628211ull;
    }
  };
  mix(static_cast<uint64_t>(count));
  mix(static_cast<uint64_t>(form));
  for (int i = 0; i < count; ++i) {
    mix(static_cast<uint64_t>(q[i].transa) | (static_cast<uint64_t>(q[i].transb) << 8));
    mix(static_cast<uint64_t>(q[i].M) | (static_cast<uint64_t>(q[i].N) << 32));
    mix(static_cast<uint64_t>(q[i].K));
  }
  return h;
}

bool lookup(const std::string& dev, int form, uint64_t sig, ugemm_tile_config* cfg, double* ms) {
  FILE* f = std::fopen(cache_path().c_str(), "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char d[128];
    int fm = 0, bn = 0, ck = 0, mc = 0;
    uint64_t s = 0;
    double t = 0;
    if (std::sscanf(line,
                    "{\"device\": \"%127[^\"]\", \"form\": %d, \"sig\": \"%" SCNx64
                    "\", \"block_n\": %d, \"chunk_k\": %d, \"max_ctas\": %d, \"ms\": %lf}",
                    d, &fm, &s, &bn, &ck, &mc, &t) == 7 &&
        dev == d && fm == form && s == sig) {
      cfg->block_n = bn;
      cfg->chunk_k = ck;
      cfg->max_ctas = mc;
      if (ms) *ms = t;
      found = true;  // the last matching line wins
    }
  }
  std::fclose(f);
  return found;
}

void store(const std::string& dev, int form, uint64_t sig, const ugemm_tile_config& c, double ms) {
  FILE* f = std::fopen(cache_path().c_str(), "a");
  if (!f) return;
  std::fprintf(f,
               "{\"device\": \"%s\", \"form\": %d, \"sig\": \"%016" PRIx64
               "\", \"block_n\": %d, \"chunk_k\": %d, \"max_ctas\": %d, \"ms\": %.6f}\n",
               dev.c_str(), form, sig, c.block_n, c.chunk_k, c.max_ctas, ms);
  std::fclose(f);
}

int norm_form(int precision) { return precision == UGEMM_PREC_AUTO ? UGEMM_PREC_BF16X6 : precision; }

}  // namespace

bool tuned_config(int count, const ugemm_problem* problems, int precision,
                  ugemm_tile_config* cfg) {
  std::lock_guard<std::mutex> l(g_tmu);
  const int form = norm_form(precision);
  return lookup(device_key(), form, signature(count, problems, form), cfg, nullptr);
}

}  // namespace ugemm

using namespace ugemm;

extern "C" {

UGEMM_API int ugemm_tune_grouped(int count, const ugemm_problem* problems, int precision,
                                 int force, ugemm_tile_config* best, double* best_ms) {
  if (!best || count <= 0 || !problems) return UGEMM_ERR_ARG;
  const int form = norm_form(precision);
  const std::string dev = device_key();
  const uint64_t sig = signature(count, problems, form);
  if (!force) {
    std::lock_guard<std::mutex> l(g_tmu);
    if (lookup(dev, form, sig, best, best_ms)) return UGEMM_OK;
  }
  std::vector<ugemm_tile_config> cands;
  if (form == UGEMM_PREC_SIMT) {
    for (int bn : {64, 128}) cands.push_back(ugemm_tile_config{bn, 0, 0});
  } else {
    // chunk_k <= 256 keeps the split form at least as accurate as FP32 SIMT
    for (int bn : {128, 256})
      for (int ck : {128, 256}) cands.push_back(ugemm_tile_config{bn, ck, 0});
  }
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return UGEMM_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_t = 1e30;
  int rc = UGEMM_ERR_UNSUPPORTED;
  for (const auto& c : cands) {
    ugemm_grouped_plan* p = nullptr;
    if (ugemm_grouped_plan_create(count, problems, form, &c, 0, &p) != UGEMM_OK) continue;
    bool ok = true;
    for (int w = 0; w < 2 && ok; ++w) ok = ugemm_grouped_run(p, st) == UGEMM_OK;
    const int reps = 5;
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps && ok; ++r) ok = ugemm_grouped_run(p, st) == UGEMM_OK;
    cudaEventRecord(e1, st);
    ok = ok && ugemm_grouped_check(p, st) == UGEMM_OK;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ugemm_grouped_plan_destroy(p);
    if (!ok) continue;
    const double t = ms / reps;
    if (t < best_t) {
      best_t = t;
      *best = c;
      rc = UGEMM_OK;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  if (rc == UGEMM_OK) {
    if (best_ms) *best_ms = best_t;
    std::lock_guard<std::mutex> l(g_tmu);
    store(dev, form, sig, *best, best_t);
  }
  return rc;
}

}  // extern "C"
