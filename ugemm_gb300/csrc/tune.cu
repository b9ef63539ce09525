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
#include <algorithm>
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

// One cache line: the chosen configuration and its time, then every
// candidate timed as [block_n, chunk_k, max_ctas, split_k, deal, transpose,
// fused, ms].
bool lookup(const std::string& dev, int form, uint64_t sig, ugemm_tile_config* cfg, double* ms) {
  FILE* f = std::fopen(cache_path().c_str(), "r");
  if (!f) return false;
  std::vector<char> line(1 << 16);
  bool found = false;
  while (std::fgets(line.data(), static_cast<int>(line.size()), f)) {
    char d[128];
    int fm = 0;
    ugemm_tile_config c{};
    uint64_t s = 0;
    double t = 0;
    if (std::sscanf(line.data(),
                    "{\"device\": \"%127[^\"]\", \"form\": %d, \"sig\": \"%" SCNx64
                    "\", \"block_n\": %d, \"chunk_k\": %d, \"max_ctas\": %d, \"split_k\": %d, "
                    "\"deal\": %d, \"transpose\": %d, \"fused\": %d, \"ms\": %lf",
                    d, &fm, &s, &c.block_n, &c.chunk_k, &c.max_ctas, &c.split_k, &c.deal,
                    &c.transpose, &c.fused, &t) == 11 &&
        dev == d && fm == form && s == sig) {
      *cfg = c;
      if (ms) *ms = t;
      found = true;  // the last matching line wins
    }
  }
  std::fclose(f);
  return found;
}

struct Timed {
  ugemm_tile_config c;
  double ms;
};

void store(const std::string& dev, int form, uint64_t sig, const ugemm_tile_config& c, double ms,
           const std::vector<Timed>& all) {
  FILE* f = std::fopen(cache_path().c_str(), "a");
  if (!f) return;
  std::fprintf(f,
               "{\"device\": \"%s\", \"form\": %d, \"sig\": \"%016" PRIx64
               "\", \"block_n\": %d, \"chunk_k\": %d, \"max_ctas\": %d, \"split_k\": %d, "
               "\"deal\": %d, \"transpose\": %d, \"fused\": %d, \"ms\": %.9g, "
               "\"candidates\": [",
               dev.c_str(), form, sig, c.block_n, c.chunk_k, c.max_ctas, c.split_k, c.deal,
               c.transpose, c.fused, ms);
  for (size_t i = 0; i < all.size(); ++i) {
    const ugemm_tile_config& x = all[i].c;
    std::fprintf(f, "%s[%d, %d, %d, %d, %d, %d, %d, %.9g]", i ? ", " : "", x.block_n,
                 x.chunk_k, x.max_ctas, x.split_k, x.deal, x.transpose, x.fused, all[i].ms);
  }
  std::fprintf(f, "]}\n");
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
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return UGEMM_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int sms = 148, dev_id = 0;
  cudaGetDevice(&dev_id);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id);
  std::vector<Timed> all;
  // time one candidate (the best of three batches of five runs); < 0: failed
  auto time_cfg = [&](const ugemm_tile_config& c) -> double {
    for (const Timed& t : all)
      if (std::memcmp(&t.c, &c, sizeof c) == 0) return t.ms;
    ugemm_grouped_plan* p = nullptr;
    if (ugemm_grouped_plan_create(count, problems, form, &c, 0, &p) != UGEMM_OK) return -1.0;
    bool ok = true;
    for (int w = 0; w < 2 && ok; ++w) ok = ugemm_grouped_run(p, st) == UGEMM_OK;
    double best = 1e30;
    for (int batch = 0; batch < 3 && ok; ++batch) {
      const int reps = 5;
      cudaEventRecord(e0, st);
      for (int r = 0; r < reps && ok; ++r) ok = ugemm_grouped_run(p, st) == UGEMM_OK;
      cudaEventRecord(e1, st);
      ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, double(ms) / reps);
    }
    ok = ok && ugemm_grouped_check(p, st) == UGEMM_OK;
    ugemm_grouped_plan_destroy(p);
    if (!ok) return -1.0;
    all.push_back(Timed{c, best});
    return best;
  };
  ugemm_tile_config cur{};
  double cur_t = 1e30;
  auto consider = [&](const ugemm_tile_config& c) {
    const double t = time_cfg(c);
    if (t >= 0 && t < cur_t) {
      cur_t = t;
      cur = c;
    }
  };
  // 1. tile shape
  if (form == UGEMM_PREC_SIMT) {
    for (int bn : {64, 128}) consider(ugemm_tile_config{bn, 0, 0, 0, 0, 0, 0});
  } else {
    // chunk_k <= 256 keeps the split form at least as accurate as FP32 SIMT
    for (int bn : {128, 256})
      for (int ck : {128, 256}) consider(ugemm_tile_config{bn, ck, 0, 0, 0, 0, 0});
    // three bf16 pieces: the operands split inside the GEMM kernel
    if (form == UGEMM_PREC_BF16X6 || form == UGEMM_PREC_BF16X9)
      for (int bn : {128, 256})
        for (int ck : {128, 256}) consider(ugemm_tile_config{bn, ck, 0, 0, 0, 0, 1});
  }
  // 2. schedule, one knob at a time from the best so far
  if (cur_t < 1e30) {
    const ugemm_tile_config base = cur;
    for (int sk : {1, 4, -1}) {
      ugemm_tile_config c = base;
      c.split_k = sk;
      consider(c);
    }
    if (form != UGEMM_PREC_SIMT) {
      ugemm_tile_config c = cur;
      c.deal = 1;
      consider(c);
      c = cur;
      c.transpose = 1;
      consider(c);
    }
    for (int mc : {sms - sms / 8, sms / 2}) {
      ugemm_tile_config c = cur;
      c.max_ctas = mc;
      consider(c);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  int rc = UGEMM_ERR_UNSUPPORTED;
  double best_t = 1e30;
  for (const Timed& t : all)  // the fastest of everything timed
    if (t.ms < best_t) {
      best_t = t.ms;
      *best = t.c;
      rc = UGEMM_OK;
    }
  if (rc == UGEMM_OK) {
    if (best_ms) *best_ms = best_t;
    std::lock_guard<std::mutex> l(g_tmu);
    store(dev, form, sig, *best, best_t, all);
  }
  return rc;
}

}  // extern "C"
