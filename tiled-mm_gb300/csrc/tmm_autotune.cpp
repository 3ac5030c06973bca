// Autotuner: tile variants of the batched kernel (timed per size class on first
// use) and tile sizes / stream count of the out-of-core pipeline (timed per size
// class over the first calls, see autotune_pick).
//
// The reference's only tile policy is the divisor rule of
// src/Tiled-MM/mm_handle.cpp:89-133 applied to user-given maxima; it stays the
// default.  TMM_TILE_POLICY_AUTOTUNE selects this tuner instead.  Batched size
// classes are log2 buckets of max(m, n) and of k.  Choices are kept in memory
// and, when TMM_AUTOTUNE_CACHE names a file, read from and appended to it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "tmm_batched.h"

namespace tmm {
namespace {

std::mutex g_mu;
std::map<std::tuple<int, int, int>, int> g_variant;  // (dtype, m-bucket, k-bucket) -> variant
bool g_loaded = false;

int bucket(int64_t v) {
  int b = 0;
  while (v > 64 && b < 12) {
    v >>= 1;
    ++b;
  }
  return b;  // 0: <= 64, 1: <= 128, ... 6: <= 4096, ...
}

int64_t bucket_rep(int b) { return (int64_t)48 << b; }  // inside the bucket (64 * 2^b * 3/4)

void load_cache() {
  if (g_loaded) return;
  g_loaded = true;
  const char* path = getenv("TMM_AUTOTUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  int dt, mb, kb, v;
  while (fscanf(f, "batch %d %d %d %d\n", &dt, &mb, &kb, &v) == 4) g_variant[{dt, mb, kb}] = v;
  fclose(f);
}

void store_cache(int dt, int mb, int kb, int v) {
  const char* path = getenv("TMM_AUTOTUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "batch %d %d %d %d\n", dt, mb, kb, v);
  fclose(f);
}

// time one variant on a synthetic batch of 8 problems of the class's representative shape
double time_variant(int dtype, int variant, int64_t m, int64_t n, int64_t k) {
  const int count = 8;
  const size_t es = dtype == TMM_DOUBLE ? 8 : 4;
  const size_t per = (size_t)(m * k + k * n + m * n) * es;
  void* buf = nullptr;
  if (cudaMalloc(&buf, per * count) != cudaSuccess) {
    cudaGetLastError();
    return 1e30;
  }
  cudaMemset(buf, 0, per * count);
  std::vector<BatchProblem> probs(count);
  for (int i = 0; i < count; ++i) {
    char* base = (char*)buf + per * i;
    probs[i] = BatchProblem{dtype, OP_N, OP_N, m, n, k, m, k, m, 1.0, 0.0, base, base + m * k * es,
                            base + (m * k + k * n) * es, variant};
  }
  std::vector<unsigned char> pb, wb;
  int n_work = 0, n_f64 = 0;
  batch_plan(probs, pb, wb, &n_work, &n_f64);
  void *dp = nullptr, *dw = nullptr;
  double best = 1e30;
  cudaStream_t s = nullptr;
  if (cudaMalloc(&dp, pb.size()) == cudaSuccess && cudaMalloc(&dw, wb.size() ? wb.size() : 16) == cudaSuccess &&
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess) {
    cudaMemcpy(dp, pb.data(), pb.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dw, wb.data(), wb.size(), cudaMemcpyHostToDevice);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, s);
      batch_launch(dp, count, dw, n_f64, n_work - n_f64, 0, s, nullptr, nullptr, nullptr);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) == cudaSuccess) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) best = std::min(best, (double)ms);
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  cudaGetLastError();
  if (s) cudaStreamDestroy(s);
  if (dp) cudaFree(dp);
  if (dw) cudaFree(dw);
  cudaFree(buf);
  return best;
}

}  // namespace

int autotune_batch_variant(int dtype, int64_t m, int64_t n, int64_t k) {
  if (dtype == TMM_DOUBLE) return BATCH_F64_64;
  if (const char* force = getenv("TMM_BATCH_F32_TILE")) return atoi(force) == 128 ? BATCH_F32_128 : BATCH_F32_64;
  const int mb = bucket(std::max(m, n)), kb = bucket(k);
  std::lock_guard<std::mutex> lock(g_mu);
  load_cache();
  auto it = g_variant.find({dtype, mb, kb});
  if (it != g_variant.end()) return it->second;
  const int64_t rm = bucket_rep(mb), rk = bucket_rep(kb);
  const double t64 = time_variant(dtype, BATCH_F32_64, rm, rm, rk);
  const double t128 = time_variant(dtype, BATCH_F32_128, rm, rm, rk);
  const int v = t128 < t64 ? BATCH_F32_128 : BATCH_F32_64;
  g_variant[{dtype, mb, kb}] = v;
  store_cache(dtype, mb, kb, v);
  return v;
}

namespace {

// Candidate tiles of a host-pointer call: the largest tiles whose working set fits 80 % of
// the memory budget (m, n tiles up to 16384, k tiles up to the context's maximum), then the
// same with the k tile halved and quartered (shorter k tiles pay more FP64 drains and
// splits per product but keep the operand planes that a wave of the engine streams closer to
// L2's size) and with the m and n tiles halved (more C tiles: more copy-compute overlap, more
// operand re-sends when the operands do not stay resident).
std::vector<TileChoice> tile_candidates(const TuneProblem& p) {
  const int dtype = p.dtype;
  const bool ozaki = p.path == TMM_PATH_OZAKI;
  const int slices = p.slices;
  const int64_t m = p.m, n = p.n, k = std::max<int64_t>(p.k, 1);
  const size_t es = dtype == TMM_FLOAT ? 4 : (dtype == TMM_COMPLEX_DOUBLE ? 16 : 8);
  // float and complex contexts on the Ozaki path cache raw tiles and give each of the two
  // streams the tile's FP64 embedding (twice as tall and deep for complex), its product
  // and its slices
  const bool embed = ozaki && dtype != TMM_DOUBLE;
  const double cf = dtype == TMM_COMPLEX_FLOAT || dtype == TMM_COMPLEX_DOUBLE ? 2.0 : 1.0;
  auto working_set = [&](int64_t a, int64_t b, int64_t c) -> double {
    if (embed) {
      const double raw = 2.0 * es * a * c + 2.0 * es * b * c + 4.0 * es * a * b;
      const double per_stream = 8.0 * cf * cf * a * c + 8.0 * cf * c * b + 8.0 * cf * a * b +
                                (double)slices * (cf * a + b) * cf * c;
      return raw + 2.0 * per_stream;
    }
    // two A tiles, two B tiles (cached form), four C tiles (2 streams x 2 slots), staging
    const double tile_a = ozaki ? (double)slices * a * c : (double)es * a * c;
    const double tile_b = ozaki ? (double)slices * b * c : (double)es * b * c;
    // float and complex float tiles on the FP32 tensor-core engine: per stream the bf16 parts
    // (6 bytes per element of the embedded operands) and, for complex, the embedding and product
    double f32 = 0.0;
    if (!ozaki && dtype == TMM_FLOAT) f32 = 2.0 * 6.0 * (double)(a + b) * c;
    if (!ozaki && dtype == TMM_COMPLEX_FLOAT)
      f32 = 2.0 * (6.0 * (2.0 * a + b) * 2.0 * c + 4.0 * (4.0 * a * c + 2.0 * c * b + 2.0 * a * b));
    return 2 * tile_a + 2 * tile_b + 4.0 * es * a * b + (ozaki ? 3.0 * 8 * std::max(a, b) * c : 0.0) + f32;
  };
  auto fit = [&](int64_t tm, int64_t tn, int64_t tk) {
    tm = std::max<int64_t>(1, std::min(tm, m));
    tn = std::max<int64_t>(1, std::min(tn, n));
    tk = std::max<int64_t>(1, std::min(tk, k));
    while (working_set(tm, tn, tk) > 0.8 * (double)p.budget && (tm > 256 || tn > 256 || tk > 256)) {
      if (tk >= tm && tk >= tn && tk > 256) tk = (tk + 1) / 2;
      else if (tm >= tn && tm > 256) tm = (tm + 1) / 2;
      else tn = (tn + 1) / 2;
    }
    const int64_t tiles = ((m + tm - 1) / tm) * ((n + tn - 1) / tn);
    return TileChoice{(int)tm, (int)tn, (int)tk, tiles > 1 ? 2 : 1};
  };
  const int64_t tm0 = std::min<int64_t>({m, (int64_t)p.max_tm, 16384});
  const int64_t tn0 = std::min<int64_t>({n, (int64_t)p.max_tn, 16384});
  const int64_t tk0 = std::min<int64_t>({k, (int64_t)p.max_tk, ozaki ? (int64_t)65536 : (int64_t)8192});
  std::vector<TileChoice> out;
  auto add = [&](TileChoice c) {
    for (const auto& o : out)
      if (o.tm == c.tm && o.tn == c.tn && o.tk == c.tk && o.streams == c.streams) return;
    out.push_back(c);
  };
  add(fit(tm0, tn0, tk0));
  const TileChoice base = out[0];
  if (base.tk / 2 >= 1024) add(fit(base.tm, base.tn, base.tk / 2));
  if (ozaki && base.tk / 4 >= 1024) add(fit(base.tm, base.tn, base.tk / 4));
  if (base.tm / 2 >= 1024 && base.tn / 2 >= 1024) add(fit(base.tm / 2, base.tn / 2, base.tk));
  return out;
}

int log2_bucket(int64_t v) {
  int b = 0;
  while (v > 1 && b < 62) {
    v = (v + 1) >> 1;
    ++b;
  }
  return b;
}

std::string class_key(const TuneProblem& p) {
  char buf[160];
  snprintf(buf, sizeof buf, "%d.%d.%d.%d.%d.%d.%d.%c%c.%d.%d.%d", p.dtype, p.path, p.engine, p.slices,
           log2_bucket(p.m), log2_bucket(p.n), log2_bucket(p.k), p.ta, p.tb, p.pinned, p.copy_back,
           log2_bucket((int64_t)(p.budget >> 30)));
  return buf;
}

struct TuneClass {
  std::vector<TileChoice> cands;
  std::vector<double> sec_per_flop;  // < 0: not timed yet
  int best = -1;
  bool from_cache = false;
  TileChoice cached{};
};
std::map<std::string, TuneClass> g_classes;
bool g_tiles_loaded = false;

void load_tile_cache() {
  if (g_tiles_loaded) return;
  g_tiles_loaded = true;
  const char* path = getenv("TMM_AUTOTUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof line, f)) {
    char key[200];
    TileChoice c{};
    if (sscanf(line, "tiles %199s %d %d %d %d", key, &c.tm, &c.tn, &c.tk, &c.streams) == 5) {
      TuneClass& tc = g_classes[key];
      tc.from_cache = true;
      tc.cached = c;
    }
  }
  fclose(f);
}

}  // namespace

TileChoice autotune_pick(const TuneProblem& p, int* index, int* state) {
  std::lock_guard<std::mutex> lock(g_mu);
  load_tile_cache();
  TuneClass& tc = g_classes[class_key(p)];
  if (tc.from_cache && tc.best < 0) {
    *index = -1;
    *state = 3;
    const TileChoice c = tc.cached;
    // a cached choice larger than this problem is clipped to it
    return TileChoice{(int)std::min<int64_t>(c.tm, p.m), (int)std::min<int64_t>(c.tn, p.n),
                      (int)std::min<int64_t>(c.tk, std::max<int64_t>(p.k, 1)), c.streams};
  }
  if (tc.cands.empty()) {
    tc.cands = tile_candidates(p);
    tc.sec_per_flop.assign(tc.cands.size(), -1.0);
  }
  if (tc.best >= 0) {
    *index = tc.best;
    *state = 2;
    return tc.cands[(size_t)tc.best];
  }
  for (size_t i = 0; i < tc.cands.size(); ++i)
    if (tc.sec_per_flop[i] < 0) {
      *index = (int)i;
      *state = 1;
      return tc.cands[i];
    }
  *index = 0;
  *state = 1;
  return tc.cands[0];
}

void autotune_report(const TuneProblem& p, int index, double seconds) {
  if (index < 0) return;
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_classes.find(class_key(p));
  if (it == g_classes.end()) return;
  TuneClass& tc = it->second;
  if (tc.best >= 0 || (size_t)index >= tc.cands.size()) return;
  const double flops = 2.0 * (double)p.m * (double)p.n * (double)std::max<int64_t>(p.k, 1);
  tc.sec_per_flop[(size_t)index] = seconds / flops;
  int best = -1;
  for (size_t i = 0; i < tc.cands.size(); ++i) {
    if (tc.sec_per_flop[i] < 0) return;  // still exploring
    if (best < 0 || tc.sec_per_flop[i] < tc.sec_per_flop[(size_t)best]) best = (int)i;
  }
  tc.best = best;
  if (const char* path = getenv("TMM_AUTOTUNE_CACHE")) {
    if (FILE* f = fopen(path, "a")) {
      const TileChoice& c = tc.cands[(size_t)best];
      fprintf(f, "tiles %s %d %d %d %d\n", class_key(p).c_str(), c.tm, c.tn, c.tk, c.streams);
      fclose(f);
    }
  }
}

std::string autotune_explain(const TuneProblem& p) {
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_classes.find(class_key(p));
  if (it == g_classes.end()) return "size class " + class_key(p) + ": no calls yet";
  const TuneClass& tc = it->second;
  std::string out = "size class " + class_key(p) + ":";
  if (tc.from_cache && tc.cands.empty()) {
    char buf[128];
    snprintf(buf, sizeof buf, " from the cache file: %dx%dx%d, %d streams", tc.cached.tm, tc.cached.tn, tc.cached.tk,
             tc.cached.streams);
    return out + buf;
  }
  for (size_t i = 0; i < tc.cands.size(); ++i) {
    char buf[160];
    const TileChoice& c = tc.cands[i];
    if (tc.sec_per_flop[i] < 0)
      snprintf(buf, sizeof buf, " [%zu] %dx%dx%d/%d untimed;", i, c.tm, c.tn, c.tk, c.streams);
    else
      snprintf(buf, sizeof buf, " [%zu] %dx%dx%d/%d %.2f TFLOP/s%s;", i, c.tm, c.tn, c.tk, c.streams,
               1e-12 / tc.sec_per_flop[i], (int)i == tc.best ? " (chosen)" : "");
    out += buf;
  }
  return out;
}

}  // namespace tmm
