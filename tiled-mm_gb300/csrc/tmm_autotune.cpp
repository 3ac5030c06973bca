// Autotuner: tile variants of the batched kernel (timed per size class on first
// use) and tile sizes / stream count of the out-of-core pipeline (model-based:
// the largest tiles whose working set fits the device memory budget).
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

TileChoice autotune_tiles(int dtype, bool ozaki, int slices, int64_t m, int64_t n, int64_t k, size_t budget,
                          int max_tm, int max_tn, int max_tk) {
  const size_t es = dtype == TMM_FLOAT ? 4 : (dtype == TMM_COMPLEX_DOUBLE ? 16 : 8);
  // The Ozaki path amortises its split and its FP64 drains over long k tiles, but past
  // 16384 the slice planes that one wave of CTAs streams outgrow L2: measured at
  // m = n = k = 32768, 11 slices: tk 8192 -> 46.1, 16384 -> 46.9, 32768 -> 43.2 TFLOP/s.
  // TMM_AUTOTUNE_OZAKI_TK overrides the cap.
  int64_t oz_cap = 16384;
  if (const char* env = getenv("TMM_AUTOTUNE_OZAKI_TK")) {
    const long long v = atoll(env);
    if (v >= 128) oz_cap = v;
  }
  int64_t tk = std::min<int64_t>({k > 0 ? k : 1, (int64_t)max_tk, ozaki ? oz_cap : 8192});
  int64_t tm = std::min<int64_t>({m, (int64_t)max_tm, 16384});
  int64_t tn = std::min<int64_t>({n, (int64_t)max_tn, 16384});
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
    return 2 * tile_a + 2 * tile_b + 4.0 * es * a * b + (ozaki ? 3.0 * 8 * std::max(a, b) * c : 0.0);
  };
  while (working_set(tm, tn, tk) > 0.8 * (double)budget && (tm > 256 || tn > 256 || tk > 256)) {
    if (tk >= tm && tk >= tn && tk > 256) tk = (tk + 1) / 2;
    else if (tm >= tn && tm > 256) tm = (tm + 1) / 2;
    else tn = (tn + 1) / 2;
  }
  const int64_t tiles = ((m + tm - 1) / tm) * ((n + tn - 1) / tn);
  return TileChoice{(int)tm, (int)tn, (int)tk, tiles > 1 ? 2 : 1};
}

}  // namespace tmm
