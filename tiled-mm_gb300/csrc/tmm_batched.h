// Internal interface of the batched persistent path and the autotuner (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <stdint.h>

#include <vector>

#include "../../include/tmm_c_api.h"
#include "tmm_kernels.h"

namespace tmm {

enum BatchVariant : int { BATCH_F64_64 = 0, BATCH_F32_64 = 1, BATCH_F32_128 = 2 };

struct BatchProblem {
  int dtype;  // TMM_FLOAT or TMM_DOUBLE
  Op opa, opb;
  int64_t m, n, k, lda, ldb, ldc;
  double alpha, beta;
  const void* a;
  const void* b;
  void* c;
  int variant;
};

// device records of the problems and the work list (items sorted by decreasing cost)
// (FP64 items first: n_f64 of the n_work)
int batch_plan(const std::vector<BatchProblem>& probs, std::vector<unsigned char>& dev_probs_bytes,
               std::vector<unsigned char>& work_bytes, int* n_work, int* n_f64);
size_t batch_problem_record_bytes();
size_t batch_work_record_bytes();
int64_t batch_item_cost(int dtype, int variant, int64_t k);
// FP64 items on s; FP32 items on s2 (forked and joined with the two events) when both kinds are present
cudaError_t batch_launch(const void* dev_probs, int count, const void* dev_work, int n_f64, int n_f32, int any_k0,
                         cudaStream_t s, cudaStream_t s2, cudaEvent_t fork, cudaEvent_t join);

// ---------------------------------------------------------------- autotuner (tmm_autotune.cpp)
// Tile variant of the batched kernel for a problem of this dtype and shape: the
// fastest of the candidates for its size class, timed on first use.
int autotune_batch_variant(int dtype, int64_t m, int64_t n, int64_t k);

struct TileChoice {
  int tm, tn, tk, streams;
};
// What the tuner needs to know about a host-pointer call (TMM_TILE_POLICY_AUTOTUNE).
struct TuneProblem {
  int dtype, path, engine, slices;
  int64_t m, n, k;
  char ta, tb;
  int pinned, copy_back;
  size_t budget;  // device bytes the context may hold
  int max_tm, max_tn, max_tk;
};
// The tile sizes and stream count for this call.  Measured tuning: each size class (dtype,
// path, engine, slices, log2 buckets of m, n, k, trans, pinning, copy-back) has a few
// candidates that fit the memory budget; the first calls of a class each run one untried
// candidate (every call computes the full, correct product) and report their time through
// autotune_report; once all are timed the fastest per flop is used, and it is appended to
// the TMM_AUTOTUNE_CACHE file when one is named.  *index identifies the candidate for the
// report (-1: the choice was read from the cache, nothing to report).
TileChoice autotune_pick(const TuneProblem& p, int* index, int* state);
void autotune_report(const TuneProblem& p, int index, double seconds);
// Text of the measurements behind the tuner's choice for this problem's size class.
std::string autotune_explain(const TuneProblem& p);

}  // namespace tmm
