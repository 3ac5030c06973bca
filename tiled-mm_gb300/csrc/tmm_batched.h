// Internal interface of the batched persistent path and the autotuner (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
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
// Tile sizes and stream count of the out-of-core pipeline for this problem and
// device memory budget (TMM_TILE_POLICY_AUTOTUNE).
TileChoice autotune_tiles(int dtype, bool ozaki, int slices, int64_t m, int64_t n, int64_t k, size_t budget_bytes,
                          int max_tm, int max_tn, int max_tk);

}  // namespace tmm
