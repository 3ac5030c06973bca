// Internal interface of the FP32 tensor-core engine (tmm_f32tc.cu; not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "tmm_kernels.h"

namespace tmm {

// Scratch of one f32tc_gemm call: a 256-byte header (the error word of the bounded waits,
// which the caller zeroes once and reads after synchronising) and the bf16 planes of op(A)
// and op(B).
size_t f32tc_scratch_bytes(int64_t m, int64_t n, int64_t k);
// One-time per-device set-up (function attributes, tensor-map encoder); call outside capture.
cudaError_t f32tc_prepare();
// C = alpha * op(A) * op(B) + beta * C in FP32 on the tcgen05 tensor cores (C not read when
// beta == 0); op in {N, T}; enqueued on s.
cudaError_t f32tc_gemm(Op opa, Op opb, int64_t m, int64_t n, int64_t k, float alpha, const float* A, int64_t lda,
                       const float* B, int64_t ldb, float beta, float* C, int64_t ldc, void* scratch,
                       size_t scratch_bytes, cudaStream_t s);

// Grouped form (a batch's FP32 problems): every product's bf16 planes live in one arena
// (f32tc_plane_bytes per operand; offsets multiples of 256 bytes), written by
// f32tc_split_lines (lines of op(A) are its rows, lines of op(B) its columns;
// lines_contiguous: consecutive lines are adjacent in memory, i.e. element (line, l) at
// X[line + l ld], else at X[l + line ld]); f32tc_grouped_image writes the launch's device
// records (at most f32tc_grouped_image_bound bytes), to be copied to dev_image, and
// f32tc_gemm_grouped multiplies all products in one persistent launch.
struct F32GroupedProduct {
  const void* a_planes;
  const void* b_planes;
  int64_t m, n, k;
  float alpha, beta;
  float* C;
  int64_t ldc;
};
size_t f32tc_plane_bytes(int64_t lines, int64_t k);
cudaError_t f32tc_split_lines(const float* X, int64_t ld, bool lines_contiguous, int64_t lines, int64_t k,
                              void* planes, cudaStream_t s);
cudaError_t f32tc_grouped_image(const std::vector<F32GroupedProduct>& prods, const void* arena, size_t arena_bytes,
                                std::vector<unsigned char>& out, int* n_items);
size_t f32tc_grouped_image_bound(const std::vector<F32GroupedProduct>& prods);
cudaError_t f32tc_gemm_grouped(const void* arena, size_t arena_bytes, const void* dev_image, int n_probs, int n_items,
                               int* err, cudaStream_t s);

// Complex float through the real embedding on this engine (tmm_ozaki_embed.cu): Ahat
// (2m x 2k, ld 2m) and Bhat (2k x n, ld 2k) in float, conjugating for op 'C'; after the engine
// has written T = Ahat Bhat (2m x n, ld 2m), C = alpha (T_top + i T_bottom) + beta C.
cudaError_t cplx_f32_embed(const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m,
                           int64_t n, int64_t k, float* Ahat, float* Bhat, cudaStream_t s);
cudaError_t cplx_f32_combine(int64_t m, int64_t n, const void* alpha, const void* beta, const float* Tm, void* C,
                             int64_t ldc, cudaStream_t s);

}  // namespace tmm
