// Internal interface of the FP32 tensor-core engine (tmm_f32tc.cu; not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

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

// Complex float through the real embedding on this engine (tmm_ozaki_embed.cu): Ahat
// (2m x 2k, ld 2m) and Bhat (2k x n, ld 2k) in float, conjugating for op 'C'; after the engine
// has written T = Ahat Bhat (2m x n, ld 2m), C = alpha (T_top + i T_bottom) + beta C.
cudaError_t cplx_f32_embed(const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m,
                           int64_t n, int64_t k, float* Ahat, float* Bhat, cudaStream_t s);
cudaError_t cplx_f32_combine(int64_t m, int64_t n, const void* alpha, const void* beta, const float* Tm, void* C,
                             int64_t ldc, cudaStream_t s);

}  // namespace tmm
