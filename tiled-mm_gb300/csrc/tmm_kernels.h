// Internal launch interface of the per-tile kernels (not part of the C ABI).
//
// Every kernel computes, on device operands,
//     C = alpha * op(A) * op(B) + beta * C      (C not read when beta == 0)
// with column-major A, B, C and arbitrary leading dimensions, the contract of
// the per-tile cuBLAS call it replaces (src/Tiled-MM/tiled_mm.cpp:181-268).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tmm {

enum Op : int { OP_N = 0, OP_T = 1, OP_C = 2 };

struct cplxf { float re, im; };
struct cplxd { double re, im; };

cudaError_t launch_gemm_f64(Op opa, Op opb, int64_t m, int64_t n, int64_t k, double alpha,
                            const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                            double* C, int64_t ldc, cudaStream_t s);
cudaError_t launch_gemm_f32(Op opa, Op opb, int64_t m, int64_t n, int64_t k, float alpha,
                            const float* A, int64_t lda, const float* B, int64_t ldb, float beta,
                            float* C, int64_t ldc, cudaStream_t s);
cudaError_t launch_gemm_c32(Op opa, Op opb, int64_t m, int64_t n, int64_t k, cplxf alpha,
                            const cplxf* A, int64_t lda, const cplxf* B, int64_t ldb, cplxf beta,
                            cplxf* C, int64_t ldc, cudaStream_t s);
cudaError_t launch_gemm_c64(Op opa, Op opb, int64_t m, int64_t n, int64_t k, cplxd alpha,
                            const cplxd* A, int64_t lda, const cplxd* B, int64_t ldb, cplxd beta,
                            cplxd* C, int64_t ldc, cudaStream_t s);

// C = beta * C over an m x n block (k == 0 quick return), C not read when beta == 0.
cudaError_t launch_scale_f64(int64_t m, int64_t n, double beta, double* C, int64_t ldc, cudaStream_t s);
cudaError_t launch_scale_f32(int64_t m, int64_t n, float beta, float* C, int64_t ldc, cudaStream_t s);
cudaError_t launch_scale_c32(int64_t m, int64_t n, cplxf beta, cplxf* C, int64_t ldc, cudaStream_t s);
cudaError_t launch_scale_c64(int64_t m, int64_t n, cplxd beta, cplxd* C, int64_t ldc, cudaStream_t s);

// Seeded synthetic fill of a rows x cols column-major device block (see tmm_datagen.h).
cudaError_t launch_fill_f64(double* X, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                            uint64_t seed, uint64_t id, cudaStream_t s);

// 2D copy by kernel (height rows of width bytes, pitches in bytes) for host memory that the
// GPU accesses through the host page tables (tmm_native.cu)
cudaError_t copy2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t height,
                         cudaStream_t s);

}  // namespace tmm
