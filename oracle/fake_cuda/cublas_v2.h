/*
 * ORACLE test infrastructure: host-only stand-in for the cuBLAS names used by
 * the reference's src/Tiled-MM/gpu_blas_api.hpp.  The ?gemm entry points are
 * a plain column-major GEMM with the published BLAS semantics
 * (C = alpha*op(A)*op(B) + beta*C, C not read when beta == 0), defined in
 * fake_cuda.cpp.  Never linked into the product.
 */
#pragma once
#include "cuda_runtime_api.h"

typedef struct fake_blas* cublasHandle_t;

typedef enum {
  CUBLAS_STATUS_SUCCESS = 0,
  CUBLAS_STATUS_NOT_INITIALIZED = 1,
  CUBLAS_STATUS_ALLOC_FAILED = 3,
  CUBLAS_STATUS_INVALID_VALUE = 7,
  CUBLAS_STATUS_ARCH_MISMATCH = 8,
  CUBLAS_STATUS_MAPPING_ERROR = 11,
  CUBLAS_STATUS_EXECUTION_FAILED = 13,
  CUBLAS_STATUS_INTERNAL_ERROR = 14,
  CUBLAS_STATUS_NOT_SUPPORTED = 15,
  CUBLAS_STATUS_LICENSE_ERROR = 16
} cublasStatus_t;

typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1, CUBLAS_OP_C = 2 } cublasOperation_t;

typedef struct { float x, y; } cuComplex;
typedef struct { double x, y; } cuDoubleComplex;

cublasStatus_t cublasCreate(cublasHandle_t* h);
cublasStatus_t cublasDestroy(cublasHandle_t h);
cublasStatus_t cublasSetStream(cublasHandle_t h, cudaStream_t s);
cublasStatus_t cublasSgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n,
                           int k, const float* alpha, const float* a, int lda, const float* b, int ldb,
                           const float* beta, float* c, int ldc);
cublasStatus_t cublasDgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n,
                           int k, const double* alpha, const double* a, int lda, const double* b,
                           int ldb, const double* beta, double* c, int ldc);
cublasStatus_t cublasCgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n,
                           int k, const cuComplex* alpha, const cuComplex* a, int lda,
                           const cuComplex* b, int ldb, const cuComplex* beta, cuComplex* c, int ldc);
cublasStatus_t cublasZgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n,
                           int k, const cuDoubleComplex* alpha, const cuDoubleComplex* a, int lda,
                           const cuDoubleComplex* b, int ldb, const cuDoubleComplex* beta,
                           cuDoubleComplex* c, int ldc);
