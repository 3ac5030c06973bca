// cublasXt-style entry over the tiled path: a handle, one block dimension for all
// three tile sizes, and ?gemm calls on host (or device) pointers with the trans
// arguments given as cublasOperation_t values (0 = N, 1 = T, 2 = C).  This is the
// call shape of the reference's comparison program (examples/cublasXt-multiply.cpp:
// 153-167: cublasXtCreate, cublasXtDeviceSelect, cublasXtSetBlockDim, cublasXtDgemm),
// so a caller written against it moves over by renaming.  Each call is tmm_gemm on a
// per-dtype context with fixed tiles of the block dimension, page-locking the host
// buffers for the call and copying C back.
#include <cstdint>
#include <mutex>

#include "../../include/tmm_c_api.h"

struct tmm_xt {
  int block_dim = 4096;
  int path = TMM_PATH_NATIVE;
  int slices = 0;
  tmm_context* ctx[4] = {nullptr, nullptr, nullptr, nullptr};
  tmm_context* last = nullptr;  // context of the last call (its error message)
  std::mutex mu;
};

namespace {

char op_char(int op) {
  switch (op) {
    case 0: return 'N';
    case 1: return 'T';
    case 2: return 'C';
    default: return '?';  // rejected by tmm_gemm
  }
}

int xt_gemm(tmm_xt* h, int dtype, int transa, int transb, int64_t m, int64_t n, int64_t k, const void* alpha,
            const void* a, int64_t lda, const void* b, int64_t ldb, const void* beta, void* c, int64_t ldc) {
  if (!h) return TMM_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(h->mu);
  tmm_context*& ctx = h->ctx[dtype];
  if (!ctx) {
    const int st = tmm_create(dtype, 2, h->block_dim, h->block_dim, h->block_dim, &ctx);
    if (st) return st;
    tmm_set_tile_policy(ctx, TMM_TILE_POLICY_FIXED);  // cublasXt tiles by the block dimension
  }
  h->last = ctx;
  const int st = tmm_set_path(ctx, h->path, h->slices);
  if (st) return st;
  return tmm_gemm(ctx, op_char(transa), op_char(transb), m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1);
}

}  // namespace

extern "C" int tmm_xt_create(tmm_xt** handle) {
  if (!handle) return TMM_ERROR_INVALID_ARGUMENT;
  *handle = new tmm_xt();
  return TMM_SUCCESS;
}

extern "C" int tmm_xt_destroy(tmm_xt* handle) {
  if (!handle) return TMM_SUCCESS;
  int st = TMM_SUCCESS;
  for (auto*& c : handle->ctx) {
    if (c) {
      const int s = tmm_destroy(c);
      if (!st) st = s;
      c = nullptr;
    }
  }
  delete handle;
  return st;
}

extern "C" int tmm_xt_set_block_dim(tmm_xt* handle, int block_dim) {
  if (!handle || block_dim < 1) return TMM_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(handle->mu);
  // contexts were created with the old block as their maximum tile: start over
  for (auto*& c : handle->ctx) {
    if (c) tmm_destroy(c);
    c = nullptr;
  }
  handle->last = nullptr;
  handle->block_dim = block_dim;
  return TMM_SUCCESS;
}

extern "C" const char* tmm_xt_last_error(tmm_xt* handle) {
  return handle && handle->last ? tmm_last_error(handle->last) : tmm_last_error(nullptr);
}

extern "C" int tmm_xt_get_block_dim(tmm_xt* handle, int* block_dim) {
  if (!handle || !block_dim) return TMM_ERROR_INVALID_ARGUMENT;
  *block_dim = handle->block_dim;
  return TMM_SUCCESS;
}

extern "C" int tmm_xt_set_path(tmm_xt* handle, int path, int ozaki_slices) {
  if (!handle || (path != TMM_PATH_NATIVE && path != TMM_PATH_OZAKI)) return TMM_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(handle->mu);
  handle->path = path;
  handle->slices = ozaki_slices;
  return TMM_SUCCESS;
}

extern "C" int tmm_xt_sgemm(tmm_xt* h, int transa, int transb, int64_t m, int64_t n, int64_t k, const float* alpha,
                            const float* a, int64_t lda, const float* b, int64_t ldb, const float* beta, float* c,
                            int64_t ldc) {
  return xt_gemm(h, TMM_FLOAT, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

extern "C" int tmm_xt_dgemm(tmm_xt* h, int transa, int transb, int64_t m, int64_t n, int64_t k, const double* alpha,
                            const double* a, int64_t lda, const double* b, int64_t ldb, const double* beta, double* c,
                            int64_t ldc) {
  return xt_gemm(h, TMM_DOUBLE, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

extern "C" int tmm_xt_cgemm(tmm_xt* h, int transa, int transb, int64_t m, int64_t n, int64_t k, const void* alpha,
                            const void* a, int64_t lda, const void* b, int64_t ldb, const void* beta, void* c,
                            int64_t ldc) {
  return xt_gemm(h, TMM_COMPLEX_FLOAT, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

extern "C" int tmm_xt_zgemm(tmm_xt* h, int transa, int transb, int64_t m, int64_t n, int64_t k, const void* alpha,
                            const void* a, int64_t lda, const void* b, int64_t ldb, const void* beta, void* c,
                            int64_t ldc) {
  return xt_gemm(h, TMM_COMPLEX_DOUBLE, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
