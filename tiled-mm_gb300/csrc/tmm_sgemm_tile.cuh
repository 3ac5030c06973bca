// FP32 tile engine shared by the plain path (per-tile cublasSgemm replacement,
// src/Tiled-MM/tiled_mm.cpp:181-198) and the batched path.
//
// 128 x 128 C tile per 256-thread CTA, 8 x 8 outputs per thread in the
// split-quad layout (rows 4tx..4tx+3 and 64+4tx.., columns 4ty.. and 64+4ty..)
// so every shared-memory fragment read is one 16-byte vector and conflict
// free; k steps of 8 double-buffered through shared memory with the next
// step's global loads held in registers.  Full FP32 FFMA accumulation (the
// semantics of cuBLAS's default, non-TF32 SGEMM), alpha/beta epilogue fused,
// beta == 0 never reads C.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tmm {
namespace sg {

constexpr int BM = 128, BN = 128, BK = 8, THREADS = 256;
constexpr int LDS = BM + 4;  // padded row: 16-byte aligned, conflict-free transposed stores
constexpr int SMEM_FLOATS = 2 * 2 * BK * LDS;  // [2 buffers][A, B][BK][LDS]

// op: 0 = N, 1 = T (conjugation is the identity on reals)
__device__ __forceinline__ void load_a(float (&r)[4], const float* __restrict__ A, int64_t lda, int op, int64_t m,
                                       int64_t k, int64_t i0, int64_t l0, int tid) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int idx = tid + q * THREADS;
    int ii, ll;
    if (op == 0) { ii = idx % BM; ll = idx / BM; } else { ll = idx % BK; ii = idx / BK; }
    const int64_t gi = i0 + ii, gl = l0 + ll;
    r[q] = (gi < m && gl < k) ? (op == 0 ? A[gi + gl * lda] : A[gl + gi * lda]) : 0.f;
  }
}
__device__ __forceinline__ void store_a(float* As, const float (&r)[4], int op, int tid) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int idx = tid + q * THREADS;
    int ii, ll;
    if (op == 0) { ii = idx % BM; ll = idx / BM; } else { ll = idx % BK; ii = idx / BK; }
    As[ll * LDS + ii] = r[q];
  }
}
__device__ __forceinline__ void load_b(float (&r)[4], const float* __restrict__ B, int64_t ldb, int op, int64_t k,
                                       int64_t n, int64_t l0, int64_t j0, int tid) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int idx = tid + q * THREADS;
    int jj, ll;
    if (op == 0) { ll = idx % BK; jj = idx / BK; } else { jj = idx % BN; ll = idx / BN; }
    const int64_t gj = j0 + jj, gl = l0 + ll;
    r[q] = (gj < n && gl < k) ? (op == 0 ? B[gl + gj * ldb] : B[gj + gl * ldb]) : 0.f;
  }
}
__device__ __forceinline__ void store_b(float* Bs, const float (&r)[4], int op, int tid) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int idx = tid + q * THREADS;
    int jj, ll;
    if (op == 0) { ll = idx % BK; jj = idx / BK; } else { jj = idx % BN; ll = idx / BN; }
    Bs[ll * LDS + jj] = r[q];
  }
}

// C[i0.., j0..] = alpha * op(A) op(B) + beta * C for one 128 x 128 tile
__device__ __forceinline__ void tile(int opa, int opb, int64_t m, int64_t n, int64_t k, float alpha,
                                     const float* __restrict__ A, int64_t lda, const float* __restrict__ B,
                                     int64_t ldb, float beta, float* __restrict__ C, int64_t ldc, int64_t i0,
                                     int64_t j0, float* smem) {
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
  float ra[4], rb[4];
  const int64_t nk = (k + BK - 1) / BK;
  if (nk > 0) {
    load_a(ra, A, lda, opa, m, k, i0, 0, tid);
    load_b(rb, B, ldb, opb, k, n, 0, j0, tid);
    store_a(smem, ra, opa, tid);
    store_b(smem + BK * LDS, rb, opb, tid);
  }
  __syncthreads();
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int buf = (int)(kt & 1);
    const float* As = smem + buf * 2 * BK * LDS;
    const float* Bs = As + BK * LDS;
    if (kt + 1 < nk) {
      load_a(ra, A, lda, opa, m, k, i0, (kt + 1) * BK, tid);
      load_b(rb, B, ldb, opb, k, n, (kt + 1) * BK, j0, tid);
    }
#pragma unroll
    for (int l = 0; l < BK; ++l) {
      const float4 a0 = *reinterpret_cast<const float4*>(As + l * LDS + 4 * tx);
      const float4 a1 = *reinterpret_cast<const float4*>(As + l * LDS + 64 + 4 * tx);
      const float4 b0 = *reinterpret_cast<const float4*>(Bs + l * LDS + 4 * ty);
      const float4 b1 = *reinterpret_cast<const float4*>(Bs + l * LDS + 64 + 4 * ty);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
    }
    if (kt + 1 < nk) {
      float* Ns = smem + (buf ^ 1) * 2 * BK * LDS;
      store_a(Ns, ra, opa, tid);
      store_b(Ns + BK * LDS, rb, opb, tid);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int64_t gi = i0 + (a < 4 ? 4 * tx + a : 64 + 4 * tx + (a - 4));
    if (gi >= m) continue;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int64_t gj = j0 + (b < 4 ? 4 * ty + b : 64 + 4 * ty + (b - 4));
      if (gj < n) {
        float* p = C + gi + gj * ldc;
        const float v = alpha * acc[a][b];
        *p = beta == 0.f ? v : v + beta * *p;
      }
    }
  }
}

}  // namespace sg
}  // namespace tmm
