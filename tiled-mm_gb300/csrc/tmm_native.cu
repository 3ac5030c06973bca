// Native per-tile kernels: the replacement of the reference's per-tile
// cublas{S,D,C,Z}gemm call (src/Tiled-MM/tiled_mm.cpp:181-268).
//
// FP64 runs on the FP64 tensor path (DMMA, mma.sync m16n8k4 f64) with the
// alpha/beta epilogue fused.  On GB300 FP64 issue is about 1.05 TFLOP/s
// whichever instruction is used (DMMA and DFMA measured alike), so a 64x64
// block tile with double-buffered shared-memory staging already keeps the
// FP64 pipe busy; operand traffic is ~8 flop/byte, far below HBM and L2 rates.
//
// FP32 and the two complex types use a register-blocked SIMT kernel (FFMA,
// full FP32/FP64 accuracy, matching cuBLAS's default non-TF32 semantics).
#include <algorithm>

#include "tmm_datagen.h"
#include "tmm_kernels.h"
#include "tmm_sgemm_tile.cuh"

namespace tmm {
namespace {

constexpr int DM_BM = 64, DM_BN = 64, DM_BK = 16, DM_THREADS = 128;
constexpr int DM_SA = DM_BM + 8;  // padded row stride (doubles): conflict-free fragment loads
constexpr int DM_SB = DM_BN + 8;

__device__ __forceinline__ void dmma_16x8x4(double (&d)[4], double a0, double a1, double b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
      : "+d"(d[0]), "+d"(d[1]), "+d"(d[2]), "+d"(d[3])
      : "d"(a0), "d"(a1), "d"(b0));
}

// Loads of one BM x BK tile of op(A) and one BK x BN tile of op(B) into
// registers, each thread 8 elements, coalesced along the stored leading
// dimension for either orientation.  Out-of-range elements read as 0.
template <int OPA>
__device__ __forceinline__ void load_a_f64(double (&r)[8], const double* __restrict__ A, int64_t lda,
                                           int64_t m, int64_t k, int64_t i0, int64_t l0, int tid) {
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int idx = tid + t * DM_THREADS;
    int ii, ll;
    if (OPA == OP_N) { ii = idx % DM_BM; ll = idx / DM_BM; }
    else             { ll = idx % DM_BK; ii = idx / DM_BK; }
    int64_t gi = i0 + ii, gl = l0 + ll;
    double v = 0.0;
    if (gi < m && gl < k) v = (OPA == OP_N) ? A[gi + gl * lda] : A[gl + gi * lda];
    r[t] = v;
  }
}
template <int OPA>
__device__ __forceinline__ void store_a_f64(double* As, const double (&r)[8], int tid) {
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int idx = tid + t * DM_THREADS;
    int ii, ll;
    if (OPA == OP_N) { ii = idx % DM_BM; ll = idx / DM_BM; }
    else             { ll = idx % DM_BK; ii = idx / DM_BK; }
    As[ll * DM_SA + ii] = r[t];
  }
}
template <int OPB>
__device__ __forceinline__ void load_b_f64(double (&r)[8], const double* __restrict__ B, int64_t ldb,
                                           int64_t k, int64_t n, int64_t l0, int64_t j0, int tid) {
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int idx = tid + t * DM_THREADS;
    int jj, ll;
    if (OPB == OP_N) { ll = idx % DM_BK; jj = idx / DM_BK; }
    else             { jj = idx % DM_BN; ll = idx / DM_BN; }
    int64_t gj = j0 + jj, gl = l0 + ll;
    double v = 0.0;
    if (gj < n && gl < k) v = (OPB == OP_N) ? B[gl + gj * ldb] : B[gj + gl * ldb];
    r[t] = v;
  }
}
template <int OPB>
__device__ __forceinline__ void store_b_f64(double* Bs, const double (&r)[8], int tid) {
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int idx = tid + t * DM_THREADS;
    int jj, ll;
    if (OPB == OP_N) { ll = idx % DM_BK; jj = idx / DM_BK; }
    else             { jj = idx % DM_BN; ll = idx / DM_BN; }
    Bs[ll * DM_SB + jj] = r[t];
  }
}

// 4 warps in a 2 x 2 grid, each warp a 32 x 32 sub-tile = 2 (m16) x 4 (n8)
// DMMA accumulators.  Fragment layout of m16n8k4.f64 (lane = 4 g + t):
//   a0 = A[g][t], a1 = A[g+8][t];  b0 = B[t][g];
//   c0,c1 = C[g][2t], C[g][2t+1];  c2,c3 = C[g+8][2t], C[g+8][2t+1].
template <int OPA, int OPB>
__global__ void __launch_bounds__(DM_THREADS)
gemm_f64_dmma(int64_t m, int64_t n, int64_t k, double alpha, const double* __restrict__ A, int64_t lda,
              const double* __restrict__ B, int64_t ldb, double beta, double* __restrict__ C, int64_t ldc) {
  __shared__ double As[2][DM_BK * DM_SA];
  __shared__ double Bs[2][DM_BK * DM_SB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  const int64_t i0 = (int64_t)blockIdx.x * DM_BM, j0 = (int64_t)blockIdx.y * DM_BN;

  double acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.0;

  double ra[8], rb[8];
  const int64_t nk = (k + DM_BK - 1) / DM_BK;
  if (nk > 0) {
    load_a_f64<OPA>(ra, A, lda, m, k, i0, 0, tid);
    load_b_f64<OPB>(rb, B, ldb, k, n, 0, j0, tid);
    store_a_f64<OPA>(As[0], ra, tid);
    store_b_f64<OPB>(Bs[0], rb, tid);
  }
  __syncthreads();
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int buf = (int)(kt & 1);
    if (kt + 1 < nk) {
      load_a_f64<OPA>(ra, A, lda, m, k, i0, (kt + 1) * DM_BK, tid);
      load_b_f64<OPB>(rb, B, ldb, k, n, (kt + 1) * DM_BK, j0, tid);
    }
    const double* as = As[buf];
    const double* bs = Bs[buf];
#pragma unroll
    for (int ks = 0; ks < DM_BK; ks += 4) {
      double af[2][2], bf[4];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        af[a][0] = as[(ks + t) * DM_SA + wm + a * 16 + g];
        af[a][1] = as[(ks + t) * DM_SA + wm + a * 16 + g + 8];
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) bf[b] = bs[(ks + t) * DM_SB + wn + b * 8 + g];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) dmma_16x8x4(acc[a][b], af[a][0], af[a][1], bf[b]);
    }
    if (kt + 1 < nk) {
      store_a_f64<OPA>(As[buf ^ 1], ra, tid);
      store_b_f64<OPB>(Bs[buf ^ 1], rb, tid);
    }
    __syncthreads();
  }
  // fused epilogue
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        int64_t gi = i0 + wm + a * 16 + g + ((c >> 1) << 3);
        int64_t gj = j0 + wn + b * 8 + 2 * t + (c & 1);
        if (gi < m && gj < n) {
          double* p = C + gi + gj * ldc;
          double v = alpha * acc[a][b][c];
          *p = (beta == 0.0) ? v : fma(beta, *p, v);
        }
      }
}

// ----------------------------------------------------------------- SIMT kernel
template <typename T> struct Num;
template <> struct Num<float> {
  __device__ static float zero() { return 0.f; }
  __device__ static float conj(float v) { return v; }
  __device__ static float mac(float acc, float a, float b) { return fmaf(a, b, acc); }
  __device__ static float mul(float a, float b) { return a * b; }
  __device__ static float add(float a, float b) { return a + b; }
  __device__ static bool is_zero(float v) { return v == 0.f; }
};
template <> struct Num<cplxf> {
  __device__ static cplxf zero() { return {0.f, 0.f}; }
  __device__ static cplxf conj(cplxf v) { return {v.re, -v.im}; }
  __device__ static cplxf mac(cplxf acc, cplxf a, cplxf b) {
    acc.re = fmaf(a.re, b.re, acc.re); acc.re = fmaf(-a.im, b.im, acc.re);
    acc.im = fmaf(a.re, b.im, acc.im); acc.im = fmaf(a.im, b.re, acc.im);
    return acc;
  }
  __device__ static cplxf mul(cplxf a, cplxf b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
  __device__ static cplxf add(cplxf a, cplxf b) { return {a.re + b.re, a.im + b.im}; }
  __device__ static bool is_zero(cplxf v) { return v.re == 0.f && v.im == 0.f; }
};
template <> struct Num<cplxd> {
  __device__ static cplxd zero() { return {0.0, 0.0}; }
  __device__ static cplxd conj(cplxd v) { return {v.re, -v.im}; }
  __device__ static cplxd mac(cplxd acc, cplxd a, cplxd b) {
    acc.re = fma(a.re, b.re, acc.re); acc.re = fma(-a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im); acc.im = fma(a.im, b.re, acc.im);
    return acc;
  }
  __device__ static cplxd mul(cplxd a, cplxd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
  __device__ static cplxd add(cplxd a, cplxd b) { return {a.re + b.re, a.im + b.im}; }
  __device__ static bool is_zero(cplxd v) { return v.re == 0.0 && v.im == 0.0; }
};
template <> struct Num<double> {
  __device__ static double zero() { return 0.0; }
  __device__ static double conj(double v) { return v; }
  __device__ static double mac(double acc, double a, double b) { return fma(a, b, acc); }
  __device__ static double mul(double a, double b) { return a * b; }
  __device__ static double add(double a, double b) { return a + b; }
  __device__ static bool is_zero(double v) { return v == 0.0; }
};

// BM x BN block tile, TM x TN outputs per thread, 256 threads.
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__(256)
gemm_simt(int opa, int opb, int64_t m, int64_t n, int64_t k, T alpha, const T* __restrict__ A, int64_t lda,
          const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc) {
  static_assert((BM / TM) * (BN / TN) == 256, "thread layout");
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % (BM / TM), ty = tid / (BM / TM);
  const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
  T acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = Num<T>::zero();
  for (int64_t l0 = 0; l0 < k; l0 += BK) {
    for (int idx = tid; idx < BM * BK; idx += 256) {
      int ii, ll;
      if (opa == OP_N) { ii = idx % BM; ll = idx / BM; } else { ll = idx % BK; ii = idx / BK; }
      int64_t gi = i0 + ii, gl = l0 + ll;
      T v = Num<T>::zero();
      if (gi < m && gl < k) {
        v = (opa == OP_N) ? A[gi + gl * lda] : A[gl + gi * lda];
        if (opa == OP_C) v = Num<T>::conj(v);
      }
      As[ll][ii] = v;
    }
    for (int idx = tid; idx < BN * BK; idx += 256) {
      int jj, ll;
      if (opb == OP_N) { ll = idx % BK; jj = idx / BK; } else { jj = idx % BN; ll = idx / BN; }
      int64_t gj = j0 + jj, gl = l0 + ll;
      T v = Num<T>::zero();
      if (gj < n && gl < k) {
        v = (opb == OP_N) ? B[gl + gj * ldb] : B[gj + gl * ldb];
        if (opb == OP_C) v = Num<T>::conj(v);
      }
      Bs[ll][jj] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int ll = 0; ll < BK; ++ll) {
      T ar[TM], br[TN];
#pragma unroll
      for (int a = 0; a < TM; ++a) ar[a] = As[ll][tx + a * (BM / TM)];
#pragma unroll
      for (int b = 0; b < TN; ++b) br[b] = Bs[ll][ty + b * (BN / TN)];
#pragma unroll
      for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = Num<T>::mac(acc[a][b], ar[a], br[b]);
    }
    __syncthreads();
  }
  const bool bz = Num<T>::is_zero(beta);
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      int64_t gi = i0 + tx + a * (BM / TM), gj = j0 + ty + b * (BN / TN);
      if (gi < m && gj < n) {
        T* p = C + gi + gj * ldc;
        T v = Num<T>::mul(alpha, acc[a][b]);
        *p = bz ? v : Num<T>::add(v, Num<T>::mul(beta, *p));
      }
    }
}

// two CTAs per SM (at most 128 registers): 16384^3 NN measured 37.9 -> 42.2 TFLOP/s
__global__ void __launch_bounds__(sg::THREADS, 2)
gemm_f32_sg(int opa, int opb, int64_t m, int64_t n, int64_t k, float alpha, const float* __restrict__ A, int64_t lda,
            const float* __restrict__ B, int64_t ldb, float beta, float* __restrict__ C, int64_t ldc) {
  __shared__ __align__(16) float smem[sg::SMEM_FLOATS];
  sg::tile(opa, opb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, (int64_t)blockIdx.x * sg::BM,
           (int64_t)blockIdx.y * sg::BN, smem);
}

template <typename T>
__global__ void scale_kernel(int64_t m, int64_t n, T beta, T* C, int64_t ldc) {
  int64_t total = m * n;
  bool bz = Num<T>::is_zero(beta);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % m, j = e / m;
    T* p = C + i + j * ldc;
    *p = bz ? Num<T>::zero() : Num<T>::mul(beta, *p);
  }
}

__global__ void fill_f64_kernel(double* X, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                                uint64_t seed, uint64_t id) {
  int64_t total = rows * cols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % rows, j = e / rows;
    X[i + j * ld] = tmm_gen_value(kind, param, seed, id, i, j, rows);
  }
}

template <typename T>
cudaError_t launch_simt(Op opa, Op opb, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda,
                        const T* B, int64_t ldb, T beta, T* C, int64_t ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  constexpr int BM = 64, BN = 64, BK = 16;
  dim3 grid((unsigned)((m + BM - 1) / BM), (unsigned)((n + BN - 1) / BN));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  gemm_simt<T, BM, BN, BK, 4, 4><<<grid, 256, 0, s>>>(opa, opb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_scale(int64_t m, int64_t n, T beta, T* C, int64_t ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  int64_t total = m * n;
  int blocks = (int)((total + 255) / 256 < 152 * 16 ? (total + 255) / 256 : 152 * 16);
  scale_kernel<T><<<blocks, 256, 0, s>>>(m, n, beta, C, ldc);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gemm_f64(Op opa, Op opb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                            int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                            cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  dim3 grid((unsigned)((m + DM_BM - 1) / DM_BM), (unsigned)((n + DM_BN - 1) / DM_BN));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  bool ta = opa != OP_N, tb = opb != OP_N;  // conjugation is the identity on reals
  if (!ta && !tb) gemm_f64_dmma<OP_N, OP_N><<<grid, DM_THREADS, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (!ta && tb) gemm_f64_dmma<OP_N, OP_T><<<grid, DM_THREADS, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (ta && !tb) gemm_f64_dmma<OP_T, OP_N><<<grid, DM_THREADS, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else gemm_f64_dmma<OP_T, OP_T><<<grid, DM_THREADS, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return cudaGetLastError();
}

cudaError_t launch_gemm_f32(Op opa, Op opb, int64_t m, int64_t n, int64_t k, float alpha, const float* A,
                            int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                            cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  dim3 grid((unsigned)((m + sg::BM - 1) / sg::BM), (unsigned)((n + sg::BN - 1) / sg::BN));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  gemm_f32_sg<<<grid, sg::THREADS, 0, s>>>(opa == OP_N ? 0 : 1, opb == OP_N ? 0 : 1, m, n, k, alpha, A, lda, B, ldb,
                                           beta, C, ldc);
  return cudaGetLastError();
}
cudaError_t launch_gemm_c32(Op opa, Op opb, int64_t m, int64_t n, int64_t k, cplxf alpha, const cplxf* A,
                            int64_t lda, const cplxf* B, int64_t ldb, cplxf beta, cplxf* C, int64_t ldc,
                            cudaStream_t s) {
  return launch_simt<cplxf>(opa, opb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
}
cudaError_t launch_gemm_c64(Op opa, Op opb, int64_t m, int64_t n, int64_t k, cplxd alpha, const cplxd* A,
                            int64_t lda, const cplxd* B, int64_t ldb, cplxd beta, cplxd* C, int64_t ldc,
                            cudaStream_t s) {
  return launch_simt<cplxd>(opa, opb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

cudaError_t launch_scale_f64(int64_t m, int64_t n, double beta, double* C, int64_t ldc, cudaStream_t s) {
  return launch_scale<double>(m, n, beta, C, ldc, s);
}
cudaError_t launch_scale_f32(int64_t m, int64_t n, float beta, float* C, int64_t ldc, cudaStream_t s) {
  return launch_scale<float>(m, n, beta, C, ldc, s);
}
cudaError_t launch_scale_c32(int64_t m, int64_t n, cplxf beta, cplxf* C, int64_t ldc, cudaStream_t s) {
  return launch_scale<cplxf>(m, n, beta, C, ldc, s);
}
cudaError_t launch_scale_c64(int64_t m, int64_t n, cplxd beta, cplxd* C, int64_t ldc, cudaStream_t s) {
  return launch_scale<cplxd>(m, n, beta, C, ldc, s);
}

cudaError_t launch_fill_f64(double* X, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                            uint64_t seed, uint64_t id, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  fill_f64_kernel<<<152 * 8, 256, 0, s>>>(X, rows, cols, ld, kind, param, seed, id);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ host <-> device tile copies by kernel
// A 2D copy (height rows of width bytes) done by loads and stores of the SMs, for host memory
// that the GPU reads and writes through the host page tables: unlike a copy-engine copy from
// pageable memory it needs no page-locked staging, and it stays asynchronous.  V is the
// widest access that every address, pitch and width allows.
template <typename V>
__global__ void copy2d_kernel(char* __restrict__ dst, size_t dpitch, const char* __restrict__ src, size_t spitch,
                              size_t nvec, size_t rows) {
  const size_t total = nvec * rows;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i / nvec, v = i - r * nvec;
    *reinterpret_cast<V*>(dst + r * dpitch + v * sizeof(V)) =
        *reinterpret_cast<const V*>(src + r * spitch + v * sizeof(V));
  }
}

cudaError_t copy2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t height,
                         cudaStream_t s) {
  if (width == 0 || height == 0) return cudaSuccess;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const uintptr_t bits = (uintptr_t)dst | (uintptr_t)src | dpitch | spitch | width;
  const size_t vb = (bits & 15) == 0 ? 16 : (bits & 7) == 0 ? 8 : (bits & 3) == 0 ? 4 : 1;
  const size_t nvec = width / vb, total = nvec * height;
  const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)sms * 4);
  switch (vb) {
    case 16: copy2d_kernel<uint4><<<grid, 256, 0, s>>>((char*)dst, dpitch, (const char*)src, spitch, nvec, height); break;
    case 8: copy2d_kernel<uint2><<<grid, 256, 0, s>>>((char*)dst, dpitch, (const char*)src, spitch, nvec, height); break;
    case 4: copy2d_kernel<uint32_t><<<grid, 256, 0, s>>>((char*)dst, dpitch, (const char*)src, spitch, nvec, height); break;
    default: copy2d_kernel<uint8_t><<<grid, 256, 0, s>>>((char*)dst, dpitch, (const char*)src, spitch, nvec, height);
  }
  return cudaGetLastError();
}

}  // namespace tmm
