// Batched GEMMs of uneven shapes and mixed precision in one persistent launch.
//
// No reference counterpart: users of the reference call gpu::gemm once per
// problem (src/Tiled-MM/tiled_mm.cpp:492-624), each call pinning, copying,
// launching per tile and synchronising the device.  Here a batch of problems
// (FP64 and FP32, any op(A)/op(B), any m, n, k) becomes one device work list
// of (problem, C tile) items walked by persistent CTAs:
//   FP64 items   64 x 64 tiles on the DMMA tensor path (mma.sync m16n8k4 f64),
//                8 warps of 32 x 16;
//   FP32 items   64 x 64 (4 x 4 per thread) or 128 x 128 (8 x 8 per thread,
//                the plain path's tile, tmm_sgemm_tile.cuh) SIMT tiles, the
//                shape picked per size class by the autotuner (tmm_autotune.cpp),
//                which times both on first use;
// the two item kinds run as two kernels on two streams, concurrently.
// Items are ordered by decreasing cost and dealt round-robin to the CTAs.
// With host operands in page-locked memory, the per-problem copies in, the
// launch and the copies out are captured once into a CUDA graph keyed by the
// batch layout and replayed by later calls with the same layout.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "tmm_batched.h"
#include "tmm_sgemm_tile.cuh"

namespace tmm {
namespace {

constexpr int THREADS = 256;
constexpr int BK = 16;

struct alignas(16) DevProblem {
  const void* a;
  const void* b;
  void* c;
  int64_t m, n, k, lda, ldb, ldc;
  double alpha, beta;
  int dtype, opa, opb, variant;
};

struct alignas(16) WorkItem {
  int problem;
  int ti, tj;  // C tile indices
  int pad;
};

__device__ __forceinline__ void dmma(double (&d)[4], double a0, double a1, double b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
      : "+d"(d[0]), "+d"(d[1]), "+d"(d[2]), "+d"(d[3])
      : "d"(a0), "d"(a1), "d"(b0));
}

// ---------------------------------------------------------------- FP64 64 x 64 tile (DMMA)
constexpr int D_BM = 64, D_BN = 64, D_S = 72;  // padded row stride in doubles

__device__ void tile_f64(const DevProblem& P, int64_t i0, int64_t j0, double* smem) {
  double* As = smem;              // [BK][D_S]
  double* Bs = smem + BK * D_S;   // [BK][D_S]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
  const double* A = (const double*)P.a;
  const double* B = (const double*)P.b;
  double acc[2][2][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.0;
  for (int64_t l0 = 0; l0 < P.k; l0 += BK) {
    // 64 x 16 A and 16 x 64 B elements, 4 each per thread, coalesced along the stored leading dimension
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + q * THREADS;
      int ii, ll;
      if (P.opa == OP_N) { ii = idx % D_BM; ll = idx / D_BM; } else { ll = idx % BK; ii = idx / BK; }
      const int64_t gi = i0 + ii, gl = l0 + ll;
      double v = 0.0;
      if (gi < P.m && gl < P.k) v = P.opa == OP_N ? A[gi + gl * P.lda] : A[gl + gi * P.lda];
      As[ll * D_S + ii] = v;
      int jj;
      if (P.opb == OP_N) { ll = idx % BK; jj = idx / BK; } else { jj = idx % D_BN; ll = idx / D_BN; }
      const int64_t gj = j0 + jj, gl2 = l0 + ll;
      double w = 0.0;
      if (gj < P.n && gl2 < P.k) w = P.opb == OP_N ? B[gl2 + gj * P.ldb] : B[gj + gl2 * P.ldb];
      Bs[ll * D_S + jj] = w;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 4) {
      double af[2][2], bf[2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        af[a][0] = As[(ks + t) * D_S + wm + a * 16 + g];
        af[a][1] = As[(ks + t) * D_S + wm + a * 16 + g + 8];
      }
#pragma unroll
      for (int b = 0; b < 2; ++b) bf[b] = Bs[(ks + t) * D_S + wn + b * 8 + g];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) dmma(acc[a][b], af[a][0], af[a][1], bf[b]);
    }
    __syncthreads();
  }
  double* C = (double*)P.c;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int64_t gi = i0 + wm + a * 16 + g + ((c >> 1) << 3);
        const int64_t gj = j0 + wn + b * 8 + 2 * t + (c & 1);
        if (gi < P.m && gj < P.n) {
          double* p = C + gi + gj * P.ldc;
          const double v = P.alpha * acc[a][b][c];
          *p = P.beta == 0.0 ? v : fma(P.beta, *p, v);
        }
      }
}

// ---------------------------------------------------------------- FP32 SIMT tiles
template <int BM, int BN, int TM, int TN>
__device__ void tile_f32(const DevProblem& P, int64_t i0, int64_t j0, float* smem) {
  static_assert((BM / TM) * (BN / TN) == THREADS, "thread layout");
  constexpr int KS = 8;
  float* As = smem;                 // [KS][BM + 4]
  float* Bs = smem + KS * (BM + 4);  // [KS][BN + 4]
  const int tid = threadIdx.x;
  const int tx = tid % (BM / TM), ty = tid / (BM / TM);
  const float* A = (const float*)P.a;
  const float* B = (const float*)P.b;
  const float alpha = (float)P.alpha, beta = (float)P.beta;
  float acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = 0.f;
  for (int64_t l0 = 0; l0 < P.k; l0 += KS) {
    for (int idx = tid; idx < BM * KS; idx += THREADS) {
      int ii, ll;
      if (P.opa == OP_N) { ii = idx % BM; ll = idx / BM; } else { ll = idx % KS; ii = idx / KS; }
      const int64_t gi = i0 + ii, gl = l0 + ll;
      As[ll * (BM + 4) + ii] = (gi < P.m && gl < P.k) ? (P.opa == OP_N ? A[gi + gl * P.lda] : A[gl + gi * P.lda]) : 0.f;
    }
    for (int idx = tid; idx < BN * KS; idx += THREADS) {
      int jj, ll;
      if (P.opb == OP_N) { ll = idx % KS; jj = idx / KS; } else { jj = idx % BN; ll = idx / BN; }
      const int64_t gj = j0 + jj, gl = l0 + ll;
      Bs[ll * (BN + 4) + jj] = (gj < P.n && gl < P.k) ? (P.opb == OP_N ? B[gl + gj * P.ldb] : B[gj + gl * P.ldb]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < KS; ++ll) {
      float ar[TM], br[TN];
#pragma unroll
      for (int a = 0; a < TM; ++a) ar[a] = As[ll * (BM + 4) + tx + a * (BM / TM)];
#pragma unroll
      for (int b = 0; b < TN; ++b) br[b] = Bs[ll * (BN + 4) + ty + b * (BN / TN)];
#pragma unroll
      for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = fmaf(ar[a], br[b], acc[a][b]);
    }
    __syncthreads();
  }
  float* C = (float*)P.c;
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const int64_t gi = i0 + tx + a * (BM / TM), gj = j0 + ty + b * (BN / TN);
      if (gi < P.m && gj < P.n) {
        float* p = C + gi + gj * P.ldc;
        const float v = alpha * acc[a][b];
        *p = beta == 0.f ? v : v + beta * *p;
      }
    }
}

constexpr size_t SMEM_F64 = 2 * BK * D_S * sizeof(double);  // 18 KB

// FP64 and FP32 items run in two kernels (on two streams, concurrently): each
// keeps its own register budget, and the FP64 items (DMMA) and the FP32 items
// (FFMA) use different pipes of the same SMs.
__global__ void __launch_bounds__(THREADS)
grouped_f64(const DevProblem* __restrict__ probs, const WorkItem* __restrict__ work, int n_work) {
  __shared__ __align__(16) double smem[SMEM_F64 / sizeof(double)];
  for (int w = blockIdx.x; w < n_work; w += gridDim.x) {
    const WorkItem it = work[w];
    const DevProblem P = probs[it.problem];
    tile_f64(P, (int64_t)it.ti * D_BM, (int64_t)it.tj * D_BN, smem);
    __syncthreads();  // shared memory is reused by the next item
  }
}

__global__ void __launch_bounds__(THREADS)
grouped_f32(const DevProblem* __restrict__ probs, const WorkItem* __restrict__ work, int n_work) {
  __shared__ __align__(16) float smem[sg::SMEM_FLOATS];
  for (int w = blockIdx.x; w < n_work; w += gridDim.x) {
    const WorkItem it = work[w];
    const DevProblem P = probs[it.problem];
    if (P.variant == BATCH_F32_128)
      sg::tile(P.opa == OP_N ? 0 : 1, P.opb == OP_N ? 0 : 1, P.m, P.n, P.k, (float)P.alpha, (const float*)P.a, P.lda,
               (const float*)P.b, P.ldb, (float)P.beta, (float*)P.c, P.ldc, (int64_t)it.ti * sg::BM,
               (int64_t)it.tj * sg::BN, smem);
    else
      tile_f32<64, 64, 4, 4>(P, (int64_t)it.ti * 64, (int64_t)it.tj * 64, smem);
    __syncthreads();
  }
}

// k == 0: C = beta * C
__global__ void scale_items(const DevProblem* __restrict__ probs, int count) {
  for (int p = 0; p < count; ++p) {
    const DevProblem P = probs[p];
    if (P.k != 0) continue;
    const int64_t total = P.m * P.n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
      const int64_t i = e % P.m, j = e / P.m;
      if (P.dtype == TMM_DOUBLE) {
        double* c = (double*)P.c + i + j * P.ldc;
        *c = P.beta == 0.0 ? 0.0 : P.beta * *c;
      } else {
        float* c = (float*)P.c + i + j * P.ldc;
        *c = P.beta == 0.0 ? 0.f : (float)P.beta * *c;
      }
    }
  }
}

int64_t tile_rows(int dtype, int variant) { return dtype == TMM_DOUBLE ? D_BM : (variant == BATCH_F32_128 ? 128 : 64); }

}  // namespace

int64_t batch_item_cost(int dtype, int variant, int64_t k) {
  // FP64 issues ~70x slower than FP32 on this part; the cost orders items for round-robin dealing
  const int64_t t = tile_rows(dtype, variant);
  return (dtype == TMM_DOUBLE ? 70 : 1) * t * t * (k > 0 ? k : 1);
}

int batch_plan(const std::vector<BatchProblem>& probs, std::vector<unsigned char>& dev_probs_bytes,
               std::vector<unsigned char>& work_bytes, int* n_work, int* n_f64) {
  std::vector<DevProblem> dp(probs.size());
  struct Item {
    WorkItem w;
    int64_t cost;
    int f64;
  };
  std::vector<Item> items;
  for (size_t i = 0; i < probs.size(); ++i) {
    const BatchProblem& p = probs[i];
    DevProblem& d = dp[i];
    d.a = p.a;
    d.b = p.b;
    d.c = p.c;
    d.m = p.m;
    d.n = p.n;
    d.k = p.k;
    d.lda = p.lda;
    d.ldb = p.ldb;
    d.ldc = p.ldc;
    d.alpha = p.alpha;
    d.beta = p.beta;
    d.dtype = p.dtype;
    d.opa = p.opa;
    d.opb = p.opb;
    d.variant = p.variant;
    if (p.k == 0 || p.m == 0 || p.n == 0) continue;
    const int64_t tr = tile_rows(p.dtype, p.variant);
    const int64_t tm = (p.m + tr - 1) / tr, tn = (p.n + tr - 1) / tr;
    const int64_t cost = batch_item_cost(p.dtype, p.variant, p.k);
    for (int64_t a = 0; a < tm; ++a)
      for (int64_t b = 0; b < tn; ++b) items.push_back({{(int)i, (int)a, (int)b, 0}, cost, p.dtype == TMM_DOUBLE});
  }
  // FP64 items first (their kernel reads the front of the list), each part by decreasing cost
  std::stable_sort(items.begin(), items.end(), [](const Item& x, const Item& y) {
    return x.f64 != y.f64 ? x.f64 > y.f64 : x.cost > y.cost;
  });
  std::vector<WorkItem> w(items.size());
  int f64 = 0;
  for (size_t i = 0; i < items.size(); ++i) {
    w[i] = items[i].w;
    f64 += items[i].f64;
  }
  dev_probs_bytes.assign((const unsigned char*)dp.data(), (const unsigned char*)dp.data() + dp.size() * sizeof(DevProblem));
  work_bytes.assign((const unsigned char*)w.data(), (const unsigned char*)w.data() + w.size() * sizeof(WorkItem));
  *n_work = (int)w.size();
  *n_f64 = f64;
  return 0;
}

size_t batch_problem_record_bytes() { return sizeof(DevProblem); }
size_t batch_work_record_bytes() { return sizeof(WorkItem); }

cudaError_t batch_launch(const void* dev_probs, int count, const void* dev_work, int n_f64, int n_f32, int any_k0,
                         cudaStream_t s, cudaStream_t s2, cudaEvent_t fork, cudaEvent_t join) {
  static int sms = 0, occ64 = 0, occ32 = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, grouped_f64, THREADS, 0) != cudaSuccess || occ64 < 1) occ64 = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ32, grouped_f32, THREADS, 0) != cudaSuccess || occ32 < 1) occ32 = 1;
    cudaGetLastError();
  }
  if (any_k0) {
    scale_items<<<sms * 4, 256, 0, s>>>((const DevProblem*)dev_probs, count);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const WorkItem* w = (const WorkItem*)dev_work;
  const bool both = n_f64 > 0 && n_f32 > 0 && s2 && fork && join;
  if (both) {  // fork the FP32 items onto the second stream, join before returning
    cudaError_t e = cudaEventRecord(fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, fork, 0);
    if (e != cudaSuccess) return e;
  }
  if (n_f64 > 0) {
    grouped_f64<<<std::min(n_f64, sms * occ64), THREADS, 0, s>>>((const DevProblem*)dev_probs, w, n_f64);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (n_f32 > 0) {
    cudaStream_t t = both ? s2 : s;
    grouped_f32<<<std::min(n_f32, sms * occ32), THREADS, 0, t>>>((const DevProblem*)dev_probs, w + n_f64, n_f32);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (both) {
    cudaError_t e = cudaEventRecord(join, s2);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace tmm
