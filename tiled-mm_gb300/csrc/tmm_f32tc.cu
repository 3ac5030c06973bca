// FP32 GEMM on the tcgen05 tensor cores: the per-tile multiply of float
// contexts (the reference calls cublasSgemm per tile, src/Tiled-MM/tiled_mm.cpp:181-198).
//
// Split (published: the multi-word bf16 splitting of FP32 operands, e.g. Henry,
// Tang, Heinecke, "Leveraging the bfloat16 artificial intelligence datatype for
// higher-precision computations", ARITH 2019): every FP32 x is the exact sum
//     x = hi + mid + lo,  hi = bf16(x), mid = bf16(x - hi), lo = bf16(x - hi - mid)
// (round to nearest; each subtraction is exact, and 3 x 8 significand bits cover
// FP32's 24).  A product x * y keeps the six terms whose weight is at least
// 2^-16 of x * y -- lo*hi, hi*lo, mid*mid, mid*hi, hi*mid, hi*hi, summed in that
// order (smallest first) -- each of them exact in FP32; the three dropped terms
// are below 2^-23 |x y| together.  The terms accumulate in FP32 in tensor memory
// over the whole k range, as an FP32 GEMM does, and the epilogue computes
// C = alpha * acc + beta * C in FP32.  An Inf or a NaN keeps its hi part and has
// zero mid and lo parts, so non-finite values reach the product (Inf times a zero
// part gives NaN where IEEE arithmetic could give +-Inf).
//
// Kernel (one CTA per SM, persistent over 128 x 256 tiles of C):
//   warp 0      TMA producer: the A plane box (128 lines x 128 bytes = 64 k) and
//               two B plane boxes per k-block into a 4-stage ring (SWIZZLE_128B);
//   warp 1      allocates 2 x 256 TMEM columns; one thread issues
//               tcgen05.mma.cta_group::1.kind::f16 (bf16 x bf16 -> f32, M 128,
//               N 256, K 16) for the tile's 6 x k/64 k-blocks into one accumulator
//               and commits it to the epilogue; the next tile uses the other one;
//   warps 2-5   drain the accumulator (one TMEM lane = one row of C per thread) and
//               store alpha * acc + beta * C.
// Planes use the blocked layout of the Ozaki digit planes: [plane][rows/128][k/64]
// [128 lines][64 bf16], so every box is one contiguous 16 KB block.  Every
// mbarrier wait is bounded (about a second), after which an error word is set and
// the CTA winds down.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "tmm_f32tc.h"
#include "tmm_tc_ptx.cuh"

namespace tmm {
namespace f32tc {

using namespace tmm::tc;

constexpr int BM = 128, BN = 256, KE = 64, KBYTES = 128;  // KE bf16 = KBYTES bytes per k-block
constexpr int LINE_BLOCK = 128;
constexpr int PLANES = 3, NPAIRS = 6;
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * KBYTES, B_BYTES = BN * KBYTES, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int THREADS = 192;
constexpr int TMEM_COLS = 512;
constexpr size_t SMEM_BYTES = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
constexpr int GROUP_M = 16;
constexpr uint32_t EPI_WAIT_HINT_NS = 20000;

// (A plane, B plane) of the six kept terms, smallest weight first: lo*hi, hi*lo, mid*mid,
// mid*hi, hi*mid, hi*hi (plane 0 = hi, 1 = mid, 2 = lo)
__host__ __device__ __forceinline__ int pair_a(int p) { return (0x001102 >> (4 * p)) & 0xF; }
__host__ __device__ __forceinline__ int pair_b(int p) { return (0x010120 >> (4 * p)) & 0xF; }

// kind::f16: D f32 (bits 4-5 = 1), A bf16 (bits 7-9 = 1), B bf16 (bits 10-12 = 1), both
// K-major, N = 256 (bits 17-22: N >> 3), M = 128 (bits 24-28: M >> 4)
constexpr uint32_t IDESC_BF16 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(IDESC_BF16), "r"(accumulate));
}

// row of 128 bytes (in the tensor map's view of the planes) where the box of plane p,
// lines line .. line + 127 (line a multiple of 128), k-block kb starts
__device__ __forceinline__ int box_y(int p, int64_t line, int kb, int64_t rows_pad, int nkb) {
  return (int)((((int64_t)p * (rows_pad / LINE_BLOCK) + line / LINE_BLOCK) * nkb + kb) * LINE_BLOCK);
}

__device__ __forceinline__ void tile_coords(int tile, int tiles_m, int tiles_n, int group, int* tm, int* tn) {
  const int per_band = group * tiles_n;
  const int band = tile / per_band, local = tile - band * per_band;
  const int rows_in_band = min(group, tiles_m - band * group);
  *tm = band * group + local % rows_in_band;
  *tn = local / rows_in_band;
}

struct Params {
  int64_t a_rows_pad, b_rows_pad;
  int nkb;
  int64_t m, n;
  float alpha, beta;
  float* C;
  int64_t ldc;
  int* err;
  int tiles_m, tiles_n;
};

// A product of a grouped launch (f32tc_gemm_grouped): its planes start at 128-byte row
// a_row0 / b_row0 of the launch's one tensor map over the arena of all products' planes.
struct GroupProblem {
  int64_t a_row0, b_row0, a_rows_pad, b_rows_pad;
  float* C;
  int64_t ldc, m, n;
  float alpha, beta;
  int nkb, pad;
};
struct GroupArgs {
  const GroupProblem* probs;
  const int4* items;  // (problem, 128-row tile, 256-column tile, unused)
  int n_items;
};

// A tile of a launch and its product's geometry and epilogue operands.
struct Job {
  int tm, tn, nkb;
  int64_t a_row0, b_row0, a_rows_pad, b_rows_pad;
  float* C;
  int64_t ldc, m, n;
  float alpha, beta;
};
template <bool GROUPED>
__device__ __forceinline__ Job job_of(int ct, const Params& P, const GroupArgs& G) {
  Job j;
  if (GROUPED) {
    const int4 it = G.items[ct];
    const GroupProblem& q = G.probs[it.x];
    j.tm = it.y;
    j.tn = it.z;
    j.nkb = q.nkb;
    j.a_row0 = q.a_row0;
    j.b_row0 = q.b_row0;
    j.a_rows_pad = q.a_rows_pad;
    j.b_rows_pad = q.b_rows_pad;
    j.C = q.C;
    j.ldc = q.ldc;
    j.m = q.m;
    j.n = q.n;
    j.alpha = q.alpha;
    j.beta = q.beta;
  } else {
    tile_coords(ct, P.tiles_m, P.tiles_n, GROUP_M, &j.tm, &j.tn);
    j.nkb = P.nkb;
    j.a_row0 = j.b_row0 = 0;
    j.a_rows_pad = P.a_rows_pad;
    j.b_rows_pad = P.b_rows_pad;
    j.C = P.C;
    j.ldc = P.ldc;
    j.m = P.m;
    j.n = P.n;
    j.alpha = P.alpha;
    j.beta = P.beta;
  }
  return j;
}

// ------------------------------------------------------------------ split: FP32 -> 3 bf16 planes
constexpr int SPL = 64, SP_THREADS = 256;

template <int TRANS>  // 0: line r, entry l at X[r + l ld];  1: at X[l + r ld]
__global__ void __launch_bounds__(SP_THREADS)
f32tc_split_kernel(const float* __restrict__ X, int64_t ld, int64_t rows, int64_t kk, __nv_bfloat16* __restrict__ planes,
                   int64_t rows_pad, int64_t k_pad) {
  __shared__ float tile[SPL][SPL + 1];
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * SPL, l0 = (int64_t)blockIdx.y * SPL;
  if (TRANS == 0) {
    const int r = tid & 63;
    for (int c = tid >> 6; c < SPL; c += SP_THREADS / SPL) {
      const int64_t l = l0 + c;
      tile[r][c] = (r0 + r < rows && l < kk) ? X[(r0 + r) + l * ld] : 0.0f;
    }
  } else {
    const int c = tid & 63;
    for (int r = tid >> 6; r < SPL; r += SP_THREADS / SPL) {
      const int64_t l = l0 + c;
      tile[r][c] = (r0 + r < rows && l < kk) ? X[l + (r0 + r) * ld] : 0.0f;
    }
  }
  __syncthreads();
  const int r = tid >> 2, c0 = (tid & 3) * 16;
  const int64_t line = r0 + r;
  const int nkb = (int)(k_pad / KE);
  const size_t plane_elems = (size_t)rows_pad * (size_t)k_pad;
  const size_t off = ((size_t)(line / LINE_BLOCK) * nkb + (size_t)(l0 / KE)) * (LINE_BLOCK * KE) +
                     (size_t)(line % LINE_BLOCK) * KE + (size_t)c0;
  __align__(16) __nv_bfloat16 hv[16], mv[16], lv[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float x = tile[r][c0 + j];
    if (!isfinite(x)) {
      hv[j] = __float2bfloat16_rn(x);
      mv[j] = __float2bfloat16_rn(0.0f);
      lv[j] = __float2bfloat16_rn(0.0f);
      continue;
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 md = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(md);
    hv[j] = h;
    mv[j] = md;
    lv[j] = __float2bfloat16_rn(r2);
  }
  const uint4* hs = (const uint4*)hv;
  const uint4* ms = (const uint4*)mv;
  const uint4* ls = (const uint4*)lv;
  uint4* d0 = (uint4*)(planes + off);
  uint4* d1 = (uint4*)(planes + plane_elems + off);
  uint4* d2 = (uint4*)(planes + 2 * plane_elems + off);
  d0[0] = hs[0];
  d0[1] = hs[1];
  d1[0] = ms[0];
  d1[1] = ms[1];
  d2[0] = ls[0];
  d2[1] = ls[1];
}

// ------------------------------------------------------------------ GEMM
template <bool GROUPED>
__global__ void __launch_bounds__(THREADS, 1)
f32tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const Params P,
                  const GroupArgs G) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + (size_t)STAGES * STAGE_BYTES);
  // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2]
  volatile int* abort_flag = (volatile int*)(bars + 2 * STAGES + 4);
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 5);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);
  const uint32_t tfull0 = smem_u32(bars + 2 * STAGES), tempty0 = smem_u32(bars + 2 * STAGES + 2);
  const int total_tiles = GROUPED ? G.n_items : P.tiles_m * P.tiles_n;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(empty0 + 8 * i, 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(tfull0 + 8 * i, 1);
      mbar_init(tempty0 + 8 * i, 4);  // one arrival per epilogue warp
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0 && lane == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tmem_slot), TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------------------------------------------------------- TMA producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int ct = blockIdx.x; ct < total_tiles && ok; ct += gridDim.x) {
        const Job J = job_of<GROUPED>(ct, P, G);
        const int steps = NPAIRS * J.nkb;  // k-blocks of this tile
        for (int t = 0; t < steps && ok; ++t) {
          const int pr = t / J.nkb, kb = t - pr * J.nkb;
          ok = mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, P.err);
          if (!ok) break;
          const uint32_t fb = full0 + 8 * stage;
          mbar_expect_tx(fb, STAGE_BYTES);
          uint8_t* sa = smem + (size_t)stage * STAGE_BYTES;
          tma_load_2d(smem_u32(sa), &tmA, 0,
                      (int)(J.a_row0 + box_y(pair_a(pr), (int64_t)J.tm * BM, kb, J.a_rows_pad, J.nkb)), fb);
#pragma unroll
          for (int j = 0; j < BN / LINE_BLOCK; ++j)
            tma_load_2d(smem_u32(sa + A_BYTES + j * LINE_BLOCK * KBYTES), &tmB, 0,
                        (int)(J.b_row0 + box_y(pair_b(pr), (int64_t)J.tn * BN + j * LINE_BLOCK, kb, J.b_rows_pad,
                                               J.nkb)), fb);
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // every issued copy has landed before the CTA may exit (bounded)
      for (int i = 0; i < STAGES; ++i) {
        (void)mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, P.err);
        if (++stage == STAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer
    if (lane == 0) {
      constexpr uint64_t STAGE_STEP = (uint64_t)(STAGE_BYTES >> 4);
      const uint32_t sa0 = smem_u32(smem);
      const uint64_t ad0 = smem_desc(sa0), bd0 = smem_desc(sa0 + A_BYTES);
      int stage = 0, buf = 0;
      uint32_t phase = 0, tph = 0;  // tph bit b: phase of accumulator b's full barrier
      bool ok = true;
      for (int ct = blockIdx.x; ct < total_tiles && ok; ct += gridDim.x) {
        const int steps = NPAIRS * (GROUPED ? G.probs[G.items[ct].x].nkb : P.nkb);
        // the accumulator is free once the epilogue has drained its previous tile
        ok = mbar_wait(tempty0 + 8 * buf, ((tph >> buf) & 1u) ^ 1u, abort_flag, P.err);
        if (!ok) break;
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + (uint32_t)(buf * BN);
        for (int t = 0; t < steps; ++t) {
          ok = mbar_wait(full0 + 8 * stage, phase, abort_flag, P.err);
          if (!ok) break;
          tc_fence_after();
          const uint64_t ad = ad0 + (uint64_t)stage * STAGE_STEP, bd = bd0 + (uint64_t)stage * STAGE_STEP;
          // K = 16 bf16 = 32 bytes per MMA: +2 in the 16-byte address field
          mma_bf16(d_tmem, ad, bd, t > 0 ? 1u : 0u);
          mma_bf16(d_tmem, ad + 2, bd + 2, 1u);
          mma_bf16(d_tmem, ad + 4, bd + 4, 1u);
          mma_bf16(d_tmem, ad + 6, bd + 6, 1u);
          mma_commit(empty0 + 8 * stage);  // the stage is free when these MMAs have read it
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (!ok) break;
        mma_commit(tfull0 + 8 * buf);  // the tile's sum is complete when its MMAs are
        tph ^= 1u << buf;
        buf ^= 1;
      }
      // wait (bounded) for the MMAs in flight before TMEM is freed
      for (int b = 0; b < 2; ++b) {
        (void)mbar_wait(tempty0 + 8 * buf, ((tph >> buf) & 1u) ^ 1u, abort_flag, P.err);
        buf ^= 1;
      }
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2..5)
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    uint32_t tphase[2] = {0, 0};
    int buf = 0;
    for (int ct = blockIdx.x; ct < total_tiles; ct += gridDim.x) {
      const Job J = job_of<GROUPED>(ct, P, G);
      int okw = 1;
      if (lane == 0) okw = mbar_wait(tfull0 + 8 * buf, tphase[buf], abort_flag, P.err, EPI_WAIT_HINT_NS) ? 1 : 0;
      const bool ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
      __syncwarp();
      if (!ok) break;
      tc_fence_after();
      const uint32_t tbase = tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * BN);
      const int64_t gi = (int64_t)J.tm * BM + row;
      const bool row_ok = gi < J.m;
      const bool read_c = J.beta != 0.0f;
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        uint32_t r[32];
        tmem_ld32(tbase + (uint32_t)(c * 32), r);
        tmem_ld_wait(r);
        if (c == BN / 32 - 1) {  // accumulator consumed: hand it back to the MMA warp
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(tempty0 + 8 * buf);
        }
        const int64_t gj0 = (int64_t)J.tn * BN + c * 32;
        if (!row_ok || gj0 >= J.n) continue;
        const int nv = J.n - gj0 < 32 ? (int)(J.n - gj0) : 32;
        float* cp = J.C + gi + gj0 * J.ldc;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          if (j >= nv) break;
          const float acc = __uint_as_float(r[j]);
          float* q = cp + (int64_t)j * J.ldc;
          *q = read_c ? fmaf(J.alpha, acc, J.beta * *q) : J.alpha * acc;
        }
      }
      tphase[buf] ^= 1;
      buf ^= 1;
    }
  }
  tc_fence_before();
  __syncwarp();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// ------------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

// the planes as one column of 128-byte rows; a box is 128 of them (one contiguous 16 KB block)
cudaError_t make_map(CUtensorMap* map, const void* planes, int64_t rows_pad, int64_t k_pad) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {(cuuint64_t)KBYTES, (cuuint64_t)PLANES * (cuuint64_t)rows_pad * (cuuint64_t)(k_pad / KE)};
  cuuint64_t strides[1] = {(cuuint64_t)KBYTES};
  cuuint32_t box[2] = {(cuuint32_t)KBYTES, (cuuint32_t)LINE_BLOCK};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(planes), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

struct DeviceSetup {
  std::once_flag once;
  cudaError_t status = cudaSuccess;
  int sms = 0;
};
constexpr int MAX_DEVICES = 64;
DeviceSetup g_setup[MAX_DEVICES];

const DeviceSetup* device_setup() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return nullptr;
  DeviceSetup& d = g_setup[dev];
  std::call_once(d.once, [&d, dev] {
    d.status = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (d.status != cudaSuccess) return;
    if (d.sms <= 0) d.sms = 1;
    d.status = cudaFuncSetAttribute(f32tc_gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (d.status != cudaSuccess) return;
    d.status = cudaFuncSetAttribute(f32tc_gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
  });
  return &d;
}

int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }
size_t plane_bytes(int64_t lines, int64_t kk) {
  const size_t b = (size_t)PLANES * (size_t)round_up(lines > 0 ? lines : 1, 256) * (size_t)round_up(kk > 0 ? kk : 1, KE) * 2;
  return (b + 1023) / 1024 * 1024;
}

}  // namespace f32tc

size_t f32tc_plane_bytes(int64_t lines, int64_t k) { return f32tc::plane_bytes(lines, k); }

cudaError_t f32tc_split_lines(const float* X, int64_t ld, bool lines_contiguous, int64_t lines, int64_t k,
                              void* planes, cudaStream_t s) {
  using namespace f32tc;
  if (lines <= 0 || k <= 0) return cudaSuccess;
  const int64_t rows_pad = round_up(lines, 256), k_pad = round_up(k, KE);
  if (k_pad / SPL > 65535) return cudaErrorInvalidValue;
  const dim3 g((unsigned)(rows_pad / SPL), (unsigned)(k_pad / SPL));
  if (lines_contiguous)
    f32tc_split_kernel<0><<<g, SP_THREADS, 0, s>>>(X, ld, lines, k, (__nv_bfloat16*)planes, rows_pad, k_pad);
  else
    f32tc_split_kernel<1><<<g, SP_THREADS, 0, s>>>(X, ld, lines, k, (__nv_bfloat16*)planes, rows_pad, k_pad);
  return cudaGetLastError();
}

cudaError_t f32tc_grouped_image(const std::vector<F32GroupedProduct>& prods, const void* arena, size_t arena_bytes,
                                std::vector<unsigned char>& out, int* n_items) {
  using namespace f32tc;
  std::vector<GroupProblem> recs;
  std::vector<int4> items;
  std::vector<int64_t> cost;
  for (const F32GroupedProduct& p : prods) {
    if (p.m <= 0 || p.n <= 0 || p.k <= 0) continue;
    const int64_t aoff = (const char*)p.a_planes - (const char*)arena, boff = (const char*)p.b_planes - (const char*)arena;
    if (aoff < 0 || boff < 0 || aoff % KBYTES || boff % KBYTES) return cudaErrorInvalidValue;
    // every box of the planes lies inside the arena that the launch's tensor map covers
    if ((size_t)aoff + plane_bytes(p.m, p.k) > arena_bytes || (size_t)boff + plane_bytes(p.n, p.k) > arena_bytes)
      return cudaErrorInvalidValue;
    GroupProblem r;
    r.a_row0 = aoff / KBYTES;
    r.b_row0 = boff / KBYTES;
    r.a_rows_pad = round_up(p.m, 256);
    r.b_rows_pad = round_up(p.n, 256);
    r.C = p.C;
    r.ldc = p.ldc;
    r.m = p.m;
    r.n = p.n;
    r.alpha = p.alpha;
    r.beta = p.beta;
    r.nkb = (int)(round_up(p.k, KE) / KE);
    r.pad = 0;
    const int idx = (int)recs.size();
    recs.push_back(r);
    for (int tm = 0; tm < (int)((p.m + BM - 1) / BM); ++tm)
      for (int tn = 0; tn < (int)((p.n + BN - 1) / BN); ++tn) {
        items.push_back(make_int4(idx, tm, tn, 0));
        cost.push_back((int64_t)r.nkb);
      }
  }
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
  const size_t rec_bytes = (recs.size() * sizeof(GroupProblem) + 255) / 256 * 256;
  out.assign(rec_bytes + items.size() * sizeof(int4), 0);
  if (!recs.empty()) memcpy(out.data(), recs.data(), recs.size() * sizeof(GroupProblem));
  int4* it = (int4*)(out.data() + rec_bytes);
  for (size_t i = 0; i < order.size(); ++i) it[i] = items[order[i]];
  *n_items = (int)items.size();
  return cudaSuccess;
}

size_t f32tc_grouped_image_bound(const std::vector<F32GroupedProduct>& prods) {
  size_t tiles = 0;
  for (const auto& p : prods) tiles += (size_t)((p.m + 127) / 128) * (size_t)((p.n + 255) / 256);
  return (prods.size() * sizeof(f32tc::GroupProblem) + 255) / 256 * 256 + tiles * sizeof(int4);
}

cudaError_t f32tc_gemm_grouped(const void* arena, size_t arena_bytes, const void* dev_image, int n_probs, int n_items,
                               int* err, cudaStream_t s) {
  using namespace f32tc;
  if (n_items <= 0) return cudaSuccess;
  if (!arena || !dev_image || !err || arena_bytes / KBYTES > (size_t)INT32_MAX) return cudaErrorInvalidValue;
  const DeviceSetup* d = device_setup();
  if (!d) return cudaErrorInvalidDevice;
  if (d->status != cudaSuccess) return d->status;
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  CUtensorMap map;
  cuuint64_t dims[2] = {(cuuint64_t)KBYTES, (cuuint64_t)(arena_bytes / KBYTES)};
  cuuint64_t strides[1] = {(cuuint64_t)KBYTES};
  cuuint32_t box[2] = {(cuuint32_t)KBYTES, (cuuint32_t)LINE_BLOCK};
  cuuint32_t estr[2] = {1, 1};
  if (fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(arena), dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  Params P{};
  P.err = err;
  const size_t rec_bytes = ((size_t)n_probs * sizeof(GroupProblem) + 255) / 256 * 256;
  const GroupArgs G{(const GroupProblem*)dev_image, (const int4*)((const char*)dev_image + rec_bytes), n_items};
  const int ctas = n_items < d->sms ? n_items : d->sms;
  f32tc_gemm_kernel<true><<<ctas, THREADS, SMEM_BYTES, s>>>(map, map, P, G);
  return cudaGetLastError();
}

size_t f32tc_scratch_bytes(int64_t m, int64_t n, int64_t k) {
  return 256 + f32tc::plane_bytes(m, k) + f32tc::plane_bytes(n, k);
}

cudaError_t f32tc_prepare() {
  if (!f32tc::encode_fn()) return cudaErrorNotSupported;
  const f32tc::DeviceSetup* d = f32tc::device_setup();
  return d ? d->status : cudaErrorInvalidDevice;
}

cudaError_t f32tc_gemm(Op opa, Op opb, int64_t m, int64_t n, int64_t k, float alpha, const float* A, int64_t lda,
                       const float* B, int64_t ldb, float beta, float* C, int64_t ldc, void* scratch,
                       size_t scratch_bytes, cudaStream_t s) {
  using namespace f32tc;
  if (m <= 0 || n <= 0) return cudaSuccess;
  if (k <= 0 || !A || !B || !C || !scratch || scratch_bytes < f32tc_scratch_bytes(m, n, k)) return cudaErrorInvalidValue;
  const DeviceSetup* d = device_setup();
  if (!d) return cudaErrorInvalidDevice;
  if (d->status != cudaSuccess) return d->status;
  const int64_t a_rows_pad = round_up(m, 256), b_rows_pad = round_up(n, 256), k_pad = round_up(k, KE);
  // TMA coordinates are 32-bit: every 128-byte row of the stacked planes must stay addressable
  if ((int64_t)PLANES * std::max(a_rows_pad, b_rows_pad) * (k_pad / KE) > INT32_MAX) return cudaErrorInvalidValue;
  if (k_pad / SPL > 65535) return cudaErrorInvalidValue;  // the split grid's y extent
  char* base = (char*)scratch;
  int* err = (int*)base;  // the first 256 bytes: the error word of the bounded waits (zeroed by the caller)
  __nv_bfloat16* pa = (__nv_bfloat16*)(base + 256);
  __nv_bfloat16* pb = (__nv_bfloat16*)(base + 256 + plane_bytes(m, k));
  // lines of A: rows of op(A); lines of B: columns of op(B)
  const dim3 ga((unsigned)(a_rows_pad / SPL), (unsigned)(k_pad / SPL)), gb((unsigned)(b_rows_pad / SPL), (unsigned)(k_pad / SPL));
  if (opa == OP_N) f32tc_split_kernel<0><<<ga, SP_THREADS, 0, s>>>(A, lda, m, k, pa, a_rows_pad, k_pad);
  else f32tc_split_kernel<1><<<ga, SP_THREADS, 0, s>>>(A, lda, m, k, pa, a_rows_pad, k_pad);
  if (opb == OP_N) f32tc_split_kernel<1><<<gb, SP_THREADS, 0, s>>>(B, ldb, n, k, pb, b_rows_pad, k_pad);
  else f32tc_split_kernel<0><<<gb, SP_THREADS, 0, s>>>(B, ldb, n, k, pb, b_rows_pad, k_pad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  CUtensorMap ma, mb;
  e = make_map(&ma, pa, a_rows_pad, k_pad);
  if (e == cudaSuccess) e = make_map(&mb, pb, b_rows_pad, k_pad);
  if (e != cudaSuccess) return e;
  Params P;
  P.a_rows_pad = a_rows_pad;
  P.b_rows_pad = b_rows_pad;
  P.nkb = (int)(k_pad / KE);
  P.m = m;
  P.n = n;
  P.alpha = alpha;
  P.beta = beta;
  P.C = C;
  P.ldc = ldc;
  P.err = err;
  P.tiles_m = (int)((m + BM - 1) / BM);
  P.tiles_n = (int)((n + BN - 1) / BN);
  const int64_t tiles = (int64_t)P.tiles_m * P.tiles_n;
  const int ctas = tiles < d->sms ? (int)tiles : d->sms;
  f32tc_gemm_kernel<false><<<ctas, THREADS, SMEM_BYTES, s>>>(ma, mb, P, GroupArgs{nullptr, nullptr, 0});
  return cudaGetLastError();
}

}  // namespace tmm
