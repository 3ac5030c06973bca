// Ozaki split-precision FP64 GEMM: the emulated-DGEMM path.
//
// Algorithm (published; no counterpart in the reference, which calls
// cublasDgemm per tile, src/Tiled-MM/tiled_mm.cpp:200-217):
//   Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix
//   multiplication by using fast routines of matrix multiplication and its
//   applications", Numer. Algorithms 59 (2012) -- error-free splitting;
//   Mukunoki, Ozaki, Ogita, Imamura, "DGEMM using tensor cores, and its
//   accurate and reproducible versions", ISC 2020; Ootomo, Ozaki, Yokota,
//   "DGEMM on integer matrix multiplication unit", IJHPCA 2024 -- integer
//   slices on tensor cores.
//
//  1. scale (FP64): line r of op(A) (rows) / op(B) (columns) over the tile's k
//     range gets e_r = frexp exponent of its largest magnitude.
//  2. split (FP64, exact): t = x * 2^-e * 16; for p < s: d_p = rint(t),
//     t = (t - d_p) * 32.  |d_p| <= 16, so a digit is exact in int8 and in
//     e4m3.  x = 2^e * sum_p d_p 2^(-4 - 5p) + O(2^(e - 5s - 5)).
//  3. multiply (tensor cores, exact): for each diagonal g = s-1 .. 0 of the
//     slice-pair triangle, sum over pairs (p, g-p) of the integer tile
//     products; partial sums are exact integers (|d_a d_b| <= 256).
//  4. recombine (FP64): acc += 2^(-5 g) * S after each exactness pass;
//     t = acc * 2^(e_i + f_j - 8); C = fma(alpha, t, beta' * C).
// The oracle (oracle/tmm_ozaki_oracle.c) performs the same FP64 operations in
// the same order, so results agree bit for bit.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "tmm_ozaki.h"

namespace tmm {

// ------------------------------------------------------------------ configuration
int ozaki_default_engine() {
  const char* e = getenv("TMM_OZAKI_ENGINE");
  if (e && strcmp(e, "imma") == 0) return OZ_ENGINE_IMMA;
  if (e && strcmp(e, "tcgen05") == 0) return OZ_ENGINE_TCGEN05;
  return OZ_ENGINE_TCGEN05;  // ~10x the IMMA engine's rate on sm_103a
}

size_t ozaki_split_bytes(int64_t rows, int64_t kk, int slices) {
  int64_t rp = oz_round_up(rows > 0 ? rows : 1, OZ_ROW_ALIGN);
  int64_t kp = oz_round_up(kk > 0 ? kk : 1, OZ_K_ALIGN);
  size_t digits = (size_t)slices * (size_t)rp * (size_t)kp;
  digits = (digits + 1023) / 1024 * 1024;
  return digits + (size_t)rp * sizeof(int32_t);
}

OzakiSplit ozaki_split_view(void* base, int64_t rows, int64_t kk, int slices, int engine) {
  OzakiSplit v;
  v.rows = rows;
  v.kk = kk;
  v.rows_pad = oz_round_up(rows > 0 ? rows : 1, OZ_ROW_ALIGN);
  v.k_pad = oz_round_up(kk > 0 ? kk : 1, OZ_K_ALIGN);
  v.slices = slices;
  v.enc = ozaki_encoding(engine);
  v.blocked = engine == OZ_ENGINE_TCGEN05 ? 1 : 0;
  size_t digits = (size_t)slices * (size_t)v.rows_pad * (size_t)v.k_pad;
  digits = (digits + 1023) / 1024 * 1024;
  v.digits = (uint8_t*)base;
  v.exps = (int32_t*)((char*)base + digits);
  return v;
}

namespace {

// ------------------------------------------------------------------ split
__device__ __forceinline__ uint32_t digit_byte(int d, int enc) {
  if (enc == OZ_ENC_INT8) return (uint32_t)(uint8_t)(int8_t)d;
  uint32_t a = (uint32_t)(d < 0 ? -d : d);
  if (a == 0) return 0;
  int e = 31 - __clz(a);                  // floor(log2 a), a <= 16
  uint32_t mant = ((a << 3) >> e) & 7u;   // 3 fraction bits (exact for a <= 16)
  return (d < 0 ? 0x80u : 0u) | ((uint32_t)(e + 7) << 3) | mant;
}

constexpr int SP_LINES = 32, SP_L = 64, SP_THREADS = 256;
constexpr int SP_KCHUNK = 512;        // k elements per digit block (at most; a multiple of SP_L)
constexpr int MX_LINES = 256, MX_KCHUNK = 256;  // k chunk of a block: at most MX_KCHUNK
constexpr int EXP_NONE = (int)0x80808080;  // "no nonzero element yet" (byte pattern of the clearing memset)

// frexp exponent of |x| from its IEEE bits (x != 0): 2^(e-1) <= |x| < 2^e
__device__ __forceinline__ int frexp_exponent_bits(uint64_t bits) {
  const int eb = (int)((bits >> 52) & 0x7FF);
  if (eb) return eb - 1022;
  return -1010 - __clzll(bits & 0xFFFFFFFFFFFFFull);  // subnormal: -1074 + bit length
}

// Pass 1: line exponents.  Each thread folds the largest frexp exponent of its
// line segment into exps[line] with one atomicMax (exps cleared to EXP_NONE).
template <int TRANS>
__global__ void __launch_bounds__(SP_THREADS)
oz_linemax_kernel(const double* __restrict__ X, int64_t ld, int64_t rows, int64_t kk, int32_t* __restrict__ exps,
                  int kchunk) {
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = k0 + kchunk < kk ? k0 + kchunk : kk;
  if (TRANS == 0) {  // lines are contiguous across r: one line per thread, coalesced across the warp
    const int64_t r = (int64_t)blockIdx.x * MX_LINES + threadIdx.x;
    if (r >= rows) return;
    uint64_t mx = 0;
#pragma unroll 8
    for (int64_t l = k0; l < k1; ++l) {
      const uint64_t b = (uint64_t)__double_as_longlong(X[r + l * ld]) & 0x7FFFFFFFFFFFFFFFull;
      mx = b > mx ? b : mx;
    }
    if (mx) atomicMax(&exps[r], frexp_exponent_bits(mx));
  } else {  // line r is contiguous along l: a warp per line segment
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll 4
    for (int64_t r = (int64_t)blockIdx.x * MX_LINES + w; r < (int64_t)(blockIdx.x + 1) * MX_LINES && r < rows; r += 8) {
      uint64_t mx = 0;
      for (int64_t l = k0 + lane; l < k1; l += 32) {
        const uint64_t b = (uint64_t)__double_as_longlong(X[l + r * ld]) & 0x7FFFFFFFFFFFFFFFull;
        mx = b > mx ? b : mx;
      }
      for (int o = 16; o > 0; o >>= 1) {
        const uint64_t v = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = v > mx ? v : mx;
      }
      if (lane == 0 && mx) atomicMax(&exps[r], frexp_exponent_bits(mx));
    }
  }
}

// One element's digits, exactly as the FP64 recurrence t = x 2^-e 16; d = rint(t);
// t = (t - d) 32 computes them (every step of which is exact), emulated on the
// integer pipes: x = m 2^E (53-bit m), t = r / 2^f with f = e - 4 - E fractional
// bits, rint = round half to even on the integer r.
struct DigitState {
  int64_t r;
  int f;
  bool neg;
  __device__ __forceinline__ void init(double x, int e) {
    const uint64_t bits = (uint64_t)__double_as_longlong(x);
    neg = (bits >> 63) != 0;
    const int eb = (int)((bits >> 52) & 0x7FF);
    const uint64_t mant = bits & 0xFFFFFFFFFFFFFull;
    r = (int64_t)(eb ? (mant | (1ull << 52)) : mant);
    f = e - 4 - (eb ? eb - 1075 : -1074);
  }
  __device__ __forceinline__ int next() {
    int64_t d;
    if (f >= 63) {
      d = 0;  // |t| < 2^53 / 2^63: rounds to 0, the remainder is unchanged
    } else if (f > 0) {
      const int64_t q = r >> f;  // floor
      const int64_t frac = r - (q << f);
      const int64_t half = (int64_t)1 << (f - 1);
      d = q + ((frac > half || (frac == half && (q & 1))) ? 1 : 0);
      r -= d << f;
    } else {
      d = r << (-f);  // t is an integer already
      r = 0;
    }
    f -= OZ_DIGIT_BITS;
    return neg ? -(int)d : (int)d;
  }
};

// Pass 2: digits of 32 lines x kchunk (<= SP_KCHUNK) k per block, staged through shared
// memory so both the FP64 reads and the byte writes are coalesced.
template <int TRANS>
__global__ void __launch_bounds__(SP_THREADS)
oz_digits_kernel(const double* __restrict__ X, int64_t ld, int64_t rows, int64_t kk, uint8_t* __restrict__ digits,
                 int32_t* __restrict__ exps, int64_t rows_pad, int64_t k_pad, int s, int enc, int blocked,
                 int kchunk) {
  __shared__ double tile[SP_LINES][SP_L + 1];
  __shared__ int sexp[SP_LINES];
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * SP_LINES;
  if (tid < SP_LINES) {
    int e = exps[r0 + tid];
    if (e == EXP_NONE) e = 0;  // all-zero (or padding) line
    sexp[tid] = e;
  }
  __syncthreads();
  if (blockIdx.y == 0 && tid < SP_LINES) exps[r0 + tid] = sexp[tid];
  const size_t plane = (size_t)rows_pad * (size_t)k_pad;
  const int64_t kbeg = (int64_t)blockIdx.y * kchunk;
  const int64_t kend = kbeg + kchunk < k_pad ? kbeg + kchunk : k_pad;
  for (int64_t l0 = kbeg; l0 < kend; l0 += SP_L) {
    if (TRANS == 0) {
      const int r = tid & 31, cg = tid >> 5;
      for (int c = cg; c < SP_L; c += 8) {
        const int64_t l = l0 + c;
        tile[r][c] = (r0 + r < rows && l < kk) ? X[(r0 + r) + l * ld] : 0.0;
      }
    } else {
      const int c = tid & 63, rq = tid >> 6;
      for (int r = rq; r < SP_LINES; r += 4) {
        const int64_t l = l0 + c;
        tile[r][c] = (r0 + r < rows && l < kk) ? X[l + (r0 + r) * ld] : 0.0;
      }
    }
    __syncthreads();
    {
      const int r = tid >> 3, c8 = (tid & 7) * 8;
      const int e = sexp[r];
      DigitState st[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) st[q].init(tile[r][c8 + q], e);
      // 8 consecutive digits of one line never straddle a 128-byte block row
      uint8_t* dst = digits + oz_digit_offset(r0 + r, l0 + c8, k_pad, blocked);
      for (int p = 0; p < s; ++p) {
        uint32_t lo = 0, hi = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint32_t b = digit_byte(st[q].next(), enc);
          if (q < 4) lo |= b << (8 * q);
          else hi |= b << (8 * (q - 4));
        }
        *reinterpret_cast<uint2*>(dst + (size_t)p * plane) = make_uint2(lo, hi);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ IMMA engine
// Exact int8 x int8 -> int32 tile products with mma.sync m16n8k32 (the
// legacy integer tensor path).  CTA tile 128 x 128, 8 warps of 64 x 32,
// k-blocks of 64 bytes in a 2-stage cp.async pipeline; the FP64 accumulators
// live in shared memory (each thread owns its positions) and are updated
// once per exactness pass.
constexpr int IM_BM = 128, IM_BN = 128, IM_KB = 64, IM_THREADS = 256;
constexpr int IM_STRIDE = IM_KB + 16;  // bytes; conflict-free fragment loads
constexpr int IM_STAGE = (IM_BM + IM_BN) * IM_STRIDE;
constexpr size_t IM_SMEM = 2 * IM_STAGE + (size_t)IM_BM * IM_BN * sizeof(double);
constexpr int64_t IM_PASS_BLOCKS = 65536;  // 65536 * 64 terms * 256 < 2^31

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void imma_16x8x32(int (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct IterState {
  int g, p, kb;
};

__global__ void __launch_bounds__(IM_THREADS, 1)
oz_gemm_imma(const uint8_t* __restrict__ Ad, const int32_t* __restrict__ ea, int64_t a_rows_pad,
             const uint8_t* __restrict__ Bd, const int32_t* __restrict__ eb, int64_t b_rows_pad, int64_t k_pad,
             int s, int64_t m, int64_t n, double alpha, double beta, int first, double* __restrict__ C,
             int64_t ldc, int64_t pass_blocks) {
  extern __shared__ __align__(16) uint8_t smem[];
  double* facc = reinterpret_cast<double*>(smem + 2 * IM_STAGE);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g8 = lane >> 2, t4 = lane & 3;
  const int wm = (warp & 1) * 64, wn = (warp >> 1) * 32;
  const int64_t i0 = (int64_t)blockIdx.x * IM_BM, j0 = (int64_t)blockIdx.y * IM_BN;
  const int64_t nkb = k_pad / IM_KB;
  const size_t plane_a = (size_t)a_rows_pad * (size_t)k_pad, plane_b = (size_t)b_rows_pad * (size_t)k_pad;

  // fragment-owned FP64 accumulator positions: (mi, ni, c) -> row, col in the CTA tile
  for (int q = tid; q < IM_BM * IM_BN; q += IM_THREADS) facc[q] = 0.0;

  int acc[4][4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0;

  auto load_stage = [&](int stage, const IterState& it) {
    uint8_t* sa = smem + stage * IM_STAGE;
    uint8_t* sb = sa + IM_BM * IM_STRIDE;
    const uint8_t* ga = Ad + (size_t)it.p * plane_a + (size_t)i0 * (size_t)k_pad + (size_t)it.kb * IM_KB;
    const uint8_t* gb = Bd + (size_t)(it.g - it.p) * plane_b + (size_t)j0 * (size_t)k_pad + (size_t)it.kb * IM_KB;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      int chunk = tid + q * IM_THREADS;  // 512 chunks of 16 bytes per operand
      int row = chunk >> 2, col = (chunk & 3) * 16;
      cp_async16(sa + row * IM_STRIDE + col, ga + (size_t)row * (size_t)k_pad + col);
      cp_async16(sb + row * IM_STRIDE + col, gb + (size_t)row * (size_t)k_pad + col);
    }
  };
  auto advance = [&](IterState& it) {
    if (++it.kb == nkb) {
      it.kb = 0;
      if (++it.p > it.g) {
        it.p = 0;
        --it.g;
      }
    }
  };

  IterState cur{s - 1, 0, 0};
  IterState nxt = cur;
  advance(nxt);
  load_stage(0, cur);
  cp_async_commit();
  int64_t used = 0;
  int stage = 0;
  while (cur.g >= 0) {
    if (nxt.g >= 0) load_stage(stage ^ 1, nxt);
    cp_async_commit();
    cp_async_wait1();
    __syncthreads();
    const uint8_t* sa = smem + stage * IM_STAGE;
    const uint8_t* sb = sa + IM_BM * IM_STRIDE;
#pragma unroll
    for (int ks = 0; ks < IM_KB; ks += 32) {
      uint32_t af[4][4], bf[4][2];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const uint8_t* base = sa + (wm + a * 16 + g8) * IM_STRIDE + ks + 4 * t4;
        af[a][0] = *reinterpret_cast<const uint32_t*>(base);
        af[a][1] = *reinterpret_cast<const uint32_t*>(base + 8 * IM_STRIDE);
        af[a][2] = *reinterpret_cast<const uint32_t*>(base + 16);
        af[a][3] = *reinterpret_cast<const uint32_t*>(base + 8 * IM_STRIDE + 16);
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const uint8_t* base = sb + (wn + b * 8 + g8) * IM_STRIDE + ks + 4 * t4;
        bf[b][0] = *reinterpret_cast<const uint32_t*>(base);
        bf[b][1] = *reinterpret_cast<const uint32_t*>(base + 16);
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) imma_16x8x32(acc[a][b], af[a], bf[b]);
    }
    __syncthreads();
    // pass boundary: at the block cap or at the end of the diagonal
    ++used;
    const bool group_end = (cur.kb == nkb - 1) && (cur.p == cur.g);
    if (used == pass_blocks || group_end) {
      const double wg = scalbn(1.0, -OZ_DIGIT_BITS * cur.g);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            int row = wm + a * 16 + g8 + ((c >> 1) << 3), col = wn + b * 8 + 2 * t4 + (c & 1);
            double* f = facc + row * IM_BN + col;
            *f = *f + wg * (double)acc[a][b][c];
            acc[a][b][c] = 0;
          }
      used = 0;
    }
    cur = nxt;
    advance(nxt);
    stage ^= 1;
  }
  cp_async_wait0();
  // fused epilogue
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        int row = wm + a * 16 + g8 + ((c >> 1) << 3), col = wn + b * 8 + 2 * t4 + (c & 1);
        int64_t gi = i0 + row, gj = j0 + col;
        if (gi < m && gj < n) {
          double t = scalbn(facc[row * IM_BN + col], ea[gi] + eb[gj] - 2 * (OZ_DIGIT_BITS - 1));
          double* cp = C + gi + gj * ldc;
          if (ea[gi] >= OZ_EXP_NONFINITE || eb[gj] >= OZ_EXP_NONFINITE) *cp = __longlong_as_double(0x7FF8000000000000ll);
          else if (!first) *cp = fma(alpha, t, *cp);
          else if (beta != 0.0) *cp = fma(alpha, t, beta * *cp);
          else *cp = alpha * t;
        }
      }
}

}  // namespace

int64_t ozaki_pass_blocks(int engine) { return engine == OZ_ENGINE_TCGEN05 ? ozaki_tc_pass_blocks() : IM_PASS_BLOCKS; }
int64_t ozaki_k_block(int engine) { return engine == OZ_ENGINE_TCGEN05 ? ozaki_tc_k_block() : IM_KB; }
size_t ozaki_workspace_bytes(int engine) { return engine == OZ_ENGINE_TCGEN05 ? ozaki_tc_workspace_bytes() : 0; }
size_t ozaki_workspace_bytes_for(int engine, int64_t m, int64_t n) {
  return engine == OZ_ENGINE_TCGEN05 ? ozaki_tc_workspace_bytes_for(m, n) : 0;
}
cudaError_t ozaki_prepare(int engine) { return engine == OZ_ENGINE_TCGEN05 ? ozaki_tc_prepare() : cudaSuccess; }

namespace {
int split_sms() {
  static int sms = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  });
  return sms;
}
}  // namespace

cudaError_t ozaki_split(const double* X, int64_t ld, Op trans, int64_t rows, int64_t kk, const OzakiSplit& out,
                        cudaStream_t s) {
  if (out.slices < 1 || out.slices > OZ_MAX_SLICES) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(out.exps, 0x80, (size_t)out.rows_pad * sizeof(int32_t), s);  // EXP_NONE
  if (e != cudaSuccess) return e;
  // k chunks shrink (down to 32 / 64 elements) until the grid has about four blocks per SM:
  // small operands are otherwise split by a few blocks that each walk a long k range
  const int64_t want = 4 * (int64_t)split_sms();
  if (rows > 0 && kk > 0) {
    const int64_t gx = (rows + MX_LINES - 1) / MX_LINES;
    int kc = MX_KCHUNK;
    while (kc > 32 && gx * ((kk + kc - 1) / kc) < want) kc /= 2;
    dim3 gm((unsigned)gx, (unsigned)((kk + kc - 1) / kc));
    if (trans == OP_N) oz_linemax_kernel<0><<<gm, SP_THREADS, 0, s>>>(X, ld, rows, kk, out.exps, kc);
    else oz_linemax_kernel<1><<<gm, SP_THREADS, 0, s>>>(X, ld, rows, kk, out.exps, kc);
  }
  const int64_t dx = out.rows_pad / SP_LINES;
  int dc = SP_KCHUNK;
  while (dc > SP_L && dx * ((out.k_pad + dc - 1) / dc) < want) dc /= 2;
  dim3 gd((unsigned)dx, (unsigned)((out.k_pad + dc - 1) / dc));
  if (trans == OP_N)
    oz_digits_kernel<0><<<gd, SP_THREADS, 0, s>>>(X, ld, rows, kk, out.digits, out.exps, out.rows_pad, out.k_pad,
                                                  out.slices, out.enc, out.blocked, dc);
  else
    oz_digits_kernel<1><<<gd, SP_THREADS, 0, s>>>(X, ld, rows, kk, out.digits, out.exps, out.rows_pad, out.k_pad,
                                                  out.slices, out.enc, out.blocked, dc);
  return cudaGetLastError();
}

cudaError_t ozaki_gemm(const OzakiSplit& A, const OzakiSplit& B, int64_t m, int64_t n, double alpha, double beta,
                       bool first_k_tile, double* C, int64_t ldc, int engine, double* work, int* err, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  if (engine == OZ_ENGINE_TCGEN05) return ozaki_gemm_tc(A, B, m, n, alpha, beta, first_k_tile, C, ldc, work, err, s);
  if (A.enc != OZ_ENC_INT8 || B.enc != OZ_ENC_INT8) return cudaErrorInvalidValue;
  if (A.k_pad != B.k_pad || A.slices != B.slices || A.rows_pad < m || B.rows_pad < n) return cudaErrorInvalidValue;
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(oz_gemm_imma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)IM_SMEM);
  });
  if (attr_err != cudaSuccess) return attr_err;
  dim3 grid((unsigned)((m + IM_BM - 1) / IM_BM), (unsigned)((n + IM_BN - 1) / IM_BN));
  oz_gemm_imma<<<grid, IM_THREADS, IM_SMEM, s>>>(A.digits, A.exps, A.rows_pad, B.digits, B.exps, B.rows_pad, A.k_pad,
                                                 A.slices, m, n, alpha, beta, first_k_tile ? 1 : 0, C, ldc,
                                                 IM_PASS_BLOCKS);
  return cudaGetLastError();
}

}  // namespace tmm
