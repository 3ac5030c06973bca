// tcgen05 engine of the Ozaki path: exact e4m3 digit-plane products on the
// 5th-generation tensor cores of sm_103a, FP64 recombination, fused epilogue.
//
// Per CTA (persistent, one per SM) output tiles of 128 x 256:
//   warp 0      TMA producer: 128 x 128-byte A and 256 x 128-byte B digit
//               tiles (SWIZZLE_128B) into a 4-stage shared-memory ring
//               (full/empty mbarriers, expect_tx byte counts);
//   warp 1      allocates 512 TMEM columns and, from one thread, issues
//               tcgen05.mma.cta_group::1.kind::f8f6f4 (M=128, N=256, K=32)
//               into one of two 256-column FP32 accumulators, committing
//               stage releases and "accumulator full" to mbarriers;
//   warps 2-5   drain a full accumulator with tcgen05.ld (one TMEM lane per
//               thread), release it, and add 2^(-5 g) * S to the tile's FP64
//               accumulator in a per-CTA workspace slot (L2-resident, each
//               thread owns its elements); after the tile's last pass they
//               apply 2^(e_i + f_j - 8), alpha and beta and store C.
// The sequence of (diagonal g, slice pair p, k-block) and the exactness
// passes (at most OZ_TC_PASS_BLOCKS k-blocks of 128: 65536 products of
// |d_a d_b| <= 256 stay below 2^24, exact in FP32) is the one the oracle
// (oracle/tmm_ozaki_oracle.c) replays.  Every mbarrier wait is bounded: after
// about a second it records an error word and the CTA winds down (waiting,
// again bounded, for its copies and MMAs in flight) and frees its TMEM.
//
// A second form (oz_gemm_tc_pair, selected with TMM_TC_CLUSTER=pair) runs the
// same sequence on CTA pairs with tcgen05.mma.cta_group::2 on 256 x 256 tiles.
// Neither form multicasts a copy: each CTA's TMA loads land in its own shared
// memory only.
// Digit planes are read in the blocked layout (tmm_ozaki.h): every box a stage
// loads is one contiguous 16 KB block.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "tmm_ozaki.h"
#include "tmm_tc_ptx.cuh"

namespace tmm {
namespace tc {

constexpr int BM = 128, BN = 256, KB = 128;  // KB: bytes (= e4m3 elements) per k-block
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * KB, B_BYTES = BN * KB, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int THREADS = 192;
constexpr int TMEM_COLS = 512;
constexpr int64_t PASS_BLOCKS = 512;  // 512 * 128 = 65536 k terms per exact FP32 pass
constexpr size_t SMEM_BYTES = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
constexpr size_t WORK_HEADER = 256;  // bytes before the accumulator slots: the pacing counter
// the epilogue waits a whole pass (tens of microseconds) for an accumulator: park, don't spin
constexpr uint32_t EPI_WAIT_HINT_NS = 20000;

// ------------------------------------------------------------------ f8 MMA forms
// kind::f8f6f4: D f32, A e4m3, B e4m3, both K-major, N = 256, M = 128
constexpr uint32_t IDESC = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

// kind::f8f6f4 across the pair: M = 256 (128 TMEM lanes in each CTA), N = 256
constexpr uint32_t IDESC_PAIR = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);

// One k-block (K = 128 = four MMAs of K = 32) with the stage release and a probe of the next
// stage's full barrier in one block of PTX: the probe is a non-blocking test_wait issued after
// the first MMA and its result is read after the commit, so the issuing thread never waits on
// a result between two MMAs.  (Measured on a CTA pair with the engine's stage handshake and no
// copies: 512 cycles per k-block, the pipe's rate; 554-630 with a try_wait probe read between
// the third and fourth MMA, 595-698 with a wait after the commit.)  Returns the probe.
__device__ __forceinline__ uint32_t kblock_f8(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t accumulate,
                                              uint32_t probe_bar, uint32_t probe_parity, uint32_t empty_bar) {
  uint32_t ready;
  asm volatile(
      "{\n .reg .pred pa, pr;\n"
      " setp.ne.b32 pa, %5, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%1], %2, %3, %4, pa;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 pr, [%6], %7;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%1], %8, %9, %4, 1;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%1], %10, %11, %4, 1;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%1], %12, %13, %4, 1;\n"
      " tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%14];\n"
      " selp.u32 %0, 1, 0, pr;\n}\n"
      : "=r"(ready)
      : "r"(d_tmem), "l"(ad), "l"(bd), "r"(IDESC), "r"(accumulate), "r"(probe_bar), "r"(probe_parity), "l"(ad + 2),
        "l"(bd + 2), "l"(ad + 4), "l"(bd + 4), "l"(ad + 6), "l"(bd + 6), "r"(empty_bar)
      : "memory");
  return ready;
}
// the same on a CTA pair: cta_group::2 MMAs, the release multicast to both CTAs' barriers
__device__ __forceinline__ uint32_t kblock_f8_pair(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t accumulate,
                                                   uint32_t probe_bar, uint32_t probe_parity, uint32_t empty_bar) {
  uint32_t ready;
  asm volatile(
      "{\n .reg .pred pa, pr;\n"
      " setp.ne.b32 pa, %5, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f8f6f4 [%1], %2, %3, %4, pa;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 pr, [%6], %7;\n"
      " tcgen05.mma.cta_group::2.kind::f8f6f4 [%1], %8, %9, %4, 1;\n"
      " tcgen05.mma.cta_group::2.kind::f8f6f4 [%1], %10, %11, %4, 1;\n"
      " tcgen05.mma.cta_group::2.kind::f8f6f4 [%1], %12, %13, %4, 1;\n"
      " tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%14], %15;\n"
      " selp.u32 %0, 1, 0, pr;\n}\n"
      : "=r"(ready)
      : "r"(d_tmem), "l"(ad), "l"(bd), "r"(IDESC_PAIR), "r"(accumulate), "r"(probe_bar), "r"(probe_parity),
        "l"(ad + 2), "l"(bd + 2), "l"(ad + 4), "l"(bd + 4), "l"(ad + 6), "l"(bd + 6), "r"(empty_bar), "h"((uint16_t)3)
      : "memory");
  return ready;
}

// ------------------------------------------------------------------ work sequence
// Per tile: for g = s-1 .. 0, p = 0 .. g (q = g - p), kb = 0 .. nkb-1; a pass ends
// after PASS_BLOCKS k-blocks or at the end of a diagonal.
struct Seq {
  int s, nkb;
  int g, p, kb;
  int used;  // k-blocks of the current pass before this one (< PASS_BLOCKS)
  __device__ void start(int s_, int nkb_) {
    s = s_;
    nkb = nkb_;
    g = s - 1;
    p = 0;
    kb = 0;
    used = 0;
  }
  __device__ bool done() const { return g < 0; }
  __device__ bool pass_first() const { return used == 0; }
  // true when the current k-block closes a pass
  __device__ bool pass_last() const { return used + 1 == PASS_BLOCKS || (kb == nkb - 1 && p == g); }
  // true on the tile's last k-block (diagonal 0 comes last)
  __device__ bool tile_last() const { return g == 0 && kb == nkb - 1; }
  __device__ void next() {
    used = pass_last() ? 0 : used + 1;
    if (++kb == nkb) {
      kb = 0;
      if (++p > g) {
        p = 0;
        --g;
      }
    }
  }
};

// The MMA issuer's walk of the same sequence.  It needs only where passes begin and end,
// not (g, p, kb), so it counts k-blocks down: between two MMAs of the pipe's short queue
// the issuing thread runs two decrements and a compare instead of the sequence's nested
// counters (measured with the loads and drains switched off in a scratch build: 658-670
// cycles per k-block of 4 MMAs with the nested counters, against 512 back to back).
// Tiles ct, ct + stride, ...; nkb_of(ct) gives tile ct's k-blocks, read one tile ahead so
// that a lookup in global memory (grouped launches) is not waited on at the tile change.
struct PassCounter {
  int ct, g, diag_left, pass_left, nkb, nkb_next;
  bool valid;
  template <typename NkbOf>
  __device__ void start(int ct0, int stride, int total, int s, NkbOf nkb_of) {
    ct = ct0;
    valid = ct < total;
    nkb = valid ? nkb_of(ct) : 1;
    nkb_next = ct + stride < total ? nkb_of(ct + stride) : 1;
    g = s - 1;
    diag_left = s * nkb;
    pass_left = diag_left < (int)PASS_BLOCKS ? diag_left : (int)PASS_BLOCKS;
  }
  // the current k-block closes a pass
  __device__ bool last() const { return pass_left == 1; }
  // step to the next k-block; true when it begins a pass (of the next diagonal or tile)
  template <typename NkbOf>
  __device__ bool next(int stride, int total, int s, NkbOf nkb_of) {
    --diag_left;
    if (--pass_left != 0) return false;
    if (diag_left == 0) {
      if (--g < 0) {
        ct += stride;
        valid = ct < total;
        g = s - 1;
        nkb = nkb_next;
        nkb_next = valid && ct + stride < total ? nkb_of(ct + stride) : 1;
      }
      diag_left = (g + 1) * nkb;
    }
    pass_left = diag_left < (int)PASS_BLOCKS ? diag_left : (int)PASS_BLOCKS;
    return true;
  }
};

// Tile order: bands of GROUP_M tile rows, n-tiles fastest inside a band, so the
// ~150 co-resident CTAs cover about 16 x 9 tiles and share their A and B panels
// in L2 (an m-fastest order has them cover 64 A panels per wave at 8192^2).
constexpr int GROUP_M = 16;
__device__ __forceinline__ void tile_coords(int tile, int tiles_m, int tiles_n, int group, int* tm, int* tn) {
  const int per_band = group * tiles_n;
  const int band = tile / per_band, local = tile - band * per_band;
  const int rows_in_band = min(group, tiles_m - band * group);
  *tm = band * group + local % rows_in_band;
  *tn = local / rows_in_band;
}

// Digit planes are in the blocked layout ([s][rows/128][k/128][128][128] bytes); the
// tensor maps view them as rows of 128 bytes.  Row coordinate of the box that starts
// at line `line` (a multiple of the box height, which divides 128) of slice p, k-block kb:
__device__ __forceinline__ int box_y(int p, int64_t line, int kb, int64_t rows_pad, int nkb) {
  return (int)((((int64_t)p * (rows_pad / OZ_BLOCK) + line / OZ_BLOCK) * nkb + kb) * OZ_BLOCK + line % OZ_BLOCK);
}

struct Params {
  const int32_t* ea;
  const int32_t* eb;
  int64_t a_rows_pad, b_rows_pad;
  int nkb, s;
  int64_t m, n;
  double alpha, beta;
  int first;
  double* C;
  int64_t ldc;
  double* work;  // gridDim.x slots of BM * BN doubles
  int* err;
  int tiles_m, tiles_n;
  int pf;  // k-blocks the producer prefetches into L2 ahead of its loads (0: none)
  uint32_t epi_hint;  // nanoseconds an epilogue warp may park per probe of a full accumulator
  int group_m;        // tile rows (of 128) per band of the tile order
  // Wave pacing: the producers publish their progress (one count per chunk of pace_chunk
  // k-blocks) to *pace, and one that is more than pace_lag chunks ahead of the average CTA
  // waits (at most pace_ns per chunk, then goes on: a hint, never an error), so that the
  // co-resident CTAs stay at about the same (diagonal, pair, k-block) position of their
  // tiles and the A and B blocks that a step shares are read from DRAM once.
  unsigned long long* pace;
  int pace_lag;  // 0: off
  int pace_chunk;  // a power of two
  uint32_t pace_ns;
};

__device__ __forceinline__ void red_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Called by a producer at the start of its chunk c (k-blocks counted over all its tiles; every
// tile has the same sequence, so equal counts are equal positions).  seen caches the last value
// read: when it already allows chunk c, a fresh read is issued for the next call and not waited on.
__device__ __forceinline__ void pace_gate(const Params& P, unsigned long long c, unsigned long long ctas,
                                          unsigned long long& seen) {
  if (c > 0) red_add_u64(P.pace, 1ull);  // chunk c - 1 issued
  if (c <= (unsigned long long)P.pace_lag) return;
  const unsigned long long need = (c - (unsigned long long)P.pace_lag) * ctas;
  if (seen >= need) {
    seen = ld_relaxed_u64(P.pace);
    return;
  }
  const uint64_t t0 = globaltimer();
  while (true) {
    seen = ld_relaxed_u64(P.pace);
    if (seen >= need || globaltimer() - t0 > P.pace_ns) return;
    __nanosleep(256);
  }
}
// a producer that has issued all its work lifts its weight off the others' gates
constexpr unsigned long long PACE_DONE = 1ull << 40;

// What the epilogue of a tile needs: its problem's exponents, sizes, scalars and C.
struct Epi {
  const int32_t* ea;
  const int32_t* eb;
  int64_t m, n;
  double alpha, beta;
  int first;
  double* C;
  int64_t ldc;
};
__device__ __forceinline__ Epi epi_of(const Params& P) {
  return Epi{P.ea, P.eb, P.m, P.n, P.alpha, P.beta, P.first, P.C, P.ldc};
}

// A problem of a grouped launch (ozaki_gemm_tc_grouped): its digit planes start at row
// a_row0 / b_row0 of the launch's tensor maps (one map over all problems' A planes, one
// over all B planes, in 128-byte rows).
struct GroupProblem {
  int64_t a_row0, b_row0, a_rows_pad, b_rows_pad;
  const int32_t* ea;
  const int32_t* eb;
  double* C;
  int64_t ldc, m, n;
  double alpha, beta;
  int nkb, first;
};
struct GroupArgs {
  const GroupProblem* probs;
  const int4* items;  // (problem, 128-row tile index, 256-column tile index, unused)
  int n_items;
};

// FP64 arithmetic issues at about two operations per clock and SM on this GPU, so the
// exact steps of the drain run on the integer pipes:
// the pass sum S is an integer-valued FP32 (|S| < 2^24, exact by the pass limit), and
// 2^-sh * S as a double is its sign and mantissa with the exponent rebased: no rounding.
// (-0 becomes +0, which is what 0.0 + 2^-sh * S gives.)
__device__ __forceinline__ double scaled_pass_sum(uint32_t fb, int sh) {
  if ((fb & 0x7FFFFFFFu) == 0) return 0.0;
  const uint32_t e = ((fb >> 23) & 0xFFu) + (1023 - 127) - (uint32_t)sh;  // >= 1023 - 50: normal
  const uint32_t hi = (fb & 0x80000000u) | (e << 20) | ((fb & 0x7FFFFFu) >> 3);
  return __hiloint2double((int)hi, (int)(fb << 29));
}
// scalbn(x, n), exactly: the exponent field is rebased when x and the result are normal;
// zeros, subnormals, overflow and non-finite values take scalbn itself
__device__ __forceinline__ double scalbn_fast(double x, int n) {
  const int hi = __double2hiint(x);
  const int e = (hi >> 20) & 0x7FF;
  if (e == 0 || e == 0x7FF || e + n < 1 || e + n > 0x7FE) return scalbn(x, n);
  return __hiloint2double((int)((unsigned)hi + ((unsigned)n << 20)), __double2loint(x));
}

// Drain of one pass by one epilogue thread (tile row `row`, global row gi, first column
// col0): acc = (first pass ? 0 : slot) + 2^(-5g) * S for the 256 columns, read from TMEM
// in chunks of 32; release() hands the accumulator back once its last chunk is in
// registers.  The slot values of a chunk are loaded while its TMEM load is in flight.  On
// the tile's last pass the sums go straight into the fused epilogue
// C = alpha * 2^(e_i + f_j - 8) * acc + beta' * C (beta' = beta on the first k tile, C not
// read when it is zero) instead of back to the slot; the loads of a chunk's exponents and
// C values are issued together.  One FP64 add per element and pass (none on the first).
template <typename Release>
__device__ __forceinline__ void drain_pass(uint32_t tbase, double* __restrict__ slot, int row, int g, bool first_pass,
                                           bool last, const Epi& P, int64_t gi, int64_t col0, Release release) {
  const int sh = OZ_DIGIT_BITS * g;
  const bool row_ok = gi < P.m;
  const int ei = last && row_ok ? P.ea[gi] : 0;
#pragma unroll 1
  for (int c = 0; c < BN / 32; ++c) {
    uint32_t r[32];
    double acc[32];
    tmem_ld32(tbase + (uint32_t)(c * 32), r);
    if (!first_pass) {
#pragma unroll
      for (int j = 0; j < 32; ++j) acc[j] = slot[(size_t)(c * 32 + j) * BM + row];
    }
    tmem_ld_wait(r);
    if (c == BN / 32 - 1) release();
    if (first_pass) {
#pragma unroll
      for (int j = 0; j < 32; ++j) acc[j] = scaled_pass_sum(r[j], sh);
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) acc[j] += scaled_pass_sum(r[j], sh);
    }
    if (!last) {
#pragma unroll
      for (int j = 0; j < 32; ++j) slot[(size_t)(c * 32 + j) * BM + row] = acc[j];
      continue;
    }
    const int64_t gj0 = col0 + c * 32;
    if (!row_ok || gj0 >= P.n) continue;
    const int nv = P.n - gj0 < 32 ? (int)(P.n - gj0) : 32;
    const bool read_c = !P.first || P.beta != 0.0;
    const bool plain = P.first && P.beta == 0.0 && P.alpha == 1.0;  // C = 2^(e_i + f_j - 8) * acc
    double* cp = P.C + gi + gj0 * P.ldc;
#pragma unroll
    for (int h = 0; h < 32; h += 16) {
      int fj[16];
      double cv[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        fj[j] = h + j < nv ? P.eb[gj0 + h + j] : 0;
        cv[j] = read_c && h + j < nv ? cp[(int64_t)(h + j) * P.ldc] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        if (h + j >= nv) break;
        const double t = scalbn_fast(acc[h + j], ei + fj[j] - 2 * (OZ_DIGIT_BITS - 1));
        double out;
        if (ei >= OZ_EXP_NONFINITE || fj[j] >= OZ_EXP_NONFINITE) out = __longlong_as_double(0x7FF8000000000000ll);
        else if (plain) out = t;
        else if (!P.first) out = fma(P.alpha, t, cv[j]);
        else if (P.beta != 0.0) out = fma(P.alpha, t, P.beta * cv[j]);
        else out = P.alpha * t;
        cp[(int64_t)(h + j) * P.ldc] = out;
      }
    }
  }
}

// A tile of a launch: its coordinates, its problem's k-blocks and plane geometry.  A plain
// launch walks the tiles of one product in band order; a grouped launch walks a work list of
// (problem, tile) items of many products whose planes share one tensor map per operand.
struct Job {
  int tm, tn, nkb;
  int64_t a_row0, b_row0, a_rows_pad, b_rows_pad;
};
template <bool GROUPED>
__device__ __forceinline__ Job job_of(int ct, const Params& P, const GroupArgs& G, int group) {
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
  } else {
    tile_coords(ct, P.tiles_m, P.tiles_n, group, &j.tm, &j.tn);
    j.nkb = P.nkb;
    j.a_row0 = j.b_row0 = 0;
    j.a_rows_pad = P.a_rows_pad;
    j.b_rows_pad = P.b_rows_pad;
  }
  return j;
}
template <bool GROUPED>
__device__ __forceinline__ Epi epi_job(int ct, const Params& P, const GroupArgs& G) {
  if (!GROUPED) return epi_of(P);
  const GroupProblem& q = G.probs[G.items[ct].x];
  return Epi{q.ea, q.eb, q.m, q.n, q.alpha, q.beta, q.first, q.C, q.ldc};
}

// One CTA per SM computes its 128 x 256 tiles alone: every TMA copy lands in
// this CTA's own shared memory (no cluster, no multicast), and a stage is
// refilled once this CTA's MMAs have read it.  GROUPED: the tiles are the items of a
// work list over several products (ozaki_gemm_tc_grouped), each with its own k-blocks,
// planes, exponents, scalars and C.
template <bool GROUPED>
__global__ void __launch_bounds__(THREADS, 1)
oz_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const Params P,
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
  const int group = P.group_m > 0 ? P.group_m : 1;
  constexpr int B_BOX = OZ_BLOCK;  // a box stays inside one 128-line block of the blocked layout

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
      unsigned long long issued = 0, seen = 0;  // k-blocks issued in this launch; last pace count read
      const unsigned long long chunk_mask = (unsigned long long)P.pace_chunk - 1;
      for (int ct = blockIdx.x; ct < total_tiles && ok; ct += gridDim.x) {
        const Job J = job_of<GROUPED>(ct, P, G, group);
        const int tm = J.tm;
        // f runs P.pf k-blocks ahead of q: its boxes are prefetched into L2 so that the
        // loads, issued when a stage frees up, find them there instead of in DRAM
        const int64_t b0 = (int64_t)J.tn * BN;
        auto ay = [&](int p_, int kb_) { return (int)(J.a_row0 + box_y(p_, (int64_t)tm * BM, kb_, J.a_rows_pad, J.nkb)); };
        auto by_ = [&](int q_, int64_t line, int kb_) { return (int)(J.b_row0 + box_y(q_, line, kb_, J.b_rows_pad, J.nkb)); };
        auto prefetch = [&](const Seq& f) {
          tma_prefetch_2d(&tmA, 0, ay(f.p, f.kb));
          for (int j = 0; j < BN / B_BOX; ++j) tma_prefetch_2d(&tmB, 0, by_(f.g - f.p, b0 + j * B_BOX, f.kb));
        };
        Seq q, f;
        f.start(P.s, J.nkb);
        for (int i = 0; i < P.pf && !f.done(); ++i, f.next()) prefetch(f);
        for (q.start(P.s, J.nkb); !q.done() && ok; q.next()) {
          if (P.pf > 0 && !f.done()) {
            prefetch(f);
            f.next();
          }
          if (P.pace_lag && (issued & chunk_mask) == 0) pace_gate(P, issued / P.pace_chunk, gridDim.x, seen);
          ++issued;
          ok = mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, P.err);
          if (!ok) break;
          const uint32_t fb = full0 + 8 * stage;
          mbar_expect_tx(fb, STAGE_BYTES);  // A box + the B boxes
          uint8_t* sa = smem + (size_t)stage * STAGE_BYTES;
          tma_load_2d(smem_u32(sa), &tmA, 0, ay(q.p, q.kb), fb);
#pragma unroll
          for (int j = 0; j < BN / B_BOX; ++j)
            tma_load_2d(smem_u32(sa + A_BYTES + j * B_BOX * KB), &tmB, 0, by_(q.g - q.p, b0 + j * B_BOX, q.kb), fb);
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      if (P.pace_lag) red_add_u64(P.pace, PACE_DONE);
      // drain: every issued copy has landed before the CTA may exit (bounded)
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
    // The tensor pipe keeps almost no queue of issued MMAs: every cycle this thread spends
    // between two MMAs is a cycle the pipe idles (a k-block of 4 MMAs takes 512 cycles when
    // they are issued back to back, 700-900 with the bookkeeping and barrier checks in
    // between).  So the next k-block's bookkeeping and a one-shot probe of its full barrier
    // run after the third MMA of the current k-block, while the pipe still has work; the
    // thread blocks on a barrier only when that probe failed or a pass begins.
    if (lane == 0) {
      static_assert(KB / 32 == 4, "four K = 32 MMAs per k-block");
      constexpr uint64_t STAGE_STEP = (uint64_t)(STAGE_BYTES >> 4);  // descriptor address field per stage
      const uint32_t sa0 = smem_u32(smem);
      const uint64_t ad0 = smem_desc(sa0), bd0 = smem_desc(sa0 + A_BYTES);
      auto nkb_of = [&](int ct) { return GROUPED ? G.probs[G.items[ct].x].nkb : P.nkb; };
      PassCounter cur{};
      cur.start(blockIdx.x, gridDim.x, total_tiles, P.s, nkb_of);
      int stage = 0, buf = 0;
      uint32_t phase = 0, tph = 0;  // tph bit b: phase of accumulator b's full barrier
      uint64_t ad = ad0, bd = bd0;
      bool ok = cur.valid;
      bool first = true, last = cur.last();
      if (ok) ok = mbar_wait(tempty0, 1, abort_flag, P.err);  // first pass: buffer 0 is free
      if (ok) ok = mbar_wait(full0, 0, abort_flag, P.err);
      tc_fence_after();
      while (ok) {
        const uint32_t d_tmem = tmem_base + (uint32_t)(buf * BN);
        const int nstage = stage + 1 == STAGES ? 0 : stage + 1;
        const uint32_t nphase = nstage == 0 ? phase ^ 1u : phase;
        // the k-block's MMAs, the stage's release (free when they have read it) and a probe
        // of the next stage (K = 32 e4m3 = 32 bytes per MMA: +2 in the 16-byte address field)
        const uint32_t probe = kblock_f8(d_tmem, ad, bd, first ? 0u : 1u, full0 + 8 * nstage, nphase, empty0 + 8 * stage);
        // ---- next k-block, while the MMAs run
        const bool nfirst = cur.next(gridDim.x, total_tiles, P.s, nkb_of);
        const bool nvalid = cur.valid, nlast = cur.last();
        const uint64_t nad = nstage == 0 ? ad0 : ad + STAGE_STEP, nbd = nstage == 0 ? bd0 : bd + STAGE_STEP;
        const bool ready = nvalid && !nfirst && probe != 0;
        if (last) {
          mma_commit(tfull0 + 8 * buf);
          tph ^= 1u << buf;
          buf ^= 1;
        }
        stage = nstage;
        phase = nphase;
        ad = nad;
        bd = nbd;
        first = nfirst;
        last = nlast;
        if (ready) {  // fast path: the next stage is loaded and no pass begins
          tc_fence_after();
          continue;
        }
        if (!nvalid) break;
        if (first) {
          ok = mbar_wait(tempty0 + 8 * buf, ((tph >> buf) & 1u) ^ 1u, abort_flag, P.err);
          if (!ok) break;
        }
        ok = mbar_wait(full0 + 8 * stage, phase, abort_flag, P.err);
        if (!ok) break;
        tc_fence_after();
      }
      // wait (bounded) for the MMAs in flight before TMEM is freed
      for (int b = 0; b < 2; ++b) {
        (void)mbar_wait(tempty0 + 8 * buf, ((tph >> buf) & 1u) ^ 1u, abort_flag, P.err);
        buf ^= 1;
      }
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2..5)
    const int quarter = warp & 3;        // TMEM lanes 32*quarter .. +31 are this warp's
    const int row = quarter * 32 + lane;  // tile row = TMEM lane
    double* slot = P.work + (size_t)blockIdx.x * (size_t)(BM * BN);
    uint32_t tphase[2] = {0, 0};
    int buf = 0;
    bool ok = true;
    for (int ct = blockIdx.x; ct < total_tiles && ok; ct += gridDim.x) {
      const Job J = job_of<GROUPED>(ct, P, G, group);
      const Epi E = epi_job<GROUPED>(ct, P, G);
      const int tm = J.tm, tn = J.tn;
      bool first_pass = true;
      Seq q;
      for (q.start(P.s, J.nkb); !q.done() && ok; q.next()) {
        if (!q.pass_last()) continue;
        // one lane waits, the warp follows: the TMEM loads below are warp-collective
        int okw = 1;
        if (lane == 0) okw = mbar_wait(tfull0 + 8 * buf, tphase[buf], abort_flag, P.err, P.epi_hint) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
        __syncwarp();
        if (!ok) break;
        tc_fence_after();
        const uint32_t tbase = tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * BN);
        const uint32_t tempty = tempty0 + 8 * buf;
        drain_pass(tbase, slot, row, q.g, first_pass, q.tile_last(), E, (int64_t)tm * BM + row, (int64_t)tn * BN,
                   [&] {  // accumulator consumed: hand it back to the MMA warp
                     tc_fence_before();
                     __syncwarp();
                     if (lane == 0) mbar_arrive(tempty);
                   });
        first_pass = false;
        tphase[buf] ^= 1;
        buf ^= 1;
      }
    }
  }
  tc_fence_before();
  __syncwarp();  // lane 0 of warps 0 and 1 ran alone
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// ------------------------------------------------------------------ CTA-pair engine
// The two CTAs of a cluster pair (on the two SMs of a TPC) compute one 256 x 256
// tile with tcgen05.mma.cta_group::2 (M = 256, N = 256, K = 32): CTA r stages rows
// 128 r .. 128 r + 127 of the A tile and of the B tile, so an SM takes in 32 KB per
// k-block for its 128 x 256 half (48 KB for the same half on one SM), and the MMA
// reads the B tile from both SMs.  The even CTA (leader) issues all MMAs; both
// CTAs' copies count their bytes on the leader's full barrier; the leader's commits
// arrive on both CTAs' empty and accumulator-full barriers; both CTAs' epilogue
// warps release an accumulator on the leader's empty-accumulator barrier (8
// arrivals).  Each CTA drains its own 128 TMEM lanes = its 128 tile rows, with the
// pass sequence, FP64 recombination and fused epilogue of oz_gemm_tc.
constexpr int PAIR_M = 256;
constexpr int PAIR_STAGES = 6;  // the default ring; a 7-stage instance fills 227 KB (TMM_TC_PAIR_STAGES=7)
constexpr int PAIR_A_BYTES = 128 * KB, PAIR_B_BYTES = 128 * KB, PAIR_STAGE_BYTES = PAIR_A_BYTES + PAIR_B_BYTES;
constexpr size_t pair_smem_bytes(int stages) { return (size_t)stages * PAIR_STAGE_BYTES + 1024 + 256; }
static_assert(pair_smem_bytes(7) <= 232448, "7 pair stages exceed the 227 KB of shared memory per CTA");

template <int NST>
__global__ void __launch_bounds__(THREADS, 1)
oz_gemm_tc_pair(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const Params P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + (size_t)NST * PAIR_STAGE_BYTES);
  // bars: full[NST], empty[NST], tfull[2], tempty[2]
  volatile int* abort_flag = (volatile int*)(bars + 2 * NST + 4);
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * NST + 5);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_ctarank();  // 0: leader
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + NST);
  const uint32_t tfull0 = smem_u32(bars + 2 * NST), tempty0 = smem_u32(bars + 2 * NST + 2);
  const uint32_t lead_full0 = mapa(full0, 0), lead_tempty0 = mapa(tempty0, 0);
  const uint32_t peer_abort = mapa(smem_u32((const void*)abort_flag), rank ^ 1u);
  const int pair_id = blockIdx.x >> 1, num_pairs = gridDim.x >> 1;
  const int total_tiles = P.tiles_m * P.tiles_n;  // tiles_m counts 256-row tiles here
  const int group = P.group_m / 2 > 0 ? P.group_m / 2 : 1;
  constexpr uint16_t BOTH = 3;

  if (threadIdx.x == 0) {
    for (int i = 0; i < NST; ++i) {
      mbar_init(full0 + 8 * i, 1);   // the leader's expect_tx arrival (+ both CTAs' bytes)
      mbar_init(empty0 + 8 * i, 1);  // one multicast commit
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(tfull0 + 8 * i, 1);
      mbar_init(tempty0 + 8 * i, 8);  // four epilogue warps in each CTA (used in the leader)
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0 && lane == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 1) tmem_alloc_pair(smem_u32(tmem_slot), TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  cluster_sync();  // both CTAs' barriers are initialised before any copy or commit lands
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------------------------------------------------------- TMA producer (both CTAs)
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      unsigned long long issued = 0, seen = 0;  // as in oz_gemm_tc: both CTAs of a pair publish
      const unsigned long long chunk_mask = (unsigned long long)P.pace_chunk - 1;
      for (int ct = pair_id; ct < total_tiles && ok; ct += num_pairs) {
        int tm, tn;
        tile_coords(ct, P.tiles_m, P.tiles_n, group, &tm, &tn);
        const int64_t arow = (int64_t)tm * PAIR_M + rank * 128;
        const int64_t brow = (int64_t)tn * BN + rank * 128;
        auto prefetch = [&](const Seq& f) {  // as in oz_gemm_tc
          tma_prefetch_2d(&tmA, 0, box_y(f.p, arow, f.kb, P.a_rows_pad, P.nkb));
          tma_prefetch_2d(&tmB, 0, box_y(f.g - f.p, brow, f.kb, P.b_rows_pad, P.nkb));
        };
        Seq q, f;
        f.start(P.s, P.nkb);
        for (int i = 0; i < P.pf && !f.done(); ++i, f.next()) prefetch(f);
        for (q.start(P.s, P.nkb); !q.done() && ok; q.next()) {
          if (P.pf > 0 && !f.done()) {
            prefetch(f);
            f.next();
          }
          if (P.pace_lag && (issued & chunk_mask) == 0) pace_gate(P, issued / P.pace_chunk, gridDim.x, seen);
          ++issued;
          ok = mbar_wait_pair<false>(empty0 + 8 * stage, phase ^ 1, abort_flag, peer_abort, P.err);
          if (!ok) break;
          if (rank == 0) mbar_expect_tx(full0 + 8 * stage, 2 * PAIR_STAGE_BYTES);
          uint8_t* sa = smem + (size_t)stage * PAIR_STAGE_BYTES;
          const uint32_t fb = lead_full0 + 8 * stage;
          tma_load_2d_pair(smem_u32(sa), &tmA, 0, box_y(q.p, arow, q.kb, P.a_rows_pad, P.nkb), fb);
          tma_load_2d_pair(smem_u32(sa + PAIR_A_BYTES), &tmB, 0, box_y(q.g - q.p, brow, q.kb, P.b_rows_pad, P.nkb), fb);
          if (++stage == NST) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      if (P.pace_lag) red_add_u64(P.pace, PACE_DONE);
      // drain: every copy issued has been consumed before the CTA may exit (bounded)
      for (int i = 0; i < NST; ++i) {
        (void)mbar_wait_pair<false>(empty0 + 8 * stage, phase ^ 1, abort_flag, peer_abort, P.err, false);
        if (++stage == NST) {
          stage = 0;
          phase ^= 1;
        }
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer (leader)
    // issue order as in oz_gemm_tc: the next k-block's bookkeeping between its third and fourth MMA
    if (lane == 0 && rank == 0) {
      constexpr uint64_t STAGE_STEP = (uint64_t)(PAIR_STAGE_BYTES >> 4);
      const uint32_t sa0 = smem_u32(smem);
      const uint64_t ad0 = smem_desc(sa0), bd0 = smem_desc(sa0 + PAIR_A_BYTES);
      auto nkb_of = [&](int) { return P.nkb; };
      PassCounter cur{};
      cur.start(pair_id, num_pairs, total_tiles, P.s, nkb_of);
      int stage = 0, buf = 0;
      uint32_t phase = 0, tph = 0;
      uint64_t ad = ad0, bd = bd0;
      bool ok = cur.valid;
      bool first = true, last = cur.last();
      if (ok) ok = mbar_wait_pair<true>(tempty0, 1, abort_flag, peer_abort, P.err);
      if (ok) ok = mbar_wait_pair<false>(full0, 0, abort_flag, peer_abort, P.err);
      tc_fence_after();
      while (ok) {
        const uint32_t d_tmem = tmem_base + (uint32_t)(buf * BN);
        const int nstage = stage + 1 == NST ? 0 : stage + 1;
        const uint32_t nphase = nstage == 0 ? phase ^ 1u : phase;
        // the k-block's MMAs, the stage's release in both CTAs and a probe of the next stage
        const uint32_t probe =
            kblock_f8_pair(d_tmem, ad, bd, first ? 0u : 1u, full0 + 8 * nstage, nphase, empty0 + 8 * stage);
        const bool nfirst = cur.next(num_pairs, total_tiles, P.s, nkb_of);
        const bool nvalid = cur.valid, nlast = cur.last();
        const uint64_t nad = nstage == 0 ? ad0 : ad + STAGE_STEP, nbd = nstage == 0 ? bd0 : bd + STAGE_STEP;
        const bool ready = nvalid && !nfirst && probe != 0;
        if (last) {
          mma_commit_pair(tfull0 + 8 * buf, BOTH);
          tph ^= 1u << buf;
          buf ^= 1;
        }
        stage = nstage;
        phase = nphase;
        ad = nad;
        bd = nbd;
        first = nfirst;
        last = nlast;
        if (ready) {
          tc_fence_after();
          continue;
        }
        if (!nvalid) break;
        if (first) {
          ok = mbar_wait_pair<true>(tempty0 + 8 * buf, ((tph >> buf) & 1u) ^ 1u, abort_flag, peer_abort, P.err);
          if (!ok) break;
        }
        ok = mbar_wait_pair<false>(full0 + 8 * stage, phase, abort_flag, peer_abort, P.err);
        if (!ok) break;
        tc_fence_after();
      }
      // both accumulators released by both CTAs: no MMA is in flight when TMEM is freed
      for (int b = 0; b < 2; ++b) {
        (void)mbar_wait_pair<true>(tempty0 + 8 * buf, ((tph >> buf) & 1u) ^ 1u, abort_flag, peer_abort, P.err, false);
        buf ^= 1;
      }
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2..5, both CTAs)
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;  // TMEM lane = row of this CTA's half of the tile
    double* slot = P.work + (size_t)blockIdx.x * (size_t)(BM * BN);
    const Epi E = epi_of(P);
    uint32_t tphase[2] = {0, 0};
    int buf = 0;
    bool ok = true;
    for (int ct = pair_id; ct < total_tiles && ok; ct += num_pairs) {
      int tm, tn;
      tile_coords(ct, P.tiles_m, P.tiles_n, group, &tm, &tn);
      bool first_pass = true;
      Seq q;
      for (q.start(P.s, P.nkb); !q.done() && ok; q.next()) {
        if (!q.pass_last()) continue;
        int okw = 1;
        if (lane == 0)
          okw = mbar_wait_pair<false>(tfull0 + 8 * buf, tphase[buf], abort_flag, peer_abort, P.err, true,
                                      P.epi_hint) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
        __syncwarp();
        if (!ok) break;
        tc_fence_after();
        const uint32_t tbase = tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * BN);
        const uint32_t tempty = lead_tempty0 + 8 * buf;
        drain_pass(tbase, slot, row, q.g, first_pass, q.tile_last(), E, (int64_t)tm * PAIR_M + rank * 128 + row,
                   (int64_t)tn * BN, [&] {
                     tc_fence_before();
                     __syncwarp();
                     if (lane == 0) mbar_arrive_cluster(tempty);
                   });
        first_pass = false;
        tphase[buf] ^= 1;
        buf ^= 1;
      }
    }
  }
  tc_fence_before();
  __syncwarp();
  __syncthreads();
  cluster_sync();  // the peer's copies, arrivals and the leader's MMAs into this CTA are over
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc_pair(tmem_base, TMEM_COLS);
  }
}

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

// the blocked digit planes as one column of 128-byte rows; a box is box_rows (<= 128) of them
cudaError_t make_map(CUtensorMap* map, const OzakiSplit& X, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {(cuuint64_t)KB, (cuuint64_t)X.slices * (cuuint64_t)X.rows_pad * (cuuint64_t)(X.k_pad / KB)};
  cuuint64_t strides[1] = {(cuuint64_t)KB};
  cuuint32_t box[2] = {(cuuint32_t)KB, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)X.digits, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Per-device launch set-up of both engine forms: the SM count, the opt-in to the large
// dynamic shared memory (a function attribute is per device) and the pair form's
// resident-cluster count.  Done once per device, with that device current, outside
// any stream capture (ozaki_tc_prepare).
struct DeviceSetup {
  std::once_flag once;
  cudaError_t status = cudaSuccess;
  int sms = 0;
  int max_pairs = 0;
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
    d.status = cudaFuncSetAttribute(oz_gemm_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (d.status != cudaSuccess) return;
    d.status = cudaFuncSetAttribute(oz_gemm_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (d.status != cudaSuccess) return;
    d.status = cudaFuncSetAttribute(oz_gemm_tc_pair<PAIR_STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)pair_smem_bytes(PAIR_STAGES));
    if (d.status != cudaSuccess) return;
    d.status = cudaFuncSetAttribute(oz_gemm_tc_pair<7>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)pair_smem_bytes(7));
    if (d.status != cudaSuccess) return;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)((d.sms / 2) * 2));
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = pair_smem_bytes(7);  // the larger instance: its count holds for both
    cfg.attrs = at;
    cfg.numAttrs = 1;
    d.status = cudaOccupancyMaxActiveClusters(&d.max_pairs, oz_gemm_tc_pair<7>, &cfg);
    if (d.status == cudaSuccess && d.max_pairs <= 0) d.status = cudaErrorInvalidConfiguration;
  });
  return &d;
}

int num_sms() {
  const DeviceSetup* d = device_setup();
  return d && d->status == cudaSuccess ? d->sms : 1;
}

// Persistent launch: one CTA per SM, at most one per tile.
cudaError_t launch(const CUtensorMap& ma, const CUtensorMap& mb, const Params& P, cudaStream_t s) {
  const DeviceSetup* d = device_setup();
  if (!d) return cudaErrorInvalidDevice;
  if (d->status != cudaSuccess) return d->status;
  const int64_t tiles = (int64_t)P.tiles_m * P.tiles_n;
  const int ctas = tiles < d->sms ? (int)tiles : d->sms;  // the workspace has one slot per SM
  oz_gemm_tc<false><<<ctas, THREADS, SMEM_BYTES, s>>>(ma, mb, P, GroupArgs{nullptr, nullptr, 0});
  return cudaGetLastError();
}

// Persistent launch of the pair engine: clusters of 2 CTAs, as many as can be resident.
cudaError_t launch_pair(const CUtensorMap& ma, const CUtensorMap& mb, const Params& P, cudaStream_t s) {
  const DeviceSetup* d = device_setup();
  if (!d) return cudaErrorInvalidDevice;
  if (d->status != cudaSuccess) return d->status;
  const int64_t tiles = (int64_t)P.tiles_m * P.tiles_n;
  const int pairs = tiles < d->max_pairs ? (int)tiles : d->max_pairs;
  if ((size_t)pairs * 2 > (size_t)d->sms) return cudaErrorInvalidConfiguration;  // workspace has one slot per SM
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(pairs * 2));
  cfg.blockDim = dim3(THREADS);
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int stages = PAIR_STAGES;
  if (const char* env = getenv("TMM_TC_PAIR_STAGES")) stages = atoi(env) == 7 ? 7 : PAIR_STAGES;
  cfg.dynamicSmemBytes = pair_smem_bytes(stages);
  if (stages == 7) return cudaLaunchKernelEx(&cfg, oz_gemm_tc_pair<7>, ma, mb, P);
  return cudaLaunchKernelEx(&cfg, oz_gemm_tc_pair<PAIR_STAGES>, ma, mb, P);
}

}  // namespace tc

cudaError_t ozaki_tc_prepare() {
  if (!tc::encode_fn()) return cudaErrorNotSupported;
  const tc::DeviceSetup* d = tc::device_setup();
  return d ? d->status : cudaErrorInvalidDevice;
}

// A launch's workspace: a 256-byte header (the wave-pacing counter) and one FP64 accumulator
// slot of 128 x 256 per CTA.
size_t ozaki_tc_workspace_bytes() { return tc::WORK_HEADER + (size_t)tc::num_sms() * tc::BM * tc::BN * sizeof(double); }
size_t ozaki_tc_workspace_bytes_for(int64_t m, int64_t n) {
  // a launch's grid is at most one CTA per SM and per tile (the pair form: per 256-row tile, two CTAs)
  const int64_t tiles_m = (m + tc::BM - 1) / tc::BM, tiles_n = (n + tc::BN - 1) / tc::BN;
  const int64_t ctas = std::min<int64_t>((int64_t)tc::num_sms(), (tiles_m + 1) / 2 * 2 * tiles_n);
  return tc::WORK_HEADER + (size_t)ctas * tc::BM * tc::BN * sizeof(double);
}
int64_t ozaki_tc_pass_blocks() { return tc::PASS_BLOCKS; }
int ozaki_tc_k_block() { return tc::KB; }

cudaError_t ozaki_tc_grouped_image(const std::vector<GroupedProduct>& prods, const void* arena, size_t arena_bytes,
                                   std::vector<unsigned char>& out, int* n_items) {
  std::vector<tc::GroupProblem> recs;
  std::vector<int4> items;
  std::vector<int64_t> cost;
  for (size_t i = 0; i < prods.size(); ++i) {
    const GroupedProduct& p = prods[i];
    const OzakiSplit& A = p.A;
    const OzakiSplit& B = p.B;
    if (p.m <= 0 || p.n <= 0) continue;
    if (A.enc != OZ_ENC_E4M3 || B.enc != OZ_ENC_E4M3 || A.k_pad != B.k_pad || A.slices != B.slices ||
        A.slices != prods[0].A.slices || A.rows_pad % tc::BM || B.rows_pad % tc::BN || A.k_pad % tc::KB ||
        !A.blocked || !B.blocked)
      return cudaErrorInvalidValue;
    const int64_t aoff = (const char*)A.digits - (const char*)arena, boff = (const char*)B.digits - (const char*)arena;
    if (aoff < 0 || boff < 0 || aoff % tc::KB || boff % tc::KB) return cudaErrorInvalidValue;
    // every box of the planes lies inside the arena that the launch's tensor map covers
    if ((size_t)aoff + (size_t)A.slices * (size_t)A.rows_pad * (size_t)A.k_pad > arena_bytes ||
        (size_t)boff + (size_t)B.slices * (size_t)B.rows_pad * (size_t)B.k_pad > arena_bytes)
      return cudaErrorInvalidValue;
    tc::GroupProblem r;
    r.a_row0 = aoff / tc::KB;
    r.b_row0 = boff / tc::KB;
    r.a_rows_pad = A.rows_pad;
    r.b_rows_pad = B.rows_pad;
    r.ea = A.exps;
    r.eb = B.exps;
    r.C = p.C;
    r.ldc = p.ldc;
    r.m = p.m;
    r.n = p.n;
    r.alpha = p.alpha;
    r.beta = p.beta;
    r.nkb = (int)(A.k_pad / tc::KB);
    r.first = p.first_k_tile ? 1 : 0;
    const int idx = (int)recs.size();
    recs.push_back(r);
    const int tm_n = (int)((p.m + tc::BM - 1) / tc::BM), tn_n = (int)((p.n + tc::BN - 1) / tc::BN);
    for (int tm = 0; tm < tm_n; ++tm)
      for (int tn = 0; tn < tn_n; ++tn) {
        items.push_back(make_int4(idx, tm, tn, 0));
        cost.push_back((int64_t)r.nkb);
      }
  }
  // largest tiles first: dealt round-robin to the CTAs, the longest sequences start first
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
  const size_t rec_bytes = (recs.size() * sizeof(tc::GroupProblem) + 255) / 256 * 256;
  out.assign(rec_bytes + items.size() * sizeof(int4), 0);
  if (!recs.empty()) memcpy(out.data(), recs.data(), recs.size() * sizeof(tc::GroupProblem));
  int4* it = (int4*)(out.data() + rec_bytes);
  for (size_t i = 0; i < order.size(); ++i) it[i] = items[order[i]];
  *n_items = (int)items.size();
  return cudaSuccess;
}

cudaError_t ozaki_gemm_tc_grouped(const void* arena, size_t arena_bytes, int slices, const void* dev_image, int n_probs,
                                  int n_items, double* work, int* err, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  if (!arena || !dev_image || !work || !err || arena_bytes / tc::KB > (size_t)INT32_MAX) return cudaErrorInvalidValue;
  const tc::DeviceSetup* d = tc::device_setup();
  if (!d) return cudaErrorInvalidDevice;
  if (d->status != cudaSuccess) return d->status;
  auto fn = tc::encode_fn();
  if (!fn) return cudaErrorNotSupported;
  // one map over the arena: A and B planes of every problem, as a column of 128-byte rows
  CUtensorMap map;
  cuuint64_t dims[2] = {(cuuint64_t)tc::KB, (cuuint64_t)(arena_bytes / tc::KB)};
  cuuint64_t strides[1] = {(cuuint64_t)tc::KB};
  cuuint32_t box[2] = {(cuuint32_t)tc::KB, (cuuint32_t)OZ_BLOCK};
  cuuint32_t estr[2] = {1, 1};
  if (fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(arena), dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  tc::Params P{};
  P.s = slices;
  P.work = (double*)((char*)work + tc::WORK_HEADER);
  P.pace = (unsigned long long*)work;
  P.err = err;
  P.group_m = tc::GROUP_M;
  P.epi_hint = tc::EPI_WAIT_HINT_NS;
  P.pace_chunk = 64;
  const size_t rec_bytes = ((size_t)n_probs * sizeof(tc::GroupProblem) + 255) / 256 * 256;
  tc::GroupArgs G{(const tc::GroupProblem*)dev_image, (const int4*)((const char*)dev_image + rec_bytes), n_items};
  const int ctas = n_items < d->sms ? n_items : d->sms;  // the workspace has one slot per SM
  tc::oz_gemm_tc<true><<<ctas, tc::THREADS, tc::SMEM_BYTES, s>>>(map, map, P, G);
  return cudaGetLastError();
}

cudaError_t ozaki_gemm_tc(const OzakiSplit& A, const OzakiSplit& B, int64_t m, int64_t n, double alpha, double beta,
                          bool first_k_tile, double* C, int64_t ldc, double* work, int* err, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  if (A.enc != OZ_ENC_E4M3 || B.enc != OZ_ENC_E4M3 || A.k_pad != B.k_pad || A.slices != B.slices ||
      A.rows_pad % tc::BM || B.rows_pad % tc::BN || A.k_pad % tc::KB || !A.blocked || !B.blocked || !work || !err)
    return cudaErrorInvalidValue;
  // TMA coordinates are 32-bit: every 128-byte row of the stacked planes must stay addressable
  if ((int64_t)A.slices * A.rows_pad * (A.k_pad / tc::KB) > INT32_MAX ||
      (int64_t)B.slices * B.rows_pad * (B.k_pad / tc::KB) > INT32_MAX)
    return cudaErrorInvalidValue;
  CUtensorMap ma, mb;
  tc::Params P;
  P.ea = A.exps;
  P.eb = B.exps;
  P.a_rows_pad = A.rows_pad;
  P.b_rows_pad = B.rows_pad;
  P.nkb = (int)(A.k_pad / tc::KB);
  P.s = A.slices;
  P.m = m;
  P.n = n;
  P.alpha = alpha;
  P.beta = beta;
  P.first = first_k_tile ? 1 : 0;
  P.C = C;
  P.ldc = ldc;
  P.pace = (unsigned long long*)work;
  P.work = (double*)((char*)work + tc::WORK_HEADER);
  P.err = err;
  // Engine form: CTA pairs issuing cta_group::2 MMAs on 256 x 256 tiles from two 128-row
  // tiles up (their operand traffic per SM is two thirds of the one-SM form's and a ring of
  // six 32 KB stages looks ahead 1.5x as far), else one CTA per SM on 128 x 256 tiles;
  // TMM_TC_CLUSTER=1 or =pair forces a form.  Wave pacing is on for the pair form, which
  // drifts apart without it, and off for the one-SM form, which it slowed by 2-4 %.  Measured
  // at m = n = 32768, k = 16384, 11 slices, under the power limit: one-SM 740-754 ms, pair
  // 871 ms, pair with a lag of 2 chunks of 64 k-blocks 700-714 ms, with a lag of 1 chunk
  // 688-700 ms per launch (the tighter lag costs ~3 % more cycles per launch but draws less
  // power, so the clock runs 5-9 % higher); at m = n = 8192: 46.5, 43.4, 43.3 ms.
  int cm = (m + tc::BM - 1) / tc::BM >= 2 ? 0 : 1;  // 0: pair
  if (const char* env = getenv("TMM_TC_CLUSTER")) {
    if (!strcmp(env, "pair")) cm = 0;
    else if (!strcmp(env, "1")) cm = 1;
  }
  P.pace_lag = cm == 0 ? 1 : 0;
  P.pace_chunk = 64;
  P.pace_ns = 20000;
  if (const char* env = getenv("TMM_TC_PACE")) P.pace_lag = atoi(env) < 0 ? 0 : atoi(env);
  if (const char* env = getenv("TMM_TC_PACE_CHUNK")) {
    const int c = atoi(env);
    if (c >= 1 && c <= 4096 && (c & (c - 1)) == 0) P.pace_chunk = c;
  }
  if (const char* env = getenv("TMM_TC_PACE_NS")) P.pace_ns = (uint32_t)(atoi(env) < 0 ? 0 : atoi(env));
  P.tiles_n = (int)((n + tc::BN - 1) / tc::BN);
  P.group_m = tc::GROUP_M;
  if (const char* env = getenv("TMM_TC_GROUP_M")) P.group_m = atoi(env) < 1 ? 1 : (atoi(env) > 256 ? 256 : atoi(env));
  P.epi_hint = tc::EPI_WAIT_HINT_NS;
  if (const char* env = getenv("TMM_TC_EPI_HINT_NS")) P.epi_hint = (uint32_t)(atoi(env) < 0 ? 0 : atoi(env));
  P.pf = 0;  // measured: any distance (4..32) slows the 8192^3 and 8192^2 x 32768 runs by 30-120 %
  if (const char* env = getenv("TMM_TC_PREFETCH")) P.pf = atoi(env) < 0 ? 0 : (atoi(env) > 64 ? 64 : atoi(env));
  if (cm == 0) {
    if (A.rows_pad % tc::PAIR_M) return cudaErrorInvalidValue;
    P.tiles_m = (int)((m + tc::PAIR_M - 1) / tc::PAIR_M);
    cudaError_t e = tc::make_map(&ma, A, 128);
    if (e == cudaSuccess) e = tc::make_map(&mb, B, 128);
    if (e == cudaSuccess && P.pace_lag) e = cudaMemsetAsync(P.pace, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    return tc::launch_pair(ma, mb, P, s);
  }
  P.tiles_m = (int)((m + tc::BM - 1) / tc::BM);
  cudaError_t e = tc::make_map(&ma, A, tc::BM);
  if (e == cudaSuccess) e = tc::make_map(&mb, B, OZ_BLOCK);
  if (e == cudaSuccess && P.pace_lag) e = cudaMemsetAsync(P.pace, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  return tc::launch(ma, mb, P, s);
}

}  // namespace tmm
