// Issue-rate probes for the instructions the library's engines are built on, on one GB300:
//   dmma    mma.sync m16n8k4 f64 (native FP64 tile kernel)
//   imma    mma.sync m16n8k32 s8 -> s32 (IMMA Ozaki engine)
//   tcgen05 tcgen05.mma.cta_group::1.kind::f8f6f4, M128 N256 K32, e4m3 operands resident in shared
//           (and kind::f16 with bf16 operands, M128 N256 K16, the FP32 engine's instruction)
//           memory, issued back to back from one thread (tcgen05 Ozaki engine, pipe ceiling)
//   pair    tcgen05.mma.cta_group::2.kind::f8f6f4, M256 N256 K32 on a cluster of two CTAs (the
//           pair engine's instruction): back to back, with a commit to a stage barrier after
//           every k-block, with that commit plus a probe of a completed barrier, with both
//           plus a tcgen05.fence::after_thread_sync per k-block, and with all of that while a
//           thread of another warp in each CTA spins on an mbarrier (as a waiting producer);
//           then back to back again on operands of Ozaki digits (pseudo-random integers in
//           [-16, 16] as e4m3) and on pseudo-random finite e4m3 bytes, instead of 1.0; and in
//           the engine's 6-stage handshake without copies (a producer thread per CTA waits for
//           each stage's release and re-arms its full barrier; the issuer probes the next
//           stage's full barrier before the fourth MMA and waits on it when the probe fails),
//           and variants of that handshake (producer parked instead of polling; issuer waiting
//           after the fourth MMA instead of probing; 4 stages; other warps parked on a barrier);
//           finally back to back and with the engine's issue block for about a second each on
//           digit operands (sustained load at the power limit), with the SM clock the cycle
//           count and the event time imply
// Every CTA runs a fixed number of iterations; the tcgen05 probe's one wait is bounded by %globaltimer.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -o engine_rates engine_rates.cu
//   ./engine_rates        # one JSON line per probe
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#define CK(x)                                                                     \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      printf("{\"error\": \"%s: %s\"}\n", #x, cudaGetErrorString(e_));            \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

__global__ void dmma_loop(double* out, int iters) {
  double acc[4][4] = {};
  const double a0 = threadIdx.x * 1e-3, a1 = a0 + 1.0, b0 = 0.5;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
      asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                   : "+d"(acc[c][0]), "+d"(acc[c][1]), "+d"(acc[c][2]), "+d"(acc[c][3])
                   : "d"(a0), "d"(a1), "d"(b0));
  }
  double s = 0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) s += acc[i][j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void imma_loop(int* out, int iters) {
  int acc[4][4] = {};
  const int a0 = 0x01020304 + threadIdx.x, a1 = a0 ^ 0x05050505, a2 = a0 + 7, a3 = a1 + 9, b0 = 0x01010101, b1 = 0x02020202;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+r"(acc[c][0]), "+r"(acc[c][1]), "+r"(acc[c][2]), "+r"(acc[c][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  int s = 0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) s += acc[i][j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major, 128-byte swizzle, 8-row groups 1024 bytes apart (the engine's operand layout)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
         ((uint64_t)2 << 61);
}

__device__ __forceinline__ bool try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}

// One CTA per SM; 4 operand stages of 16 KB (A, 128 x 128 bytes) + 32 KB (B, 256 x 128 bytes) filled
// with e4m3 1.0; `kblocks` k-blocks of 4 MMAs into two alternating TMEM accumulators.
// mode 0: back to back, the next stage's descriptors computed between the third and fourth MMA;
// mode 1: descriptors, accumulator and flags computed after the fourth MMA, then a check of a
//         barrier that has already completed (up to 256 probes), as a straightforward loop does;
// mode 2: mode 0 plus a one-shot probe of that barrier between the third and fourth MMA.
__global__ void __launch_bounds__(128, 1) tcgen05_loop(int kblocks, int mode, long long* cycles, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t fin, done0;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < 4 * 49152 / 4; i += blockDim.x) ((uint32_t*)smem)[i] = 0x38383838u;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&fin)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done0)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&done0)) : "memory");  // phase 0 done
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)), "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  if (warp == 0 && lane == 0) {
    const uint64_t ad0 = smem_desc(smem_u32(smem)), bd0 = smem_desc(smem_u32(smem + 16384));
    const long long t0 = clock64();
    uint64_t ad = ad0, bd = bd0;
    const uint32_t d0 = smem_u32(&done0);
    if (mode == 1) {
      for (int kb = 0; kb < kblocks; ++kb) {
        for (int i = 0; i < 256; ++i)
          if (try_wait(d0, 0)) break;
        const int st = kb & 3;
        const uint64_t a = smem_desc(smem_u32(smem + st * 49152)), b = smem_desc(smem_u32(smem + st * 49152 + 16384));
        const uint32_t d = tmem + (uint32_t)(((kb / 512) & 1) * 256);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint32_t acc = (kb % 512 == 0 && kk == 0) ? 0u : 1u;
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
                       ::"r"(d), "l"(a + 2 * kk), "l"(b + 2 * kk), "r"(IDESC), "r"(acc));
        }
      }
    }
    if (mode == 3) {  // kind::f16, bf16 operands (the FP32 engine's instruction), back to back
      constexpr uint32_t IDESC_BF16 =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      for (int kb = 0; kb < kblocks; ++kb) {
        const uint32_t d = tmem + (uint32_t)(((kb >> 9) & 1) * 256);
        const uint32_t acc0 = (kb & 511) ? 1u : 0u;
        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                     ::"r"(d), "l"(ad), "l"(bd), "r"(IDESC_BF16), "r"(acc0));
        asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 2), "l"(bd + 2), "r"(IDESC_BF16));
        asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 4), "l"(bd + 4), "r"(IDESC_BF16));
        asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 6), "l"(bd + 6), "r"(IDESC_BF16));
        const bool wrap = (kb & 3) == 3;
        ad = wrap ? ad0 : ad + (49152 >> 4);
        bd = wrap ? bd0 : bd + (49152 >> 4);
      }
    }
    for (int kb = 0; mode != 1 && mode != 3 && kb < kblocks; ++kb) {
      const uint32_t d = tmem + (uint32_t)(((kb >> 9) & 1) * 256);
      const uint32_t acc0 = (kb & 511) ? 1u : 0u;
      asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
                   ::"r"(d), "l"(ad), "l"(bd), "r"(IDESC), "r"(acc0));
      asm volatile("tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 2), "l"(bd + 2), "r"(IDESC));
      asm volatile("tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 4), "l"(bd + 4), "r"(IDESC));
      const bool wrap = (kb & 3) == 3;
      const uint64_t nad = wrap ? ad0 : ad + (49152 >> 4), nbd = wrap ? bd0 : bd + (49152 >> 4);
      if (mode == 2 && !try_wait(d0, 0)) atomicOr(err, 2);
      asm volatile("tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 6), "l"(bd + 6), "r"(IDESC));
      ad = nad;
      bd = nbd;
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&fin)) : "memory");
    uint64_t g0, g1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
    while (true) {
      uint32_t ok;
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                   : "=r"(ok) : "r"(smem_u32(&fin)) : "memory");
      if (ok) break;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
      if (g1 - g0 > 1000000000ull) {
        atomicOr(err, 1);
        break;
      }
    }
    cycles[blockIdx.x] = clock64() - t0;
  }
  __syncwarp();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

// Cluster of two CTAs on one TPC; each stages 4 x (16 KB of A rows + 16 KB of its half of B)
// filled with e4m3 1.0; the leader issues `kblocks` k-blocks of 4 cta_group::2 MMAs
// (M256 N256 K32) into two alternating TMEM accumulators.
// mode 0: back to back; mode 1: plus a commit of each k-block to a stage barrier in both CTAs
// (multicast arrive, as the engine releases a stage); mode 2: mode 1 plus a probe of an
// already-completed barrier between the third and fourth MMA; mode 3: mode 2 plus a
// tcgen05.fence::after_thread_sync after each k-block's commit; mode 4: mode 3 while lane 0
// of warp 1 in both CTAs polls the final barrier with try_wait until the MMAs are done.
// mode 5: the engine's stage handshake on 6 stages of 16 KB + 16 KB, no copies: lane 0 of warp 1
// in each CTA waits (bounded) on the stage's empty barrier, which the issuer's per-k-block
// commit releases in both CTAs, and the leader's re-arms the stage's full barrier; the issuer
// probes the next stage's full barrier between the third and fourth MMA and, when the probe
// fails, waits on it (bounded) before the next k-block.  mode 6: the producers park in try_wait
// with a 1 us suspend hint instead of polling; mode 7: the issuer waits on the next full barrier
// after the commit instead of probing it before the fourth MMA; mode 8: mode 5 on 4 stages;
// mode 9: mode 5 while warps 2-3 of both CTAs park on the final barrier (20 us hint); mode 10:
// mode 5 with the probe made by mbarrier.test_wait (never suspends) instead of try_wait;
// mode 11: the test_wait probe issued right after the first MMA, its result read only after
// the fourth MMA and the commit (one asm block).
// fill 0: every operand byte e4m3 1.0; 1: digits, uniform integers in [-16, 16]; 2: uniform
// finite e4m3 bytes (NaN codes replaced by 0).
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ uint8_t fill_byte(int fill, uint32_t i, uint32_t salt) {
  // e4m3 codes of the integers 0..16
  const uint8_t code[17] = {0x00, 0x38, 0x40, 0x44, 0x48, 0x4A, 0x4C, 0x4E, 0x50,
                            0x51, 0x52, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58};
  if (fill == 0) return 0x38;
  const uint32_t h = mix32(i * 2654435761u + salt);
  if (fill == 1) {
    const int d = (int)(h % 33u) - 16;
    return (uint8_t)((d < 0 ? 0x80 : 0x00) | code[d < 0 ? -d : d]);
  }
  const uint8_t b = (uint8_t)(h >> 8);
  return (b & 0x7F) == 0x7F ? 0 : b;
}
__global__ void __launch_bounds__(128, 1) tcgen05_pair_loop(int kblocks, int mode, long long* cycles, int* err,
                                                            int fill) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t fin, done0, stage_bar[4], full6[6], empty6[6];
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t rank;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
  const int nstage = mode >= 5 ? 6 : 4;
  for (int i = threadIdx.x; i < nstage * 32768; i += blockDim.x) smem[i] = fill_byte(fill, (uint32_t)i, blockIdx.x);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&fin)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done0)));
    for (int i = 0; i < 4; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&stage_bar[i])));
    for (int i = 0; i < 6; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full6[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty6[i])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&done0)) : "memory");  // phase 0 done
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)), "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n barrier.cluster.wait.acquire.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  constexpr uint32_t IDESC2 = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
  const long long t0 = clock64();
  auto bounded_wait = [&](uint32_t bar, uint32_t parity, int code) {
    if (try_wait(bar, parity)) return;
    uint64_t g0, g1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
    while (!try_wait(bar, parity)) {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
      if (g1 - g0 > 1000000000ull) {
        atomicOr(err, code);
        return;
      }
    }
  };
  const bool hs = mode >= 5;  // the handshake modes
  const int ns = mode == 8 ? 4 : 6;
  if (mode == 9 && (warp == 2 || warp == 3)) {  // parked neighbours, bounded by %globaltimer
    uint64_t g0, g1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
    while (true) {
      uint32_t ok;
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0, %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                   : "=r"(ok) : "r"(smem_u32(&fin)), "r"(20000u) : "memory");
      if (ok) break;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
      if (g1 - g0 > 1000000000ull) {
        atomicOr(err, 32);
        break;
      }
    }
  }
  if (hs && warp == 1 && lane == 0) {  // producer: no copies, only the handshake
    int st = 0;
    uint32_t ph = 0;
    for (int kb = 0; kb < kblocks; ++kb) {
      if (mode == 6) {
        uint64_t g0, g1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
        while (true) {
          uint32_t ok;
          asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
                       : "=r"(ok) : "r"(smem_u32(&empty6[st])), "r"(ph ^ 1u), "r"(1000u) : "memory");
          if (ok) break;
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
          if (g1 - g0 > 1000000000ull) {
            atomicOr(err, 8);
            break;
          }
        }
      } else {
        bounded_wait(smem_u32(&empty6[st]), ph ^ 1u, 8);
      }
      if (rank == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full6[st])) : "memory");
      if (++st == ns) {
        st = 0;
        ph ^= 1u;
      }
    }
  }
  if (mode == 11 && warp == 0 && lane == 0 && rank == 0) {  // deferred-probe issuer
    const uint64_t ad0 = smem_desc(smem_u32(smem)), bd0 = smem_desc(smem_u32(smem + 16384));
    uint64_t ad = ad0, bd = bd0;
    int st = 0;
    uint32_t ph = 0;
    bounded_wait(smem_u32(&full6[0]), 0, 16);
    for (int kb = 0; kb < kblocks; ++kb) {
      const uint32_t d = tmem + (uint32_t)(((kb >> 9) & 1) * 256);
      const uint32_t acc0 = (kb & 511) ? 1u : 0u;
      const int nst = st + 1 == 6 ? 0 : st + 1;
      const uint32_t nph = nst == 0 ? ph ^ 1u : ph;
      uint32_t okv;
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
          : "=r"(okv)
          : "r"(d), "l"(ad), "l"(bd), "r"(IDESC2), "r"(acc0), "r"(smem_u32(&full6[nst])), "r"(nph), "l"(ad + 2),
            "l"(bd + 2), "l"(ad + 4), "l"(bd + 4), "l"(ad + 6), "l"(bd + 6), "r"(smem_u32(&empty6[st])), "h"((uint16_t)3)
          : "memory");
      const bool ready = kb + 1 == kblocks || okv != 0;
      ad = nst == 0 ? ad0 : ad + (32768 >> 4);
      bd = nst == 0 ? bd0 : bd + (32768 >> 4);
      st = nst;
      ph = nph;
      if (!ready) {
        atomicAdd(err + 1, 1);
        bounded_wait(smem_u32(&full6[st]), ph, 16);
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(smem_u32(&fin)), "h"((uint16_t)3) : "memory");
  }
  if (hs && mode != 11 && warp == 0 && lane == 0 && rank == 0) {  // issuer with the engine's handshake
    const uint64_t ad0 = smem_desc(smem_u32(smem)), bd0 = smem_desc(smem_u32(smem + 16384));
    uint64_t ad = ad0, bd = bd0;
    int st = 0;
    uint32_t ph = 0;
    bounded_wait(smem_u32(&full6[0]), 0, 16);
    for (int kb = 0; kb < kblocks; ++kb) {
      const uint32_t d = tmem + (uint32_t)(((kb >> 9) & 1) * 256);
      const uint32_t acc0 = (kb & 511) ? 1u : 0u;
      asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
                   ::"r"(d), "l"(ad), "l"(bd), "r"(IDESC2), "r"(acc0));
      asm volatile("tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 2), "l"(bd + 2), "r"(IDESC2));
      asm volatile("tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 4), "l"(bd + 4), "r"(IDESC2));
      const int nst = st + 1 == ns ? 0 : st + 1;
      const uint32_t nph = nst == 0 ? ph ^ 1u : ph;
      const uint64_t nad = nst == 0 ? ad0 : ad + (32768 >> 4), nbd = nst == 0 ? bd0 : bd + (32768 >> 4);
      bool ready;
      if (mode == 10) {
        uint32_t okv;
        asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(okv) : "r"(smem_u32(&full6[nst])), "r"(nph) : "memory");
        ready = kb + 1 == kblocks || okv != 0;
      } else {
        ready = kb + 1 == kblocks || (mode != 7 && try_wait(smem_u32(&full6[nst]), nph));
      }
      asm volatile("tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 6), "l"(bd + 6), "r"(IDESC2));
      asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                   ::"r"(smem_u32(&empty6[st])), "h"((uint16_t)3) : "memory");
      st = nst;
      ph = nph;
      ad = nad;
      bd = nbd;
      if (!ready) {
        if (mode != 7) atomicAdd(err + 1, 1);  // probes that failed
        bounded_wait(smem_u32(&full6[st]), ph, 16);
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(smem_u32(&fin)), "h"((uint16_t)3) : "memory");
  }
  if (!hs && warp == 0 && lane == 0 && rank == 0) {
    const uint64_t ad0 = smem_desc(smem_u32(smem)), bd0 = smem_desc(smem_u32(smem + 16384));
    uint64_t ad = ad0, bd = bd0;
    const uint32_t d0 = smem_u32(&done0);
    for (int kb = 0; kb < kblocks; ++kb) {
      const uint32_t d = tmem + (uint32_t)(((kb >> 9) & 1) * 256);
      const uint32_t acc0 = (kb & 511) ? 1u : 0u;
      asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
                   ::"r"(d), "l"(ad), "l"(bd), "r"(IDESC2), "r"(acc0));
      asm volatile("tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 2), "l"(bd + 2), "r"(IDESC2));
      asm volatile("tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 4), "l"(bd + 4), "r"(IDESC2));
      const bool wrap = (kb & 3) == 3;
      const uint64_t nad = wrap ? ad0 : ad + (32768 >> 4), nbd = wrap ? bd0 : bd + (32768 >> 4);
      if (mode == 2 && !try_wait(d0, 0)) atomicOr(err, 2);
      asm volatile("tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, 1;" ::"r"(d), "l"(ad + 6), "l"(bd + 6), "r"(IDESC2));
      if (mode >= 1)
        asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                     ::"r"(smem_u32(&stage_bar[kb & 3])), "h"((uint16_t)3) : "memory");
      if (mode >= 3) asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      ad = nad;
      bd = nbd;
    }
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(smem_u32(&fin)), "h"((uint16_t)3) : "memory");
  }
  if (mode == 4 && warp == 1 && lane == 0) {  // a spinning neighbour, bounded by %globaltimer
    uint64_t g0, g1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
    while (!try_wait(smem_u32(&fin), 0)) {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
      if (g1 - g0 > 1000000000ull) {
        atomicOr(err, 4);
        break;
      }
    }
  }
  if (warp == 0 && lane == 0) {  // both CTAs: the leader's last commit arrives here too
    uint64_t g0, g1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
    while (true) {
      uint32_t ok;
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                   : "=r"(ok) : "r"(smem_u32(&fin)) : "memory");
      if (ok) break;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
      if (g1 - g0 > 1000000000ull) {
        atomicOr(err, 1);
        break;
      }
    }
    if (rank == 0) cycles[blockIdx.x >> 1] = clock64() - t0;
  }
  __syncwarp();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n barrier.cluster.wait.acquire.aligned;" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

static float time_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

int main() {
  int dev = 0, sms = 0, clk_khz = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  void* out = nullptr;
  CK(cudaMalloc(&out, (size_t)sms * 8 * 256 * sizeof(double)));
  {  // DMMA: 8 warps per CTA, 2 CTAs per SM
    const int iters = 20000, block = 256, grid = sms * 2;
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(e0));
      dmma_loop<<<grid, block>>>((double*)out, iters);
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      const double flop = (double)grid * (block / 32) * iters * 4 * (2.0 * 16 * 8 * 4);
      if (rep) printf("{\"probe\": \"dmma_m16n8k4_f64\", \"tflops\": %.3f}\n", flop / time_ms(e0, e1) / 1e9);
    }
  }
  {  // IMMA s8
    const int iters = 20000, block = 256, grid = sms * 2;
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(e0));
      imma_loop<<<grid, block>>>((int*)out, iters);
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      const double ops = (double)grid * (block / 32) * iters * 4 * (2.0 * 16 * 8 * 32);
      if (rep) printf("{\"probe\": \"imma_m16n8k32_s8\", \"tops\": %.3f}\n", ops / time_ms(e0, e1) / 1e9);
    }
  }
  for (int mode = 0; mode < 4; ++mode) {  // tcgen05 e4m3 pipe (modes 0-2), bf16 pipe (mode 3)
    const int kblocks = 20000;
    const int smem = 4 * 49152 + 1024;
    long long* cyc = nullptr;
    int* err = nullptr;
    CK(cudaMalloc(&cyc, sms * sizeof(long long)));
    CK(cudaMalloc(&err, sizeof(int)));
    CK(cudaMemset(err, 0, sizeof(int)));
    CK(cudaFuncSetAttribute(tcgen05_loop, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(e0));
      tcgen05_loop<<<sms, 128, smem>>>(kblocks, mode, cyc, err);
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      if (!rep) continue;
      long long h[512];
      int herr = 0;
      const int n = sms < 512 ? sms : 512;
      CK(cudaMemcpy(h, cyc, n * sizeof(long long), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
      double c = 0;
      for (int i = 0; i < n; ++i) c += (double)h[i];
      c /= n;
      // a k-block is 128 bytes of K: 128 e4m3 or 64 bf16 elements
      const double kel = mode == 3 ? 64.0 : 128.0;
      const double flop = (double)sms * kblocks * (2.0 * 128 * 256 * kel);
      static const char* form[4] = {"back_to_back", "bookkeeping_after_4th_mma", "probe_between_3rd_and_4th",
                                    "back_to_back"};
      printf("{\"probe\": \"%s\", \"issue_loop\": \"%s\", \"tflops\": %.1f, "
             "\"cycles_per_kblock\": %.1f, \"flop_per_clk_per_sm\": %.0f, \"tflops_at_max_clock\": %.1f, "
             "\"wait_error\": %d}\n",
             mode == 3 ? "tcgen05_f16_bf16_m128n256k16" : "tcgen05_f8f6f4_m128n256k32", form[mode],
             flop / time_ms(e0, e1) / 1e9, c / kblocks, 2.0 * 128 * 256 * kel * kblocks / c,
             2.0 * 128 * 256 * kel * kblocks / c * sms * (clk_khz * 1e3) / 1e12, herr);
    }
    CK(cudaFree(cyc));
    CK(cudaFree(err));
  }
  for (int run = 0; run < 17; ++run) {  // tcgen05 cta_group::2 e4m3 pipe on CTA pairs
    const int mode = run < 5 ? run : (run < 7 ? 0 : (run < 9 ? 5 : (run < 15 ? run - 3 : (run == 15 ? 0 : 11))));
    const int fill = run < 5 ? 0 : (run < 7 ? run - 4 : (run < 9 ? run - 7 : (run < 15 ? 0 : 1)));
    const bool sustained = run >= 15;
    const int kblocks = sustained ? 3000000 : 20000, pairs = sms / 2;
    const int smem = 6 * 32768 + 1024;
    long long* cyc = nullptr;
    int* err = nullptr;
    CK(cudaMalloc(&cyc, pairs * sizeof(long long)));
    CK(cudaMalloc(&err, 2 * sizeof(int)));
    CK(cudaMemset(err, 0, 2 * sizeof(int)));
    CK(cudaFuncSetAttribute(tcgen05_pair_loop, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(pairs * 2));
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(e0));
      CK(cudaLaunchKernelEx(&cfg, tcgen05_pair_loop, kblocks, mode, cyc, err, fill));
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      if (!rep) continue;
      long long h[256];
      int herr[2] = {0, 0};
      const int n = pairs < 256 ? pairs : 256;
      CK(cudaMemcpy(h, cyc, n * sizeof(long long), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(herr, err, 2 * sizeof(int), cudaMemcpyDeviceToHost));
      double c = 0;
      for (int i = 0; i < n; ++i) c += (double)h[i];
      c /= n;
      // per SM: a 128 x 256 half of the M256 tile, 128 e4m3 of K per k-block
      const double flop_sm = 2.0 * 128 * 256 * 128;
      static const char* form[12] = {"back_to_back", "commit_per_kblock", "commit_and_probe_per_kblock",
                                     "commit_probe_and_fence_per_kblock", "same_with_a_spinning_neighbour_warp",
                                     "engine_stage_handshake_no_copies", "handshake_producer_parked",
                                     "handshake_issuer_waits_after_commit", "handshake_4_stages",
                                     "handshake_with_parked_neighbour_warps", "handshake_test_wait_probe",
                                     "handshake_test_wait_probe_read_after_4th_mma"};
      static const char* fills[3] = {"e4m3_one", "ozaki_digits", "random_finite_e4m3"};
      printf("{\"probe\": \"tcgen05_pair_f8f6f4_m256n256k32\", \"issue_loop\": \"%s\", \"operands\": \"%s\", "
             "\"kblocks\": %d, \"ms\": %.1f, \"tflops\": %.1f, \"cycles_per_kblock\": %.1f, "
             "\"flop_per_clk_per_sm\": %.0f, \"implied_sm_mhz\": %.0f, \"wait_error\": %d, \"failed_probes\": %d}\n",
             form[mode], fills[fill], kblocks, time_ms(e0, e1), flop_sm * 2 * pairs * kblocks / time_ms(e0, e1) / 1e9,
             c / kblocks, flop_sm * kblocks / c, c / (time_ms(e0, e1) * 1e3), herr[0], herr[1]);
    }
    CK(cudaFree(cyc));
    CK(cudaFree(err));
  }
  return 0;
}
