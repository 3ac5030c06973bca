/*
 * Counter-based synthetic matrix generator shared by host C, C++ and CUDA code.
 *
 * Element (matrix id, linear index) -> splitmix64(seed ^ (id << 56) ^ index).
 * The value of an element depends only on (seed, id, row, col, ld-independent
 * linear index row + col * rows), so a host buffer, a device buffer and an
 * oracle that regenerates single entries all agree bit for bit, whatever the
 * leading dimension or the thread count that filled them.
 *
 * Distributions (kind):
 *   TMM_GEN_UNIFORM   u in [-1, 1): the top 53 bits of the hash, scaled by 2^-52, minus 1.
 *   TMM_GEN_INT09     integers 0..9 (the reference's known-answer inputs, any product
 *                     and partial sum of which is exact in FP64 while 81*k < 2^53).
 *   TMM_GEN_UEXP      u * 2^e, u uniform [-1,1), e uniform integer in [-p, p]
 *                     (p = param; e comes from an independent hash stream).
 *   TMM_GEN_NORMAL_ROWEXP  N(0,1) (Box-Muller on two counters) * 2^{f(row)},
 *                     f(row) uniform real in [-p, p] drawn per row (param = p).
 *   TMM_GEN_NORMAL_COLEXP  same with the factor drawn per column.
 *   TMM_GEN_SMALLINT  integers in [-param, param] (used by exactness tests).
 */
#ifndef TMM_DATAGEN_H
#define TMM_DATAGEN_H

#include <stdint.h>

#if defined(__CUDACC__)
#define TMM_HD __host__ __device__ __forceinline__
#else
#define TMM_HD static inline
#endif

enum tmm_gen_kind {
  TMM_GEN_UNIFORM = 0,
  TMM_GEN_INT09 = 1,
  TMM_GEN_UEXP = 2,
  TMM_GEN_NORMAL_ROWEXP = 3,
  TMM_GEN_NORMAL_COLEXP = 4,
  TMM_GEN_SMALLINT = 5
};

TMM_HD uint64_t tmm_splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* uniform in [-1, 1) with 53 random bits */
TMM_HD double tmm_u_from_hash(uint64_t h) {
  return (double)(h >> 11) * (1.0 / 4503599627370496.0) - 1.0; /* 2^52 */
}

/* uniform in [0, 1) with 53 random bits */
TMM_HD double tmm_u01_from_hash(uint64_t h) {
  return (double)(h >> 11) * (1.0 / 9007199254740992.0); /* 2^53 */
}

TMM_HD uint64_t tmm_key(uint64_t seed, uint64_t id, uint64_t idx) {
  return seed ^ (id << 56) ^ idx;
}

/* independent streams are separated by flipping high bits of the id */
#define TMM_STREAM_EXP 0x40ull
#define TMM_STREAM_BM2 0x80ull

/* power of two 2^e for integer e in [-1022, 1023] without libm */
TMM_HD double tmm_pow2i(int e) {
  union { uint64_t u; double d; } v;
  v.u = (uint64_t)(e + 1023) << 52;
  return v.d;
}

/*
 * Box-Muller needs log, sqrt and cos.  These are called from host code only
 * for the NORMAL kinds; device generation of the NORMAL kinds uses the CUDA
 * math library, and the two sides are compared with a tolerance, never bit for
 * bit (the other kinds are bit-exact on both sides).
 */
#if defined(__CUDACC__)
#define TMM_LOG log
#define TMM_SQRT sqrt
#define TMM_COS cospi
#define TMM_EXP2 exp2
#else
#include <math.h>
#define TMM_LOG log
#define TMM_SQRT sqrt
#define TMM_COS(x) cos(3.14159265358979323846 * (x))
#define TMM_EXP2 exp2
#endif

/* value of element (row, col) of a rows x cols matrix */
TMM_HD double tmm_gen_value(int kind, double param, uint64_t seed, uint64_t id,
                            int64_t row, int64_t col, int64_t rows) {
  uint64_t idx = (uint64_t)row + (uint64_t)col * (uint64_t)rows;
  uint64_t h = tmm_splitmix64(tmm_key(seed, id, idx));
  switch (kind) {
    case TMM_GEN_INT09:
      return (double)(h % 10ull);
    case TMM_GEN_SMALLINT: {
      uint64_t span = (uint64_t)(2.0 * param + 1.0);
      return (double)(int64_t)(h % span) - param;
    }
    case TMM_GEN_UEXP: {
      int p = (int)param;
      uint64_t he = tmm_splitmix64(tmm_key(seed, id ^ TMM_STREAM_EXP, idx));
      int e = (int)(he % (uint64_t)(2 * p + 1)) - p;
      return tmm_u_from_hash(h) * tmm_pow2i(e);
    }
    case TMM_GEN_NORMAL_ROWEXP:
    case TMM_GEN_NORMAL_COLEXP: {
      uint64_t h2 = tmm_splitmix64(tmm_key(seed, id ^ TMM_STREAM_BM2, idx));
      double u1 = 1.0 - tmm_u01_from_hash(h); /* (0, 1] */
      double u2 = tmm_u01_from_hash(h2);
      double z = TMM_SQRT(-2.0 * TMM_LOG(u1)) * TMM_COS(2.0 * u2);
      uint64_t line = (kind == TMM_GEN_NORMAL_ROWEXP) ? (uint64_t)row : (uint64_t)col;
      uint64_t hf = tmm_splitmix64(tmm_key(seed, id ^ TMM_STREAM_EXP, line));
      double f = (2.0 * tmm_u01_from_hash(hf) - 1.0) * param;
      return z * TMM_EXP2(f);
    }
    case TMM_GEN_UNIFORM:
    default:
      return tmm_u_from_hash(h);
  }
}

#endif /* TMM_DATAGEN_H */
