/*
 * ORACLE — test infrastructure only.
 *
 * A CPU restatement of Tiled-MM's out-of-core tiled GEMM, used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline / reference legs of bench.py as
 * the checker.  Nothing in the product library links, loads or calls this
 * file; the product path fails loudly when its CUDA library is missing.
 *
 * Parity is pinned two ways (see tests/test_oracle.py):
 *   1. against the reference's own host code (src/Tiled-MM/*.cpp) compiled
 *      here with a host stand-in for the CUDA runtime and cuBLAS
 *      (oracle/fake_cuda, built by oracle/Makefile into oracle/_ref/): same
 *      tile policy, same tile geometry, same results on the reference's
 *      integer known-answer inputs (tests/test-multiply.cpp:58-66) and on the
 *      reference CI shapes (ci/daint-alps.yml:48-64);
 *   2. against golden vectors under tests/golden/ produced by that build.
 *
 * What each function restates (file:line in the reference project):
 *   tmmo_optimal_tile_size   src/Tiled-MM/mm_handle.cpp:89-110
 *   tmmo_optimal_tile_sizes  src/Tiled-MM/mm_handle.cpp:117-133
 *   tmmo_tile_extent         src/Tiled-MM/tiled_matrix.cpp:8-23,31-39,75-80
 *   tmmo_gemm                src/Tiled-MM/tiled_mm.cpp:492-624 (driver),
 *                            270-365 (round_robin, copy_c_back = true),
 *                            367-454 (round_robin_without_copy_c),
 *                            168-268 (per-tile ?gemm: cuBLAS, restated as a
 *                            plain column-major GEMM, the published BLAS
 *                            semantics: C = alpha*op(A)*op(B) + beta*C, C not
 *                            read when beta == 0)
 * Indexing is 64-bit throughout (the reference's int offsets overflow past
 * 2^31 elements, tiled_matrix.cpp:62-66).
 *
 * Build: gcc -O3 -ffp-contract=off -fPIC -shared (oracle/Makefile).  No
 * architecture-specific flags: the same results on x86-64 and aarch64.
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;
typedef float complex cf;
typedef double complex cd;

enum { TMMO_S = 0, TMMO_D = 1, TMMO_C = 2, TMMO_Z = 3 };

static int upper(char c) { return (c >= 'a' && c <= 'z') ? c - 32 : c; }

/* ---------------------------------------------------------------- policy */

/* mm_handle.cpp:89-110: grow to dim when possible, else the largest divisor
 * of dim that is <= max_tile, kept only when within max_tile/2 of max_tile. */
int tmmo_optimal_tile_size(int dim, int curr_tile_size, int max_tile_size) {
  if (curr_tile_size < max_tile_size && dim <= max_tile_size) return dim;
  int limit = max_tile_size < dim ? max_tile_size : dim;
  int tile = 1;
  for (int i = 1; i <= limit; ++i)
    if (dim % i == 0) tile = i;
  int diff = max_tile_size - tile;
  if (diff < 0) diff = -diff;
  if (diff <= max_tile_size / 2) return tile;
  return limit;
}

/* mm_handle.cpp:117-133: the current tile sizes are the C buffer's (rows,
 * cols) for m and n and the A buffer's cols for k. */
void tmmo_optimal_tile_sizes(int m, int n, int k, int cur_m, int cur_n, int cur_k,
                             int max_m, int max_n, int max_k, int* out3) {
  out3[0] = tmmo_optimal_tile_size(m, cur_m, max_m);
  out3[1] = tmmo_optimal_tile_size(n, cur_n, max_n);
  out3[2] = tmmo_optimal_tile_size(k, cur_k, max_k);
}

/* ---------------------------------------------------------------- geometry */

/* tiled_matrix.cpp:13-22: the tile is clipped to the matrix; the number of
 * tiles is ceil(len/tile); the last tile is short when len % tile != 0. */
i64 tmmo_num_tiles(i64 len, i64 tile) {
  if (tile > len) tile = len;
  if (tile <= 0) return 0;
  return (len + tile - 1) / tile;
}

/* tiled_matrix.cpp:75-80 */
i64 tmmo_tile_extent(i64 len, i64 tile, i64 id) {
  if (tile > len) tile = len;
  i64 n = tmmo_num_tiles(len, tile);
  i64 rem = len % tile;
  return (id == n - 1 && rem > 0) ? rem : tile;
}

/* ---------------------------------------------------------------- per-tile GEMM */

/* element accessors: op(X)(r, c) of a stored column-major matrix */
static inline double getd(const double* x, i64 ld, int op, i64 r, i64 c) {
  return op == 'N' ? x[r + c * ld] : x[c + r * ld];
}
static inline float gets(const float* x, i64 ld, int op, i64 r, i64 c) {
  return op == 'N' ? x[r + c * ld] : x[c + r * ld];
}
static inline cd getz(const cd* x, i64 ld, int op, i64 r, i64 c) {
  if (op == 'N') return x[r + c * ld];
  cd v = x[c + r * ld];
  return op == 'C' ? conj(v) : v;
}
static inline cf getc(const cf* x, i64 ld, int op, i64 r, i64 c) {
  if (op == 'N') return x[r + c * ld];
  cf v = x[c + r * ld];
  return op == 'C' ? conjf(v) : v;
}

typedef struct {
  int dtype, ta, tb;
  i64 m, n, k, tm, tn, tk;
  const void *alpha, *beta;
  const void *a, *b;
  i64 lda, ldb;
  void* c; /* host C (copy_c_back) */
  i64 ldc;
  int copy_c_back;
  void* full_c; /* compact m x n (ld = m) device-side C when !copy_c_back */
  i64 j_begin, j_end; /* column tiles owned by this worker */
} job_t;

/*
 * One worker computes every C tile in a range of tile columns, in the
 * reference's k-tile order (tiled_mm.cpp:301-309,339-348 and 402-446):
 *   k-tile 0:  Ct = alpha * op(At) op(Bt) + beta * Ct   (Ct not read when beta == 0;
 *              when beta != 0 Ct starts as the host tile: tiled_mm.cpp:325-330, 425-431)
 *   k-tile t:  Ct = alpha * op(At) op(Bt) + 1 * Ct
 * and the tile product is the plain sum over the tile's k in increasing order.
 * The result goes to host C (copy_c_back) or to the compact full C (ld = m).
 */
#define TILE_LOOP_BODY(T, GET, ZERO)                                                     \
  const T* A = (const T*)J->a;                                                           \
  const T* B = (const T*)J->b;                                                           \
  T alpha = *(const T*)J->alpha, beta = *(const T*)J->beta;                               \
  int beta_nz = (beta != ZERO);                                                          \
  i64 ntm = tmmo_num_tiles(J->m, J->tm), ntn = tmmo_num_tiles(J->n, J->tn),               \
      ntk = tmmo_num_tiles(J->k, J->tk);                                                 \
  i64 tmc = J->tm < J->m ? J->tm : J->m, tnc = J->tn < J->n ? J->tn : J->n,              \
      tkc = J->tk < J->k ? J->tk : J->k;                                                 \
  T* acc = (T*)malloc(sizeof(T) * (size_t)tmc);                                          \
  T* ct = (T*)malloc(sizeof(T) * (size_t)tmc * (size_t)tnc);                             \
  T* ap = (T*)malloc(sizeof(T) * (size_t)tmc * (size_t)tkc);                             \
  for (i64 nt = J->j_begin; nt < J->j_end; ++nt) {                                       \
    i64 n0 = nt * tnc, nn = tmmo_tile_extent(J->n, J->tn, nt);                            \
    for (i64 mt = 0; mt < ntm; ++mt) {                                                   \
      i64 m0 = mt * tmc, mm = tmmo_tile_extent(J->m, J->tm, mt);                          \
      T* Cout = J->copy_c_back ? (T*)J->c : (T*)J->full_c;                               \
      i64 ldo = J->copy_c_back ? J->ldc : J->m;                                          \
      const T* Cin = (const T*)J->c;                                                     \
      for (i64 kt = 0; kt < ntk; ++kt) {                                                 \
        i64 k0 = kt * tkc, kk = tmmo_tile_extent(J->k, J->tk, kt);                        \
        /* pack op(A) tile column-major (mm x kk) */                                     \
        for (i64 l = 0; l < kk; ++l)                                                     \
          for (i64 i = 0; i < mm; ++i) ap[i + l * mm] = GET(A, J->lda, J->ta, m0 + i, k0 + l); \
        for (i64 j = 0; j < nn; ++j) {                                                   \
          for (i64 i = 0; i < mm; ++i) acc[i] = ZERO;                                    \
          for (i64 l = 0; l < kk; ++l) {                                                 \
            T bv = GET(B, J->ldb, J->tb, k0 + l, n0 + j);                                 \
            const T* acol = ap + l * mm;                                                 \
            for (i64 i = 0; i < mm; ++i) acc[i] = acc[i] + acol[i] * bv;                 \
          }                                                                              \
          T* cc = ct + j * mm;                                                           \
          if (kt == 0) {                                                                 \
            if (beta_nz) {                                                               \
              for (i64 i = 0; i < mm; ++i)                                               \
                cc[i] = alpha * acc[i] + beta * Cin[(m0 + i) + (n0 + j) * J->ldc];       \
            } else {                                                                     \
              for (i64 i = 0; i < mm; ++i) cc[i] = alpha * acc[i];                       \
            }                                                                            \
          } else {                                                                       \
            for (i64 i = 0; i < mm; ++i) cc[i] = alpha * acc[i] + cc[i];                 \
          }                                                                              \
        }                                                                                \
      }                                                                                  \
      if (ntk == 0) { /* k == 0: C = beta * C (BLAS quick-return semantics) */           \
        for (i64 j = 0; j < nn; ++j)                                                     \
          for (i64 i = 0; i < mm; ++i)                                                   \
            ct[i + j * mm] = beta_nz ? beta * Cin[(m0 + i) + (n0 + j) * J->ldc] : ZERO;  \
      }                                                                                  \
      for (i64 j = 0; j < nn; ++j)                                                       \
        for (i64 i = 0; i < mm; ++i) Cout[(m0 + i) + (n0 + j) * ldo] = ct[i + j * mm];   \
    }                                                                                    \
  }                                                                                      \
  free(acc); free(ct); free(ap);

static void run_s(job_t* J) { TILE_LOOP_BODY(float, gets, 0.0f) }
static void run_d(job_t* J) { TILE_LOOP_BODY(double, getd, 0.0) }
static void run_c(job_t* J) { TILE_LOOP_BODY(cf, getc, (cf)0) }
static void run_z(job_t* J) { TILE_LOOP_BODY(cd, getz, (cd)0) }

static void* worker(void* p) {
  job_t* J = (job_t*)p;
  switch (J->dtype) {
    case TMMO_S: run_s(J); break;
    case TMMO_D: run_d(J); break;
    case TMMO_C: run_c(J); break;
    default: run_z(J); break;
  }
  return NULL;
}

/*
 * C = alpha * op(A) * op(B) + beta * C on the host, tile by tile, with the
 * reference's tile semantics.  Tiles (tm, tn, tk) are used as given (callers
 * apply tmmo_optimal_tile_sizes first to mirror the reference driver,
 * tiled_mm.cpp:557-560).  Returns 0, or -1 on invalid arguments (the
 * reference constructs but never throws these errors, tiled_mm.cpp:516-527).
 * nthreads splits the tile columns; results do not depend on it.
 */
int tmmo_gemm(int dtype, char trans_a, char trans_b, i64 m, i64 n, i64 k,
              const void* alpha, const void* a, i64 lda, const void* b, i64 ldb,
              const void* beta, void* c, i64 ldc, int copy_c_back, void* full_c,
              i64 tm, i64 tn, i64 tk, int nthreads) {
  int ta = upper(trans_a), tb = upper(trans_b);
  if ((ta != 'N' && ta != 'T' && ta != 'C') || (tb != 'N' && tb != 'T' && tb != 'C')) return -1;
  if (m < 0 || n < 0 || k < 0 || tm <= 0 || tn <= 0 || tk <= 0) return -1;
  if (dtype < TMMO_C) { /* conjugate transpose of a real matrix is its transpose */
    if (ta == 'C') ta = 'T';
    if (tb == 'C') tb = 'T';
  }
  i64 a_rows = ta == 'N' ? m : k, b_rows = tb == 'N' ? k : n;
  if (lda < (a_rows > 1 ? a_rows : 1) || ldb < (b_rows > 1 ? b_rows : 1) || ldc < (m > 1 ? m : 1)) return -1;
  if (m == 0 || n == 0) return 0;
  if (!copy_c_back && !full_c) return -1;
  i64 ntn = tmmo_num_tiles(n, tn);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > ntn) nthreads = (int)ntn;
  job_t base = {dtype, ta, tb, m, n, k, tm, tn, tk, alpha, beta, a, b, lda, ldb, c, ldc, copy_c_back, full_c, 0, 0};
  job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = base;
    jobs[t].j_begin = ntn * t / nthreads;
    jobs[t].j_end = ntn * (t + 1) / nthreads;
  }
  for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, worker, &jobs[t]);
  worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  return 0;
}

/* ---------------------------------------------------------------- double-double */

/* Ogita, Rump, Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput.
 * 26(6), 2005: TwoSum (Knuth) and TwoProduct via FMA; Dot2 accumulates the
 * product errors and the sum errors separately and adds them at the end. */
static inline void two_sum(double a, double b, double* s, double* e) {
  double x = a + b, z = x - a;
  *s = x;
  *e = (a - (x - z)) + (b - z);
}
static inline void two_prod(double a, double b, double* p, double* e) {
  double x = a * b;
  *p = x;
  *e = fma(a, b, -x);
}

/*
 * For each sample (ii[t], jj[t]) compute the correctly-rounded-ish (Dot2,
 * twice-working-precision) value of (alpha*op(A)*op(B) + beta*C0)(i, j) and the
 * magnitude |alpha| * sum_l |op(A)(i,l)| |op(B)(l,j)| + |beta| |C0(i,j)|, the
 * normaliser of the componentwise error metric  |C - C*| / (k u mag).
 * C0 is the input C (not read when beta == 0).
 */
void tmmo_dd_entries(char trans_a, char trans_b, i64 m, i64 n, i64 k, double alpha,
                     const double* a, i64 lda, const double* b, i64 ldb, double beta,
                     const double* c0, i64 ldc, i64 nsamp, const i64* ii, const i64* jj,
                     double* out, double* mag) {
  int ta = upper(trans_a), tb = upper(trans_b);
  if (ta == 'C') ta = 'T';
  if (tb == 'C') tb = 'T';
  (void)m; (void)n;
  for (i64 t = 0; t < nsamp; ++t) {
    i64 i = ii[t], j = jj[t];
    double s = 0, err = 0, am = 0;
    for (i64 l = 0; l < k; ++l) {
      double x = getd(a, lda, ta, i, l), y = getd(b, ldb, tb, l, j);
      double p, pe, s2, se;
      two_prod(x, y, &p, &pe);
      two_sum(s, p, &s2, &se);
      s = s2;
      err += pe + se;
      am += fabs(x) * fabs(y);
    }
    /* alpha * (s + err) + beta * c in the same compensated way */
    double hi, lo, p, pe;
    two_prod(alpha, s, &hi, &lo);
    lo += alpha * err;
    double mg = fabs(alpha) * am;
    if (beta != 0.0) {
      double cv = c0[i + j * ldc];
      two_prod(beta, cv, &p, &pe);
      double s2, se;
      two_sum(hi, p, &s2, &se);
      hi = s2;
      lo += se + pe;
      mg += fabs(beta) * fabs(cv);
    }
    out[t] = hi + lo;
    mag[t] = mg;
  }
}

/* max over samples of |x - ref| / (k * 2^-53 * mag); mag == 0 entries must be exact */
double tmmo_error_metric(i64 nsamp, const double* x, const double* ref, const double* mag, i64 k) {
  double u = 1.1102230246251565e-16, worst = 0;
  double kk = k > 0 ? (double)k : 1.0;
  for (i64 t = 0; t < nsamp; ++t) {
    double d = fabs(x[t] - ref[t]);
    if (d != d) return INFINITY; /* NaN */
    if (mag[t] == 0) {
      if (d != 0) return INFINITY;
      continue;
    }
    double r = d / (kk * u * mag[t]);
    if (r > worst) worst = r;
  }
  return worst;
}
