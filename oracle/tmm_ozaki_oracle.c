/*
 * ORACLE — test infrastructure only (see tmm_oracle.c for the rules).
 *
 * CPU restatement of the Ozaki split-precision FP64 GEMM that the GPU path
 * runs.  The reference has no counterpart (it calls cublasDgemm per tile,
 * src/Tiled-MM/tiled_mm.cpp:200-217); the algorithm is the published
 * error-free splitting of Ozaki, Ogita, Oishi and Rump, "Error-free
 * transformations of matrix multiplication by using fast routines of matrix
 * multiplication and its applications", Numer. Algorithms 59 (2012), with
 * integer slices as in Mukunoki, Ozaki, Ogita and Imamura, "DGEMM using
 * tensor cores, and its accurate and reproducible versions", ISC 2020, and
 * Ootomo, Ozaki and Yokota, "DGEMM on integer matrix multiplication unit",
 * IJHPCA 2024.  Every step here is the one the GPU performs, in the same
 * order, so the two agree bit for bit whenever the GPU's low-precision
 * products are exact (they are integers below 2^24 by construction):
 *
 *  1. scale: for row i of op(A) (column j of op(B)) over the tile's k range,
 *     e = frexp exponent of the largest magnitude (2^(e-1) <= max < 2^e);
 *     an all-zero line has e = 0 and zero digits.
 *  2. split: x = v * 2^-e in (-1, 1);  t = x * D with D = 2^(w-1);
 *     for p = 0..s-1:  d_p = rint(t);  t = (t - d_p) * 2^w.
 *     Every step is exact in FP64 and |d_p| <= D, so v ~= 2^e * D^-1 *
 *     sum_p d_p 2^(-w p) with |error| <= 2^(e - w s) per element.
 *     (w = digit width in bits: 5 for e4m3 slices, 8 for bf16 slices.)
 *  3. multiply: for each group g = s-1 down to 0 and every slice pair
 *     (p, q = g - p), p ascending, the exact integer products of the digit
 *     planes over the tile's k, accumulated in passes of at most
 *     pass_blocks k-blocks of kb elements (a pass never spans two groups);
 *     after each pass:  acc = acc + 2^(-w g) * S_pass   (one FP64 rounding).
 *  4. epilogue: t = acc * 2^(e_i + f_j - 2(w-1));
 *     (a line holding an Inf or a NaN gets exponent 1025 and no digits; the product's
 *     entries in its row or column are NaN)
 *     C = fma(alpha, t, beta * C)   (k-tile 0, C not read when beta == 0)
 *     C = fma(alpha, t, C)          (later k-tiles: beta' = 1)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;

static int up(char c) { return (c >= 'a' && c <= 'z') ? c - 32 : c; }

static inline double at(const double* x, i64 ld, int op, i64 r, i64 c) {
  return op == 'N' ? x[r + c * ld] : x[c + r * ld];
}

/* frexp exponent of the largest magnitude of a line (0 for an all-zero line) */
static int line_exponent(double amax) {
  if (amax == 0.0) return 0;
  int e;
  frexp(amax, &e);
  return e;
}

/*
 * Split rows of op(X) (rows x kk, op(X)(r, l)) into s digit planes
 * digits[p * rows * kpad + r * kpad + l] (int8, l < kk; zero padding up to
 * kpad) and exponents exps[r].  For B pass op = transpose of op(B), i.e. the
 * caller supplies the accessor orientation through (x, ld, op) such that
 * element (r, l) is the r-th line's l-th entry along k.
 */
void tmmo_ozaki_split(const double* x, i64 ld, char op, i64 rows, i64 kk, i64 kpad, int s, int w,
                      int8_t* digits, int32_t* exps) {
  int o = up(op);
  if (o == 'C') o = 'T';
  double D = ldexp(1.0, w - 1), W = ldexp(1.0, w);
  memset(digits, 0, (size_t)s * (size_t)rows * (size_t)kpad);
  for (i64 r = 0; r < rows; ++r) {
    double amax = 0;
    int nonfinite = 0;
    for (i64 l = 0; l < kk; ++l) {
      double v = fabs(at(x, ld, o, r, l));
      if (!isfinite(v)) nonfinite = 1;
      else if (v > amax) amax = v;
    }
    /* a line holding an Inf or a NaN: exponent 1025 (above every finite line exponent), no
     * digits; its row or column of the product is NaN */
    int e = nonfinite ? 1025 : line_exponent(amax);
    exps[r] = e;
    if (amax == 0.0 || nonfinite) continue;
    for (i64 l = 0; l < kk; ++l) {
      double t = ldexp(at(x, ld, o, r, l), -e) * D;
      for (int p = 0; p < s; ++p) {
        double d = rint(t);
        digits[(size_t)p * rows * kpad + (size_t)r * kpad + l] = (int8_t)d;
        t = (t - d) * W;
      }
    }
  }
}

/*
 * The slice-product GEMM plus epilogue on split operands:
 *   ad [s][m][kpad], ea[m]  (rows of op(A))
 *   bd [s][n][kpad], eb[n]  (columns of op(B), stored as lines along k)
 * C (m x n, ldc) is updated in place: first_k_tile selects beta (else 1).
 * kb = k elements per k-block; pass_blocks = k-blocks per exact FP32 pass.
 * nslices_used: pairs with p + q <= s-1 (triangular truncation).
 */
void tmmo_ozaki_gemm_split(i64 m, i64 n, i64 kpad, int s, int w, const int8_t* ad, const int32_t* ea,
                           const int8_t* bd, const int32_t* eb, double alpha, double beta,
                           int first_k_tile, double* c, i64 ldc, i64 kb, i64 pass_blocks) {
  i64 nkb = kpad / kb;
  int64_t* part = (int64_t*)malloc(sizeof(int64_t) * (size_t)s * (size_t)s * (size_t)nkb);
  for (i64 i = 0; i < m; ++i) {
    for (i64 j = 0; j < n; ++j) {
      /* exact integer dot products of every pair over every k-block */
      for (int p = 0; p < s; ++p)
        for (int q = 0; q + p < s; ++q) {
          const int8_t* ar = ad + (size_t)p * m * kpad + (size_t)i * kpad;
          const int8_t* br = bd + (size_t)q * n * kpad + (size_t)j * kpad;
          for (i64 b = 0; b < nkb; ++b) {
            int64_t acc = 0;
            for (i64 l = b * kb; l < (b + 1) * kb; ++l) acc += (int64_t)ar[l] * (int64_t)br[l];
            part[((size_t)p * s + q) * nkb + b] = acc;
          }
        }
      double acc = 0.0;
      for (int g = s - 1; g >= 0; --g) {
        double wg = ldexp(1.0, -w * g);
        int64_t pass = 0;
        i64 used = 0;
        for (int p = 0; p <= g; ++p) {
          int q = g - p;
          for (i64 b = 0; b < nkb; ++b) {
            pass += part[((size_t)p * s + q) * nkb + b];
            if (++used == pass_blocks) {
              acc = acc + wg * (double)pass;
              pass = 0;
              used = 0;
            }
          }
        }
        if (used > 0) acc = acc + wg * (double)pass;
      }
      double t = ldexp(acc, ea[i] + eb[j] - 2 * (w - 1));
      double* cp = c + i + j * ldc;
      if (ea[i] >= 1025 || eb[j] >= 1025)
        *cp = NAN;
      else if (!first_k_tile)
        *cp = fma(alpha, t, *cp);
      else if (beta != 0.0)
        *cp = fma(alpha, t, beta * *cp);
      else
        *cp = alpha * t;
    }
  }
  free(part);
}

/*
 * Whole Ozaki GEMM on host operands, k cut into tiles of tk (per-k-tile
 * scaling, exactly as the out-of-core schedule does):  C = alpha op(A) op(B) + beta C.
 */
int tmmo_ozaki_gemm(char trans_a, char trans_b, i64 m, i64 n, i64 k, double alpha, const double* a, i64 lda,
                    const double* b, i64 ldb, double beta, double* c, i64 ldc, int s, int w, i64 tk, i64 kb,
                    i64 pass_blocks) {
  int ta = up(trans_a), tb = up(trans_b);
  if (ta == 'C') ta = 'T';
  if (tb == 'C') tb = 'T';
  if (tk <= 0 || kb <= 0 || s <= 0) return -1;
  if (k == 0) {
    for (i64 j = 0; j < n; ++j)
      for (i64 i = 0; i < m; ++i) c[i + j * ldc] = beta != 0.0 ? beta * c[i + j * ldc] : 0.0;
    return 0;
  }
  for (i64 k0 = 0, kt = 0; k0 < k; k0 += tk, ++kt) {
    i64 kk = (k - k0) < tk ? (k - k0) : tk;
    /* k is padded to whole 128-byte k-blocks, as the GPU split does */
    i64 kal = kb > 128 ? kb : 128;
    i64 kpad = (kk + kal - 1) / kal * kal;
    int8_t* ad = (int8_t*)malloc((size_t)s * m * kpad);
    int8_t* bd = (int8_t*)malloc((size_t)s * n * kpad);
    int32_t* ea = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
    int32_t* eb = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    /* rows of op(A) restricted to columns k0..k0+kk: shift the base pointer */
    const double* abase = ta == 'N' ? a + k0 * lda : a + k0;
    tmmo_ozaki_split(abase, lda, (char)ta, m, kk, kpad, s, w, ad, ea);
    /* columns of op(B) as lines along k: element (j, l) = op(B)(l, j) */
    const double* bbase = tb == 'N' ? b + k0 : b + k0 * ldb;
    tmmo_ozaki_split(bbase, ldb, tb == 'N' ? 'T' : 'N', n, kk, kpad, s, w, bd, eb);
    tmmo_ozaki_gemm_split(m, n, kpad, s, w, ad, ea, bd, eb, alpha, beta, kt == 0, c, ldc, kb, pass_blocks);
    free(ad); free(bd); free(ea); free(eb);
  }
  return 0;
}
