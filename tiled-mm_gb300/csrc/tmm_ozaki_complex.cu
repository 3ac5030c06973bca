// Complex double GEMM on the Ozaki engine through the real embedding
//
//   [Re C]   [Re A  -Im A] [Re B]
//   [Im C] = [Im A   Re A] [Im B]        (op(A) m x k, op(B) k x n, complex)
//
// i.e. one real product of a 2m x 2k by a 2k x n matrix: 8mnk real flops, exactly the
// complex flop count, on the same split and slice-product kernels as the real path.  op
// 'C' conjugates while embedding.  A combine kernel applies the complex alpha and beta.
#include <cuda_runtime.h>

#include "tmm_ozaki.h"

namespace tmm {
namespace {

constexpr int TT = 32;  // transpose tile

// element (i, l) of op(X) for stored column-major complex X (interleaved re, im)
__device__ __forceinline__ double2 op_elem(const double2* __restrict__ X, int64_t ld, Op op, int64_t i, int64_t l) {
  if (op == OP_N) return X[i + l * ld];
  double2 v = X[l + i * ld];
  if (op == OP_C) v.y = -v.y;
  return v;
}

// Ahat (2m x 2k, ld 2m): [[re, -im], [im, re]] of op(A).  Transposed operands go through a
// shared-memory tile so that both the reads of A and the writes of Ahat are coalesced.
__global__ void embed_a_kernel(const double2* __restrict__ A, int64_t lda, Op op, int64_t m, int64_t k,
                               double* __restrict__ Ahat) {
  __shared__ double2 tile[TT][TT + 1];
  const int64_t i0 = (int64_t)blockIdx.x * TT, l0 = (int64_t)blockIdx.y * TT;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < TT; r += 8) {
    // op N: thread x runs along i (contiguous in A); op T / C: along l (contiguous in A)
    const int64_t i = op == OP_N ? i0 + tx : i0 + r, l = op == OP_N ? l0 + r : l0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (i < m && l < k) v = op_elem(A, lda, op, i, l);
    if (op == OP_N) tile[r][tx] = v;  // tile[l - l0][i - i0]
    else tile[tx][r] = v;
  }
  __syncthreads();
  const int64_t m2 = 2 * m;
  for (int r = ty; r < TT; r += 8) {
    const int64_t i = i0 + tx, l = l0 + r;
    if (i >= m || l >= k) continue;
    const double2 v = tile[r][tx];
    Ahat[i + l * m2] = v.x;            // top-left: Re A
    Ahat[(m + i) + l * m2] = v.y;      // bottom-left: Im A
    Ahat[i + (k + l) * m2] = -v.y;     // top-right: -Im A
    Ahat[(m + i) + (k + l) * m2] = v.x;  // bottom-right: Re A
  }
}

// Bhat (2k x n, ld 2k): [re; im] of op(B)
__global__ void embed_b_kernel(const double2* __restrict__ B, int64_t ldb, Op op, int64_t k, int64_t n,
                               double* __restrict__ Bhat) {
  __shared__ double2 tile[TT][TT + 1];
  const int64_t l0 = (int64_t)blockIdx.x * TT, j0 = (int64_t)blockIdx.y * TT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TT; r += 8) {
    // op N: B(l, j) contiguous along l; op T / C: B(j, l) contiguous along j
    const int64_t l = op == OP_N ? l0 + tx : l0 + r, j = op == OP_N ? j0 + r : j0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (l < k && j < n) v = op_elem(B, ldb, op, l, j);
    if (op == OP_N) tile[r][tx] = v;  // tile[j - j0][l - l0]
    else tile[tx][r] = v;
  }
  __syncthreads();
  const int64_t k2 = 2 * k;
  for (int r = ty; r < TT; r += 8) {
    const int64_t l = l0 + tx, j = j0 + r;
    if (l >= k || j >= n) continue;
    const double2 v = tile[r][tx];
    Bhat[l + j * k2] = v.x;
    Bhat[(k + l) + j * k2] = v.y;
  }
}

// C = alpha * (T_top + i T_bottom) + beta' * C; beta' == 0: C is not read
__global__ void combine_kernel(int64_t m, int64_t n, double2 alpha, double2 beta, int first, const double* __restrict__ T,
                               double2* __restrict__ C, int64_t ldc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= m || j >= n) return;
  const double tr = T[i + j * 2 * m], ti = T[m + i + j * 2 * m];
  double2 r;
  r.x = fma(alpha.x, tr, -alpha.y * ti);
  r.y = fma(alpha.x, ti, alpha.y * tr);
  double2* cp = C + i + j * ldc;
  if (!first) {
    const double2 c = *cp;
    r.x += c.x;
    r.y += c.y;
  } else if (beta.x != 0.0 || beta.y != 0.0) {
    const double2 c = *cp;
    r.x += fma(beta.x, c.x, -beta.y * c.y);
    r.y += fma(beta.x, c.y, beta.y * c.x);
  }
  *cp = r;
}

}  // namespace

cudaError_t ozaki_complex_embed(const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m,
                                int64_t n, int64_t k, double* Ahat, double* Bhat, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if ((k + TT - 1) / TT > 65535 || (n + TT - 1) / TT > 65535) return cudaErrorInvalidValue;  // grid y
  const dim3 block(TT, 8);
  embed_a_kernel<<<dim3((unsigned)((m + TT - 1) / TT), (unsigned)((k + TT - 1) / TT)), block, 0, s>>>(
      (const double2*)A, lda, opa, m, k, Ahat);
  embed_b_kernel<<<dim3((unsigned)((k + TT - 1) / TT), (unsigned)((n + TT - 1) / TT)), block, 0, s>>>(
      (const double2*)B, ldb, opb, k, n, Bhat);
  return cudaGetLastError();
}

cudaError_t ozaki_complex_combine(int64_t m, int64_t n, const double* alpha, const double* beta, bool first,
                                  const double* T, void* C, int64_t ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  if (n > 65535) {  // grid y is 16-bit: column panels
    for (int64_t j0 = 0; j0 < n; j0 += 65535) {
      const int64_t nn = n - j0 < 65535 ? n - j0 : 65535;
      cudaError_t e = ozaki_complex_combine(m, nn, alpha, beta, first, T + j0 * 2 * m,
                                            (double2*)C + j0 * ldc, ldc, s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  combine_kernel<<<dim3((unsigned)((m + 255) / 256), (unsigned)n), 256, 0, s>>>(
      m, n, make_double2(alpha[0], alpha[1]), make_double2(beta[0], beta[1]), first ? 1 : 0, T, (double2*)C, ldc);
  return cudaGetLastError();
}

}  // namespace tmm
