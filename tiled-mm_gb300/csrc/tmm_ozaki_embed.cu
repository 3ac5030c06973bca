// Float, complex float and complex double GEMMs on the Ozaki engine, which multiplies real
// FP64 matrices.  Each operand is embedded into a real FP64 matrix:
//
//   real float:    Ahat = op(A) (m x k),  Bhat = op(B) (k x n), converted exactly
//   complex:       [Re C]   [Re A  -Im A] [Re B]
//                  [Im C] = [Im A   Re A] [Im B]     Ahat 2m x 2k, Bhat 2k x n
//
// so that the real product T = Ahat Bhat holds the result (for complex: Re C on top of
// Im C; 8mnk real flops, exactly the complex flop count), and op 'C' conjugates while
// embedding.  A combine kernel applies alpha and beta and rounds once to the output type.
#include <cuda_runtime.h>

#include "tmm_f32tc.h"
#include "tmm_ozaki.h"

namespace tmm {
namespace {

constexpr int TT = 32;  // transpose tile

// element (i, l) of op(X) for stored column-major X, as (re, im) in double
template <typename T>
__device__ __forceinline__ double2 ld_op(const T* __restrict__ X, int64_t ld, Op op, int64_t i, int64_t l);
template <>
__device__ __forceinline__ double2 ld_op<float>(const float* __restrict__ X, int64_t ld, Op op, int64_t i, int64_t l) {
  return make_double2((double)(op == OP_N ? X[i + l * ld] : X[l + i * ld]), 0.0);
}
template <>
__device__ __forceinline__ double2 ld_op<float2>(const float2* __restrict__ X, int64_t ld, Op op, int64_t i,
                                                 int64_t l) {
  const float2 v = op == OP_N ? X[i + l * ld] : X[l + i * ld];
  return make_double2((double)v.x, op == OP_C ? -(double)v.y : (double)v.y);
}
template <>
__device__ __forceinline__ double2 ld_op<double2>(const double2* __restrict__ X, int64_t ld, Op op, int64_t i,
                                                  int64_t l) {
  double2 v = op == OP_N ? X[i + l * ld] : X[l + i * ld];
  if (op == OP_C) v.y = -v.y;
  return v;
}

template <typename T>
constexpr bool is_complex() {
  return sizeof(T) != sizeof(float);
}

// Ahat of op(A) (m x k).  Transposed operands go through a shared-memory tile so that
// both the reads of A and the writes of Ahat are coalesced.
template <typename T, typename O = double>
__global__ void embed_a_kernel(const T* __restrict__ A, int64_t lda, Op op, int64_t m, int64_t k,
                               O* __restrict__ Ahat) {
  __shared__ double2 tile[TT][TT + 1];
  const int64_t i0 = (int64_t)blockIdx.x * TT, l0 = (int64_t)blockIdx.y * TT;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < TT; r += 8) {
    // op N: thread x runs along i (contiguous in A); op T / C: along l (contiguous in A)
    const int64_t i = op == OP_N ? i0 + tx : i0 + r, l = op == OP_N ? l0 + r : l0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (i < m && l < k) v = ld_op<T>(A, lda, op, i, l);
    if (op == OP_N) tile[r][tx] = v;  // tile[l - l0][i - i0]
    else tile[tx][r] = v;
  }
  __syncthreads();
  const int64_t mm = is_complex<T>() ? 2 * m : m;
  for (int r = ty; r < TT; r += 8) {
    const int64_t i = i0 + tx, l = l0 + r;
    if (i >= m || l >= k) continue;
    const double2 v = tile[r][tx];
    Ahat[i + l * mm] = (O)v.x;  // (top-left): Re A
    if (is_complex<T>()) {
      Ahat[(m + i) + l * mm] = (O)v.y;        // bottom-left: Im A
      Ahat[i + (k + l) * mm] = (O)-v.y;       // top-right: -Im A
      Ahat[(m + i) + (k + l) * mm] = (O)v.x;  // bottom-right: Re A
    }
  }
}

// Bhat of op(B) (k x n): op(B) itself, or [Re; Im] for complex
template <typename T, typename O = double>
__global__ void embed_b_kernel(const T* __restrict__ B, int64_t ldb, Op op, int64_t k, int64_t n,
                               O* __restrict__ Bhat) {
  __shared__ double2 tile[TT][TT + 1];
  const int64_t l0 = (int64_t)blockIdx.x * TT, j0 = (int64_t)blockIdx.y * TT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TT; r += 8) {
    // op N: B(l, j) contiguous along l; op T / C: B(j, l) contiguous along j
    const int64_t l = op == OP_N ? l0 + tx : l0 + r, j = op == OP_N ? j0 + r : j0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (l < k && j < n) v = ld_op<T>(B, ldb, op, l, j);
    if (op == OP_N) tile[r][tx] = v;  // tile[j - j0][l - l0]
    else tile[tx][r] = v;
  }
  __syncthreads();
  const int64_t kk = is_complex<T>() ? 2 * k : k;
  for (int r = ty; r < TT; r += 8) {
    const int64_t l = l0 + tx, j = j0 + r;
    if (l >= k || j >= n) continue;
    const double2 v = tile[r][tx];
    Bhat[l + j * kk] = (O)v.x;
    if (is_complex<T>()) Bhat[(k + l) + j * kk] = (O)v.y;
  }
}

template <typename T>
__device__ __forceinline__ double2 ld_c(const T* p);
template <>
__device__ __forceinline__ double2 ld_c<float>(const float* p) {
  return make_double2((double)*p, 0.0);
}
template <>
__device__ __forceinline__ double2 ld_c<float2>(const float2* p) {
  return make_double2((double)p->x, (double)p->y);
}
template <>
__device__ __forceinline__ double2 ld_c<double2>(const double2* p) {
  return *p;
}
template <typename T>
__device__ __forceinline__ void st_c(T* p, double2 v);
template <>
__device__ __forceinline__ void st_c<float>(float* p, double2 v) {
  *p = (float)v.x;
}
template <>
__device__ __forceinline__ void st_c<float2>(float2* p, double2 v) {
  *p = make_float2((float)v.x, (float)v.y);
}
template <>
__device__ __forceinline__ void st_c<double2>(double2* p, double2 v) {
  *p = v;
}

// C = alpha * T + beta' * C, computed in double and rounded once to the output type;
// beta' == 0 on the first k tile: C is not read.  Real: fma(alpha, t, beta c) / alpha t /
// fma(alpha, t, c), as the real engine's epilogue.  Complex: the products of alpha and
// beta with a complex value each take one fma per component.
template <typename T, typename TE = double>
__global__ void combine_kernel(int64_t m, int64_t n, double2 alpha, double2 beta, int first,
                               const TE* __restrict__ Tm, T* __restrict__ C, int64_t ldc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= m || j >= n) return;
  T* cp = C + i + j * ldc;
  if (!is_complex<T>()) {
    const double t = (double)Tm[i + j * m];
    double r;
    if (!first) r = fma(alpha.x, t, ld_c<T>(cp).x);
    else if (beta.x != 0.0) r = fma(alpha.x, t, beta.x * ld_c<T>(cp).x);
    else r = alpha.x * t;
    st_c<T>(cp, make_double2(r, 0.0));
    return;
  }
  const double tr = (double)Tm[i + j * 2 * m], ti = (double)Tm[m + i + j * 2 * m];
  double2 r;
  r.x = fma(alpha.x, tr, -alpha.y * ti);
  r.y = fma(alpha.x, ti, alpha.y * tr);
  if (!first) {
    const double2 c = ld_c<T>(cp);
    r.x += c.x;
    r.y += c.y;
  } else if (beta.x != 0.0 || beta.y != 0.0) {
    const double2 c = ld_c<T>(cp);
    r.x += fma(beta.x, c.x, -beta.y * c.y);
    r.y += fma(beta.x, c.y, beta.y * c.x);
  }
  st_c<T>(cp, r);
}

template <typename T>
cudaError_t embed_t(const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m, int64_t n,
                    int64_t k, double* Ahat, double* Bhat, cudaStream_t s) {
  const dim3 block(TT, 8);
  embed_a_kernel<T><<<dim3((unsigned)((m + TT - 1) / TT), (unsigned)((k + TT - 1) / TT)), block, 0, s>>>(
      (const T*)A, lda, opa, m, k, Ahat);
  embed_b_kernel<T><<<dim3((unsigned)((k + TT - 1) / TT), (unsigned)((n + TT - 1) / TT)), block, 0, s>>>(
      (const T*)B, ldb, opb, k, n, Bhat);
  return cudaGetLastError();
}

template <typename T>
cudaError_t combine_t(int64_t m, int64_t n, double2 alpha, double2 beta, bool first, const double* Tm, void* C,
                      int64_t ldc, cudaStream_t s) {
  const int64_t mm = is_complex<T>() ? 2 * m : m;
  for (int64_t j0 = 0; j0 < n; j0 += 65535) {  // grid y is 16-bit: column panels
    const int64_t nn = n - j0 < 65535 ? n - j0 : 65535;
    combine_kernel<T><<<dim3((unsigned)((m + 255) / 256), (unsigned)nn), 256, 0, s>>>(
        m, nn, alpha, beta, first ? 1 : 0, Tm + j0 * mm, (T*)C + j0 * ldc, ldc);
  }
  return cudaGetLastError();
}

}  // namespace

// Complex float on the FP32 tensor-core engine: the same real embedding in float (exact), and
// C = alpha * T + beta * C from the engine's float product T (2m x n: Re C over Im C),
// computed in double and rounded once to complex float.
cudaError_t cplx_f32_embed(const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m,
                           int64_t n, int64_t k, float* Ahat, float* Bhat, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if ((k + TT - 1) / TT > 65535 || (n + TT - 1) / TT > 65535) return cudaErrorInvalidValue;  // grid y
  const dim3 block(TT, 8);
  embed_a_kernel<float2, float><<<dim3((unsigned)((m + TT - 1) / TT), (unsigned)((k + TT - 1) / TT)), block, 0, s>>>(
      (const float2*)A, lda, opa, m, k, Ahat);
  embed_b_kernel<float2, float><<<dim3((unsigned)((k + TT - 1) / TT), (unsigned)((n + TT - 1) / TT)), block, 0, s>>>(
      (const float2*)B, ldb, opb, k, n, Bhat);
  return cudaGetLastError();
}

cudaError_t cplx_f32_combine(int64_t m, int64_t n, const void* alpha, const void* beta, const float* Tm, void* C,
                             int64_t ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  const double2 al = make_double2((double)((const float*)alpha)[0], (double)((const float*)alpha)[1]);
  const double2 be = make_double2((double)((const float*)beta)[0], (double)((const float*)beta)[1]);
  for (int64_t j0 = 0; j0 < n; j0 += 65535) {  // grid y is 16-bit: column panels
    const int64_t nn = n - j0 < 65535 ? n - j0 : 65535;
    combine_kernel<float2, float><<<dim3((unsigned)((m + 255) / 256), (unsigned)nn), 256, 0, s>>>(
        m, nn, al, be, 1, Tm + j0 * 2 * m, (float2*)C + j0 * ldc, ldc);
  }
  return cudaGetLastError();
}

bool ozaki_embedded_dtype(int dtype) {
  return dtype == TMM_FLOAT || dtype == TMM_COMPLEX_FLOAT || dtype == TMM_COMPLEX_DOUBLE;
}

cudaError_t ozaki_embed(int dtype, const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m,
                        int64_t n, int64_t k, double* Ahat, double* Bhat, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if ((k + TT - 1) / TT > 65535 || (n + TT - 1) / TT > 65535) return cudaErrorInvalidValue;  // grid y
  switch (dtype) {
    case TMM_FLOAT: return embed_t<float>(A, lda, opa, B, ldb, opb, m, n, k, Ahat, Bhat, s);
    case TMM_COMPLEX_FLOAT: return embed_t<float2>(A, lda, opa, B, ldb, opb, m, n, k, Ahat, Bhat, s);
    case TMM_COMPLEX_DOUBLE: return embed_t<double2>(A, lda, opa, B, ldb, opb, m, n, k, Ahat, Bhat, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t ozaki_combine(int dtype, int64_t m, int64_t n, const void* alpha, const void* beta, bool first,
                          const double* Tm, void* C, int64_t ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  double2 al, be;
  switch (dtype) {
    case TMM_FLOAT:
      al = make_double2((double)*(const float*)alpha, 0.0);
      be = make_double2((double)*(const float*)beta, 0.0);
      return combine_t<float>(m, n, al, be, first, Tm, C, ldc, s);
    case TMM_COMPLEX_FLOAT:
      al = make_double2((double)((const float*)alpha)[0], (double)((const float*)alpha)[1]);
      be = make_double2((double)((const float*)beta)[0], (double)((const float*)beta)[1]);
      return combine_t<float2>(m, n, al, be, first, Tm, C, ldc, s);
    case TMM_COMPLEX_DOUBLE:
      al = make_double2(((const double*)alpha)[0], ((const double*)alpha)[1]);
      be = make_double2(((const double*)beta)[0], ((const double*)beta)[1]);
      return combine_t<double2>(m, n, al, be, first, Tm, C, ldc, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace tmm
