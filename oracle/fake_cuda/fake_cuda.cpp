// ORACLE test infrastructure: definitions behind oracle/fake_cuda/*.h.
//
// "Device" memory is host memory; every copy, event and BLAS call runs
// synchronously when issued.  The reference issues all work of one gemm call
// in an order that respects its own stream/event dependencies, so running it
// in issue order is one of the executions a GPU may produce.  A small trace
// (bytes per direction, per-tile GEMM calls) lets tests compare schedules.
#include "cuda_runtime_api.h"
#include "cublas_v2.h"

#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

namespace {
struct Trace {
  uint64_t h2d_bytes = 0, d2h_bytes = 0, gemm_calls = 0, gemm_flops = 0;
  uint64_t registers = 0, device_allocs = 0, device_alloc_bytes = 0;
};
Trace g_trace;
std::map<uintptr_t, size_t> g_registered;
std::map<uintptr_t, size_t> g_device;
std::mutex g_mu;

bool is_device(const void* p) {
  auto it = g_device.upper_bound((uintptr_t)p);
  if (it == g_device.begin()) return false;
  --it;
  return (uintptr_t)p < it->first + it->second;
}

void count(const void* dst, const void* src, size_t bytes) {
  bool d_dev = is_device(dst), s_dev = is_device(src);
  if (d_dev && !s_dev) g_trace.h2d_bytes += bytes;
  if (!d_dev && s_dev) g_trace.d2h_bytes += bytes;
}
}  // namespace

struct fake_stream { int id; };
struct fake_event { int id; };
struct fake_blas { cudaStream_t s; };

extern "C" {
void fake_trace_reset() { g_trace = Trace(); }
void fake_trace_get(uint64_t* out7) {
  out7[0] = g_trace.h2d_bytes;
  out7[1] = g_trace.d2h_bytes;
  out7[2] = g_trace.gemm_calls;
  out7[3] = g_trace.gemm_flops;
  out7[4] = g_trace.registers;
  out7[5] = g_trace.device_allocs;
  out7[6] = g_trace.device_alloc_bytes;
}
}

cudaError_t cudaHostRegister(void* ptr, size_t size, unsigned int) {
  std::lock_guard<std::mutex> l(g_mu);
  if (g_registered.count((uintptr_t)ptr)) return cudaErrorHostMemoryAlreadyRegistered;
  g_registered[(uintptr_t)ptr] = size;
  g_trace.registers++;
  return cudaSuccess;
}
cudaError_t cudaHostUnregister(void* ptr) {
  std::lock_guard<std::mutex> l(g_mu);
  if (!g_registered.erase((uintptr_t)ptr)) return cudaErrorHostMemoryNotRegistered;
  return cudaSuccess;
}
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned int) { *s = new fake_stream{0}; return cudaSuccess; }
cudaError_t cudaStreamDestroy(cudaStream_t s) { delete s; return cudaSuccess; }
cudaError_t cudaStreamWaitEvent(cudaStream_t, cudaEvent_t, unsigned int) { return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned int) { *e = new fake_event{0}; return cudaSuccess; }
cudaError_t cudaEventDestroy(cudaEvent_t e) { delete e; return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) { *ms = 0; return cudaSuccess; }
cudaError_t cudaMalloc(void** p, size_t size) {
  std::lock_guard<std::mutex> l(g_mu);
  void* q = nullptr;
  if (posix_memalign(&q, 256, size ? size : 1)) return cudaErrorMemoryAllocation;
  g_device[(uintptr_t)q] = size;
  g_trace.device_allocs++;
  g_trace.device_alloc_bytes += size;
  *p = q;
  return cudaSuccess;
}
cudaError_t cudaHostAlloc(void** p, size_t size, unsigned int) {
  void* q = nullptr;
  if (posix_memalign(&q, 256, size ? size : 1)) return cudaErrorMemoryAllocation;
  *p = q;
  return cudaSuccess;
}
cudaError_t cudaFree(void* p) {
  std::lock_guard<std::mutex> l(g_mu);
  g_device.erase((uintptr_t)p);
  free(p);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, enum cudaMemcpyKind) {
  count(dst, src, n);
  memmove(dst, src, n);
  return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t n, enum cudaMemcpyKind k, cudaStream_t) {
  return cudaMemcpy(dst, src, n, k);
}
cudaError_t cudaMemcpy2D(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                         size_t height, enum cudaMemcpyKind) {
  if (width > dpitch || width > spitch) return cudaErrorInvalidValue;
  for (size_t r = 0; r < height; ++r)
    memmove((char*)dst + r * dpitch, (const char*)src + r * spitch, width);
  count(dst, src, width * height);
  return cudaSuccess;
}
cudaError_t cudaMemcpy2DAsync(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                              size_t height, enum cudaMemcpyKind k, cudaStream_t) {
  return cudaMemcpy2D(dst, dpitch, src, spitch, width, height, k);
}
cudaError_t cudaGetDevice(int* d) { *d = 0; return cudaSuccess; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDeviceCount(int* n) { *n = 1; return cudaSuccess; }
cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t) { memset(p, v, n); return cudaSuccess; }
cudaError_t cudaPointerGetAttributes(struct cudaPointerAttributes* a, const void* p) {
  a->type = is_device(p) ? cudaMemoryTypeDevice : cudaMemoryTypeUnregistered;
  a->device = 0;
  a->devicePointer = (void*)p;
  a->hostPointer = (void*)p;
  return cudaSuccess;
}
cudaError_t cudaMemGetInfo(size_t* f, size_t* t) { *f = (size_t)1 << 40; *t = (size_t)1 << 40; return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "fake cuda error"; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }

// ---------------------------------------------------------------- BLAS
cublasStatus_t cublasCreate(cublasHandle_t* h) { *h = new fake_blas{nullptr}; return CUBLAS_STATUS_SUCCESS; }
cublasStatus_t cublasDestroy(cublasHandle_t h) { delete h; return CUBLAS_STATUS_SUCCESS; }
cublasStatus_t cublasSetStream(cublasHandle_t h, cudaStream_t s) { h->s = s; return CUBLAS_STATUS_SUCCESS; }

namespace {
template <typename T> T conj_if(T v, bool) { return v; }
template <typename R> std::complex<R> conj_if(std::complex<R> v, bool c) { return c ? std::conj(v) : v; }

// Plain column-major GEMM: for each column j, acc(i) = sum_l op(A)(i,l) op(B)(l,j)
// in increasing l; then C(i,j) = alpha*acc(i) + beta*C(i,j), or alpha*acc(i)
// when beta == 0 (C not read).
template <typename T>
cublasStatus_t gemm(cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k, T alpha,
                    const T* a, int lda, const T* b, int ldb, T beta, T* c, int ldc) {
  if (m < 0 || n < 0 || k < 0) return CUBLAS_STATUS_INVALID_VALUE;
  g_trace.gemm_calls++;
  g_trace.gemm_flops += 2ull * (uint64_t)m * (uint64_t)n * (uint64_t)k;
  T* ap = (T*)malloc(sizeof(T) * ((size_t)m * (size_t)k + 1));
  T* acc = (T*)malloc(sizeof(T) * ((size_t)m + 1));
  for (int l = 0; l < k; ++l)
    for (int i = 0; i < m; ++i)
      ap[i + (size_t)l * m] = ta == CUBLAS_OP_N ? a[i + (size_t)l * lda]
                                                : conj_if(a[l + (size_t)i * lda], ta == CUBLAS_OP_C);
  bool beta_nz = !(beta == T(0));
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < m; ++i) acc[i] = T(0);
    for (int l = 0; l < k; ++l) {
      T bv = tb == CUBLAS_OP_N ? b[l + (size_t)j * ldb] : conj_if(b[j + (size_t)l * ldb], tb == CUBLAS_OP_C);
      const T* col = ap + (size_t)l * m;
      for (int i = 0; i < m; ++i) acc[i] = acc[i] + col[i] * bv;
    }
    T* cc = c + (size_t)j * ldc;
    if (beta_nz)
      for (int i = 0; i < m; ++i) cc[i] = alpha * acc[i] + beta * cc[i];
    else
      for (int i = 0; i < m; ++i) cc[i] = alpha * acc[i];
  }
  free(ap);
  free(acc);
  return CUBLAS_STATUS_SUCCESS;
}
}  // namespace

cublasStatus_t cublasSgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const float* alpha, const float* a, int lda, const float* b, int ldb,
                           const float* beta, float* c, int ldc) {
  return gemm<float>(ta, tb, m, n, k, *alpha, a, lda, b, ldb, *beta, c, ldc);
}
cublasStatus_t cublasDgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const double* alpha, const double* a, int lda, const double* b, int ldb,
                           const double* beta, double* c, int ldc) {
  return gemm<double>(ta, tb, m, n, k, *alpha, a, lda, b, ldb, *beta, c, ldc);
}
cublasStatus_t cublasCgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const cuComplex* alpha, const cuComplex* a, int lda, const cuComplex* b, int ldb,
                           const cuComplex* beta, cuComplex* c, int ldc) {
  typedef std::complex<float> T;
  return gemm<T>(ta, tb, m, n, k, *(const T*)alpha, (const T*)a, lda, (const T*)b, ldb, *(const T*)beta,
                 (T*)c, ldc);
}
cublasStatus_t cublasZgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const cuDoubleComplex* alpha, const cuDoubleComplex* a, int lda,
                           const cuDoubleComplex* b, int ldb, const cuDoubleComplex* beta, cuDoubleComplex* c,
                           int ldc) {
  typedef std::complex<double> T;
  return gemm<T>(ta, tb, m, n, k, *(const T*)alpha, (const T*)a, lda, (const T*)b, ldb, *(const T*)beta,
                 (T*)c, ldc);
}
