// The compiled half of the drop-in C++ API and the C-ABI entries behind its
// stream, event and device-buffer classes.
//
// As in the reference (src/Tiled-MM/tiled_mm.cpp:626-668), gpu::gemm is a
// template declared in <Tiled-MM/tiled_mm.hpp> and defined here, with explicit
// instantiations for the four scalar types, so that programs link against this
// library exactly as they link against the reference's.
#include <cuda_runtime.h>

#include <complex>
#include <string>

#include "../../include/Tiled-MM/tiled_mm.hpp"
#include "tmm_context.h"

namespace {

int bad(tmm_context* ctx, const char* msg) {
  if (ctx) ctx->last_error = msg;
  return TMM_ERROR_INVALID_ARGUMENT;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return TMM_SUCCESS;
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? TMM_ERROR_OUT_OF_MEMORY : TMM_ERROR_CUDA;
}

}  // namespace

extern "C" int tmm_get_stream(tmm_context* ctx, int stream_id, void** stream) {
  if (!ctx || !stream) return bad(ctx, "tmm_get_stream: null argument");
  if (stream_id < 0 || stream_id >= (int)ctx->streams.size())
    return bad(ctx, "tmm_get_stream: stream id has to be in the range [0, n_streams)");
  *stream = (void*)ctx->streams[(size_t)stream_id];
  return TMM_SUCCESS;
}

extern "C" int tmm_get_result_stream(tmm_context* ctx, void** stream) {
  if (!ctx || !stream) return bad(ctx, "tmm_get_result_stream: null argument");
  *stream = (void*)ctx->d2h;
  return TMM_SUCCESS;
}

extern "C" int tmm_get_device_buffer(tmm_context* ctx, char which, int stream_id, void** ptr) {
  if (!ctx || !ptr) return bad(ctx, "tmm_get_device_buffer: null argument");
  *ptr = nullptr;
  switch (which) {
    case 'a': case 'A':
    case 'b': case 'B': {
      const bool is_a = which == 'a' || which == 'A';
      const tmm::TileCache& cache = is_a ? ctx->cache_a : ctx->cache_b;
      const tmm::GrowBuffer& pool = is_a ? ctx->pool_a : ctx->pool_b;
      if (stream_id < 0) *ptr = pool.ptr;
      else if ((size_t)stream_id < cache.slots.size()) *ptr = cache.slots[(size_t)stream_id].ptr;
      return TMM_SUCCESS;
    }
    case 'c': case 'C':
      if (stream_id < 0) *ptr = ctx->pool_c.ptr;
      else if ((size_t)stream_id * 2 < ctx->cslots.size()) *ptr = ctx->cslots[(size_t)stream_id * 2].ptr;
      return TMM_SUCCESS;
    default:
      return bad(ctx, "tmm_get_device_buffer: which must be 'a', 'b' or 'c'");
  }
}

extern "C" int tmm_stream_create(void** stream) {
  if (!stream) return TMM_ERROR_INVALID_ARGUMENT;
  cudaStream_t s = nullptr;
  const int st = cuda_status(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = st == TMM_SUCCESS ? (void*)s : nullptr;
  return st;
}

extern "C" int tmm_stream_destroy(void* stream) {
  return stream ? cuda_status(cudaStreamDestroy((cudaStream_t)stream)) : TMM_SUCCESS;
}

extern "C" int tmm_event_create(void** event) {
  if (!event) return TMM_ERROR_INVALID_ARGUMENT;
  cudaEvent_t e = nullptr;
  const int st = cuda_status(cudaEventCreate(&e));
  *event = st == TMM_SUCCESS ? (void*)e : nullptr;
  return st;
}

extern "C" int tmm_event_destroy(void* event) {
  return event ? cuda_status(cudaEventDestroy((cudaEvent_t)event)) : TMM_SUCCESS;
}

extern "C" int tmm_event_record(void* event, void* stream) {
  if (!event) return TMM_ERROR_INVALID_ARGUMENT;
  return cuda_status(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream));
}

extern "C" int tmm_event_synchronize(void* event) {
  if (!event) return TMM_ERROR_INVALID_ARGUMENT;
  return cuda_status(cudaEventSynchronize((cudaEvent_t)event));
}

extern "C" int tmm_event_elapsed(void* start, void* end, double* seconds) {
  if (!start || !end || !seconds) return TMM_ERROR_INVALID_ARGUMENT;
  float ms = 0.0f;
  const int st = cuda_status(cudaEventElapsedTime(&ms, (cudaEvent_t)start, (cudaEvent_t)end));
  *seconds = 1e-3 * (double)ms;
  return st;
}

extern "C" int tmm_stream_wait_event(void* stream, void* event) {
  if (!event) return TMM_ERROR_INVALID_ARGUMENT;
  return cuda_status(cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)event, 0));
}

namespace gpu {

// tiled_mm.cpp:492-624: the whole call is the C-ABI tmm_gemm on the handle's context
template <typename Scalar>
void gemm(mm_handle<Scalar>& handle, char trans_a, char trans_b, int m, int n, int k, Scalar alpha, Scalar* a,
          int ld_a, Scalar* b, int ld_b, Scalar beta, Scalar* c, int ld_c, bool pin_host_buffers, bool copy_c_back) {
  const int st = tmm_gemm(handle.native(), trans_a, trans_b, m, n, k, &alpha, a, ld_a, b, ld_b, &beta, c, ld_c,
                          pin_host_buffers ? 1 : 0, copy_c_back ? 1 : 0);
  check_tmm_status(st, handle.native());
  handle.after_gemm();
}

template void gemm<float>(mm_handle<float>&, char, char, int, int, int, float, float*, int, float*, int, float, float*,
                          int, bool, bool);
template void gemm<double>(mm_handle<double>&, char, char, int, int, int, double, double*, int, double*, int, double,
                           double*, int, bool, bool);
template void gemm<std::complex<float>>(mm_handle<std::complex<float>>&, char, char, int, int, int,
                                        std::complex<float>, std::complex<float>*, int, std::complex<float>*, int,
                                        std::complex<float>, std::complex<float>*, int, bool, bool);
template void gemm<std::complex<double>>(mm_handle<std::complex<double>>&, char, char, int, int, int,
                                         std::complex<double>, std::complex<double>*, int, std::complex<double>*, int,
                                         std::complex<double>, std::complex<double>*, int, bool, bool);

}  // namespace gpu
