// Host side of the C ABI: context, tile policy, tile cache and the
// C-stationary stream pipeline that replaces the reference's round-robin
// schedules (src/Tiled-MM/tiled_mm.cpp:270-454) and driver
// (src/Tiled-MM/tiled_mm.cpp:492-624).
//
// Schedule.  C tiles are visited row panel by row panel (the reference's
// row-major tile order, tiled_mm.cpp:300-301), with the column order
// reversed on every other panel so the B tiles used last are used first
// again.  A C tile stays on one compute stream for its whole k loop (beta on
// k-tile 0, 1 afterwards: tiled_mm.cpp:309, 402).  A and B tiles live in two
// device tile caches (LRU); a tile is copied to the device once and reused
// by every C tile that needs it while it stays resident, so with enough HBM
// each operand crosses the host link exactly once (the reference re-sends A
// n_tiles_n times and B n_tiles_m times).  Copies run on their own stream and
// are ordered against compute with events only; each compute stream owns two
// C tile slots, so the copy-back of one tile overlaps the next tile's k loop.
#include <algorithm>
#include <numeric>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>

#include "tmm_context.h"
#include "tmm_f32tc.h"
#include "tmm_kernels.h"
#include "tmm_ozaki.h"
#include "tmm_datagen.h"
#include "tmm_batched.h"

using tmm::Op;

namespace {

thread_local std::string g_last_error = "no error";

int fail(tmm_context* ctx, int status, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  g_last_error = msg;
  return status;
}

int cuda_fail(tmm_context* ctx, cudaError_t e, const char* what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(ctx, e == cudaErrorMemoryAllocation ? TMM_ERROR_OUT_OF_MEMORY : TMM_ERROR_CUDA, msg);
}

#define TMM_CUDA(ctx, call)                                        \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);     \
  } while (0)

size_t elem_size(int dtype) {
  switch (dtype) {
    case TMM_FLOAT: return 4;
    case TMM_DOUBLE: return 8;
    case TMM_COMPLEX_FLOAT: return 8;
    default: return 16;
  }
}

bool is_zero(int dtype, const void* v) {
  switch (dtype) {
    case TMM_FLOAT: return *(const float*)v == 0.f;
    case TMM_DOUBLE: return *(const double*)v == 0.0;
    case TMM_COMPLEX_FLOAT: return ((const float*)v)[0] == 0.f && ((const float*)v)[1] == 0.f;
    default: return ((const double*)v)[0] == 0.0 && ((const double*)v)[1] == 0.0;
  }
}

int upper(char c) { return (c >= 'a' && c <= 'z') ? c - 32 : c; }

bool parse_op(char c, int dtype, Op* op) {
  switch (upper(c)) {
    case 'N': *op = tmm::OP_N; return true;
    case 'T': *op = tmm::OP_T; return true;
    case 'C': *op = (dtype == TMM_COMPLEX_FLOAT || dtype == TMM_COMPLEX_DOUBLE) ? tmm::OP_C : tmm::OP_T; return true;
    default: return false;
  }
}

// The reference's tile policy (src/Tiled-MM/mm_handle.cpp:89-110).
int optimal_tile_size(int64_t dim, int curr, int max_tile) {
  if (curr < max_tile && dim <= max_tile) return (int)dim;
  int64_t limit = std::min<int64_t>(max_tile, dim);
  int64_t tile = 1;
  for (int64_t i = 1; i <= limit; ++i)
    if (dim % i == 0) tile = i;
  if (std::llabs((int64_t)max_tile - tile) <= max_tile / 2) return (int)tile;
  return (int)limit;
}

// restores the caller's current device on scope exit
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    else prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Brackets one engine launch with a pair of events on its stream when kernel timing is on.
struct KernelTimer {
  tmm_context* ctx;
  cudaStream_t s;
  std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
  KernelTimer(tmm_context* c, cudaStream_t st) : ctx(c), s(st) {
    if (!ctx->ktime) return;
    if (!ctx->kt_free.empty()) {
      ev = ctx->kt_free.back();
      ctx->kt_free.pop_back();
    } else {
      if (cudaEventCreate(&ev.first) != cudaSuccess) {
        ev = {nullptr, nullptr};
        return;
      }
      if (cudaEventCreate(&ev.second) != cudaSuccess) {
        cudaEventDestroy(ev.first);
        ev = {nullptr, nullptr};
        return;
      }
    }
    cudaEventRecord(ev.first, s);
  }
  void done() {
    if (!ev.first) return;
    cudaEventRecord(ev.second, s);
    ctx->kt_pending.push_back(ev);
    ev = {nullptr, nullptr};
  }
};

// Scratch of the FP32 tensor-core engine for launches on stream s (one buffer per compute
// stream, one more for any other stream); its error word is zeroed when it is first allocated.
int f32_scratch(tmm_context* ctx, cudaStream_t s, size_t bytes, void** ptr) {
  size_t slot = ctx->streams.size();
  for (size_t i = 0; i < ctx->streams.size(); ++i)
    if (ctx->streams[i] == s) slot = i;
  if (ctx->f32_scratch.size() <= slot) ctx->f32_scratch.resize(slot + 1);
  tmm::GrowBuffer& buf = ctx->f32_scratch[slot];
  const bool fresh = bytes > buf.capacity;
  TMM_CUDA(ctx, buf.reserve(bytes));
  if (fresh) TMM_CUDA(ctx, cudaMemset(buf.ptr, 0, 256));
  *ptr = buf.ptr;
  return TMM_SUCCESS;
}

// after synchronisation: a bounded wait of the FP32 engine that gave up
int check_f32_error(tmm_context* ctx) {
  std::vector<tmm::GrowBuffer*> bufs;
  for (auto& b : ctx->f32_scratch) bufs.push_back(&b);
  bufs.push_back(&ctx->batch_f32_scratch);
  for (tmm::GrowBuffer* bp : bufs) {
    tmm::GrowBuffer& b = *bp;
    if (!b.ptr) continue;
    int word = 0;
    TMM_CUDA(ctx, cudaMemcpy(&word, b.ptr, sizeof(int), cudaMemcpyDeviceToHost));
    if (word) {
      cudaMemset(b.ptr, 0, 256);
      return fail(ctx, TMM_ERROR_TIMEOUT, "FP32 tensor-core kernel: a pipeline wait timed out");
    }
  }
  return TMM_SUCCESS;
}

int launch_tile_gemm(tmm_context* ctx, Op opa, Op opb, int64_t m, int64_t n, int64_t k, const void* alpha,
                     const void* A, int64_t lda, const void* B, int64_t ldb, const void* beta, void* C,
                     int64_t ldc, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (ctx->dtype == TMM_COMPLEX_FLOAT && k > 0 && !ctx->f32_simt) {
    // the per-tile cublasCgemm of src/Tiled-MM/tiled_mm.cpp:226-245: the real embedding
    // [[Re A, -Im A], [Im A, Re A]] x [Re B; Im B] (8mnk real flops, the complex count) on the
    // FP32 tensor-core engine, then C = alpha (Re + i Im) + beta C
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t ahat = up((size_t)(2 * m) * (size_t)(2 * k) * 4), bhat = up((size_t)(2 * k) * (size_t)n * 4);
    const size_t tbuf = up((size_t)(2 * m) * (size_t)n * 4);
    const size_t eng = tmm::f32tc_scratch_bytes(2 * m, n, 2 * k);
    void* scratch = nullptr;
    if (int st = f32_scratch(ctx, s, eng + ahat + bhat + tbuf, &scratch)) return st;
    TMM_CUDA(ctx, tmm::f32tc_prepare());
    float* Ahat = (float*)((char*)scratch + eng);
    float* Bhat = (float*)((char*)scratch + eng + ahat);
    float* T = (float*)((char*)scratch + eng + ahat + bhat);
    KernelTimer timer(ctx, s);
    e = tmm::cplx_f32_embed(A, lda, opa, B, ldb, opb, m, n, k, Ahat, Bhat, s);
    if (e == cudaSuccess)
      e = tmm::f32tc_gemm(Op::OP_N, Op::OP_N, 2 * m, n, 2 * k, 1.0f, Ahat, 2 * m, Bhat, 2 * k, 0.0f, T, 2 * m, scratch,
                          eng, s);
    if (e == cudaSuccess) e = tmm::cplx_f32_combine(m, n, alpha, beta, T, C, ldc, s);
    timer.done();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "complex FP32 tensor-core launch");
    ctx->stats.kernels += 6;  // two embeddings, two splits, the product, the combine
    return TMM_SUCCESS;
  }
  if (ctx->dtype == TMM_FLOAT && k > 0 && !ctx->f32_simt) {
    // the per-tile cublasSgemm of src/Tiled-MM/tiled_mm.cpp:181-198 on the tcgen05 tensor cores
    void* scratch = nullptr;
    const size_t bytes = tmm::f32tc_scratch_bytes(m, n, k);
    if (int st = f32_scratch(ctx, s, bytes, &scratch)) return st;
    TMM_CUDA(ctx, tmm::f32tc_prepare());
    KernelTimer timer(ctx, s);
    e = tmm::f32tc_gemm(opa, opb, m, n, k, *(const float*)alpha, (const float*)A, lda, (const float*)B, ldb,
                        *(const float*)beta, (float*)C, ldc, scratch, bytes, s);
    timer.done();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "FP32 tensor-core launch");
    ctx->stats.kernels += 3;  // two splits, the product
    return TMM_SUCCESS;
  }
  KernelTimer timer(ctx, s);
  switch (ctx->dtype) {
    case TMM_FLOAT:
      e = k == 0 ? tmm::launch_scale_f32(m, n, *(const float*)beta, (float*)C, ldc, s)
                 : tmm::launch_gemm_f32(opa, opb, m, n, k, *(const float*)alpha, (const float*)A, lda,
                                        (const float*)B, ldb, *(const float*)beta, (float*)C, ldc, s);
      break;
    case TMM_DOUBLE:
      e = k == 0 ? tmm::launch_scale_f64(m, n, *(const double*)beta, (double*)C, ldc, s)
                 : tmm::launch_gemm_f64(opa, opb, m, n, k, *(const double*)alpha, (const double*)A, lda,
                                        (const double*)B, ldb, *(const double*)beta, (double*)C, ldc, s);
      break;
    case TMM_COMPLEX_FLOAT:
      e = k == 0 ? tmm::launch_scale_c32(m, n, *(const tmm::cplxf*)beta, (tmm::cplxf*)C, ldc, s)
                 : tmm::launch_gemm_c32(opa, opb, m, n, k, *(const tmm::cplxf*)alpha, (const tmm::cplxf*)A, lda,
                                        (const tmm::cplxf*)B, ldb, *(const tmm::cplxf*)beta, (tmm::cplxf*)C, ldc, s);
      break;
    default:
      e = k == 0 ? tmm::launch_scale_c64(m, n, *(const tmm::cplxd*)beta, (tmm::cplxd*)C, ldc, s)
                 : tmm::launch_gemm_c64(opa, opb, m, n, k, *(const tmm::cplxd*)alpha, (const tmm::cplxd*)A, lda,
                                        (const tmm::cplxd*)B, ldb, *(const tmm::cplxd*)beta, (tmm::cplxd*)C, ldc, s);
  }
  timer.done();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tile kernel launch");
  ctx->stats.kernels++;
  return TMM_SUCCESS;
}

int make_events(tmm_context* ctx, tmm::TileCache& c) {
  for (auto& s : c.slots) {
    if (!s.ready) TMM_CUDA(ctx, cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming));
    if (!s.last_use) TMM_CUDA(ctx, cudaEventCreateWithFlags(&s.last_use, cudaEventDisableTiming));
  }
  return TMM_SUCCESS;
}

void destroy_events(tmm::TileCache& c) {
  for (auto& s : c.slots) {
    if (s.ready) cudaEventDestroy(s.ready);
    if (s.last_use) cudaEventDestroy(s.last_use);
    s.ready = s.last_use = nullptr;
  }
}

// Host-range registration for one call (src/Tiled-MM/tiled_mm.cpp:529-554).
// Registers exactly the bytes the matrix spans: ld*(cols-1)+rows elements.
struct Pin {
  void* ptr = nullptr;
  bool owned = false;
};

// device or managed memory: the GPU reads it directly (cudaPointerGetAttributes, the
// query the reference's runtime shim forwards unused: gpu_runtime_api.hpp:223-226)
bool device_accessible(const void* p) {
  if (!p) return false;
  cudaPointerAttributes attr;
  const bool ok = cudaPointerGetAttributes(&attr, p) == cudaSuccess;
  cudaGetLastError();
  return ok && (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged);
}

int pin_range(tmm_context* ctx, const void* p, size_t bytes, Pin* out) {
  out->ptr = nullptr;
  out->owned = false;
  if (!p || bytes == 0) return TMM_SUCCESS;
  // page-locked already (cudaHostAlloc / cudaMallocHost / an earlier registration), or
  // device / managed memory: use as is
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type != cudaMemoryTypeUnregistered) {
    cudaGetLastError();
    return TMM_SUCCESS;
  }
  cudaGetLastError();
  cudaError_t e = cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterDefault);
  if (e == cudaSuccess) {
    out->ptr = const_cast<void*>(p);
    out->owned = true;
    return TMM_SUCCESS;
  }
  cudaGetLastError();  // clear the sticky-free error state of the failed call
  if (e == cudaErrorHostMemoryAlreadyRegistered) return TMM_SUCCESS;
  return cuda_fail(ctx, e, "cudaHostRegister");
}

void unpin(Pin& p) {
  if (p.owned) cudaHostUnregister(p.ptr);
  p.owned = false;
}

}  // namespace

void tmm::set_last_error_message(const char* msg) { g_last_error = msg ? msg : ""; }

// ------------------------------------------------------------------ GrowBuffer
cudaError_t tmm::GrowBuffer::reserve(size_t want) {
  if (want <= capacity) {
    bytes = want;
    return cudaSuccess;
  }
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  capacity = 0;
  size_t cap = (size_t)std::ceil(1.2 * (double)want);
  cap = (cap + 255) / 256 * 256;
  cudaError_t e = cudaMalloc(&ptr, cap);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&ptr, want);  // no headroom left: exact size
    if (e != cudaSuccess) {
      cudaGetLastError();
      ptr = nullptr;
      return cudaErrorMemoryAllocation;
    }
    cap = want;
  }
  capacity = cap;
  bytes = want;
  return cudaSuccess;
}

void tmm::GrowBuffer::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = capacity = 0;
}

// ------------------------------------------------------------------ C ABI: context
extern "C" int tmm_create(int dtype, int n_streams, int max_tile_m, int max_tile_n, int max_tile_k,
                          tmm_context** out) {
  if (!out) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_create: null output");
  *out = nullptr;
  if (dtype < TMM_FLOAT || dtype > TMM_COMPLEX_DOUBLE)
    return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_create: unknown dtype");
  if (n_streams < 1 || max_tile_m < 1 || max_tile_n < 1 || max_tile_k < 1)
    return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_create: streams and tile sizes must be positive");
  auto* ctx = new tmm_context();
  ctx->dtype = dtype;
  ctx->n_streams = n_streams;
  ctx->max_tile_m = max_tile_m;
  ctx->max_tile_n = max_tile_n;
  ctx->max_tile_k = max_tile_k;
  ctx->oz_engine = tmm::ozaki_default_engine();
  if (const char* f32 = getenv("TMM_F32_KERNEL")) ctx->f32_simt = strcmp(f32, "simt") == 0;
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e == cudaSuccess) {
    int pageable = 0, host_tables = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, ctx->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device) !=
            cudaSuccess)
      pageable = host_tables = 0;
    // opt-in: the copy engines already read pageable memory near the link rate here (190-202 GB/s),
    // and copy kernels beside the slice-product engine slowed the out-of-core update by 9 %
    const char* env = getenv("TMM_DIRECT_HOST");
    ctx->direct_host = pageable && host_tables && env && env[0] == '1';
    cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->prep, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking);
  for (int i = 0; e == cudaSuccess && i < n_streams; ++i) {
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) ctx->streams.push_back(s);
  }
  if (e != cudaSuccess) {
    int st = cuda_fail(nullptr, e, "tmm_create");
    tmm_destroy(ctx);
    return st;
  }
  *out = ctx;
  return TMM_SUCCESS;
}

extern "C" int tmm_destroy(tmm_context* ctx) {
  if (!ctx) return TMM_SUCCESS;
  DeviceGuard dg(ctx->device);
  for (auto s : ctx->streams) cudaStreamSynchronize(s);
  if (ctx->h2d) cudaStreamSynchronize(ctx->h2d);
  if (ctx->prep) cudaStreamSynchronize(ctx->prep);
  if (ctx->d2h) cudaStreamSynchronize(ctx->d2h);
  destroy_events(ctx->cache_a);
  destroy_events(ctx->cache_b);
  for (auto& c : ctx->cslots)
    if (c.done) cudaEventDestroy(c.done);
  for (auto e : ctx->staging_free)
    if (e) cudaEventDestroy(e);
  ctx->pool_a.release();
  ctx->pool_b.release();
  ctx->pool_c.release();
  ctx->full_c.release();
  ctx->staging.release();
  ctx->scratch.release();
  ctx->oz_work.release();
  if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
  if (ctx->batch_aux) cudaStreamDestroy(ctx->batch_aux);
  if (ctx->batch_fork) cudaEventDestroy(ctx->batch_fork);
  if (ctx->batch_join) cudaEventDestroy(ctx->batch_join);
  for (auto* v : {&ctx->kt_pending, &ctx->kt_free})
    for (auto& ev : *v) {
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
  if (ctx->kt_origin) cudaEventDestroy(ctx->kt_origin);
  ctx->batch_arena.release();
  ctx->batch_meta.release();
  ctx->batch_oz_scratch.release();
  ctx->batch_f32_scratch.release();
  if (ctx->batch_f32_stream) cudaStreamDestroy(ctx->batch_f32_stream);
  if (ctx->batch_f32_fork) cudaEventDestroy(ctx->batch_f32_fork);
  if (ctx->batch_f32_join) cudaEventDestroy(ctx->batch_f32_join);
  for (auto b : ctx->batch_lanes) cudaStreamDestroy(b);
  for (auto e : ctx->batch_lane_events) cudaEventDestroy(e);
  for (auto& b : ctx->cz_scratch) b.release();
  for (auto& b : ctx->f32_scratch) b.release();
  for (auto b : ctx->oz_branches) cudaStreamDestroy(b);
  for (auto e : ctx->oz_branch_done) cudaEventDestroy(e);
  if (ctx->oz_fork) cudaEventDestroy(ctx->oz_fork);
  for (auto s : ctx->streams) cudaStreamDestroy(s);
  if (ctx->h2d) cudaStreamDestroy(ctx->h2d);
  if (ctx->prep) cudaStreamDestroy(ctx->prep);
  if (ctx->d2h) cudaStreamDestroy(ctx->d2h);
  delete ctx;
  return TMM_SUCCESS;
}

// ------------------------------------------------------------------ settings
extern "C" int tmm_set_num_streams(tmm_context* ctx, int n) {
  if (!ctx || n < 1) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_num_streams: need n >= 1");
  DeviceGuard dg(ctx->device);
  while ((int)ctx->streams.size() < n) {
    cudaStream_t s;
    TMM_CUDA(ctx, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    ctx->streams.push_back(s);
  }
  ctx->n_streams = n;
  return TMM_SUCCESS;
}

extern "C" int tmm_get_num_streams(tmm_context* ctx, int* n) {
  if (!ctx || !n) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_num_streams: null argument");
  *n = ctx->n_streams;
  return TMM_SUCCESS;
}

extern "C" int tmm_set_tile_sizes(tmm_context* ctx, int tm, int tn, int tk) {
  if (!ctx || tm < 1 || tn < 1 || tk < 1) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_tile_sizes: need positive sizes");
  // src/Tiled-MM/mm_handle.cpp:58-66 asserts tile <= max tile
  if (tm > ctx->max_tile_m || tn > ctx->max_tile_n || tk > ctx->max_tile_k)
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_tile_sizes: tile larger than the context's maximum");
  ctx->cur_tile_m = tm;
  ctx->cur_tile_n = tn;
  ctx->cur_tile_k = tk;
  return TMM_SUCCESS;
}

extern "C" int tmm_get_tile_sizes(tmm_context* ctx, int* tm, int* tn, int* tk) {
  if (!ctx || !tm || !tn || !tk) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_tile_sizes: null argument");
  *tm = ctx->cur_tile_m;
  *tn = ctx->cur_tile_n;
  *tk = ctx->cur_tile_k;
  return TMM_SUCCESS;
}

extern "C" int tmm_set_full_sizes(tmm_context* ctx, int64_t m, int64_t n, int64_t k) {
  if (!ctx || m <= 0 || n <= 0 || k <= 0) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_full_sizes: need positive sizes");
  DeviceGuard dg(ctx->device);
  TMM_CUDA(ctx, ctx->full_c.reserve((size_t)m * (size_t)n * elem_size(ctx->dtype)));
  ctx->full_c_elems = (size_t)m * (size_t)n;
  return TMM_SUCCESS;
}

extern "C" int tmm_optimal_tile_sizes(tmm_context* ctx, int64_t m, int64_t n, int64_t k, int* tm, int* tn, int* tk) {
  if (!ctx || !tm || !tn || !tk) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_optimal_tile_sizes: null argument");
  *tm = optimal_tile_size(m, ctx->cur_tile_m, ctx->max_tile_m);
  *tn = optimal_tile_size(n, ctx->cur_tile_n, ctx->max_tile_n);
  *tk = optimal_tile_size(k, ctx->cur_tile_k, ctx->max_tile_k);
  return TMM_SUCCESS;
}

extern "C" int tmm_get_max_tile_sizes(tmm_context* ctx, int* tm, int* tn, int* tk) {
  if (!ctx || !tm || !tn || !tk) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_max_tile_sizes: null argument");
  *tm = ctx->max_tile_m;
  *tn = ctx->max_tile_n;
  *tk = ctx->max_tile_k;
  return TMM_SUCCESS;
}

extern "C" int tmm_set_streams_and_tiles(tmm_context* ctx, int n_streams, int tm, int tn, int tk) {
  int st = tmm_set_num_streams(ctx, n_streams);
  if (st != TMM_SUCCESS) return st;
  return tmm_set_tile_sizes(ctx, tm, tn, tk);
}

extern "C" int tmm_set_path(tmm_context* ctx, int path, int slices) {
  if (!ctx) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_path: null context");
  if (path != TMM_PATH_NATIVE && path != TMM_PATH_OZAKI)
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_path: unknown path");
  if (slices > tmm::OZ_MAX_SLICES)
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_path: too many slices");
  ctx->path = path;
  ctx->ozaki_slices = slices > 0 ? slices : tmm::oz_default_slices(ctx->dtype);
  return TMM_SUCCESS;
}

extern "C" int tmm_get_path(tmm_context* ctx, int* path, int* slices) {
  if (!ctx || !path || !slices) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_path: null argument");
  *path = ctx->path;
  *slices = ctx->path == TMM_PATH_OZAKI ? ctx->ozaki_slices : 0;
  return TMM_SUCCESS;
}

extern "C" int tmm_set_ozaki_engine(tmm_context* ctx, int engine) {
  if (!ctx || (engine != tmm::OZ_ENGINE_IMMA && engine != tmm::OZ_ENGINE_TCGEN05))
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_ozaki_engine: unknown engine");
  ctx->oz_engine = engine;
  return TMM_SUCCESS;
}

extern "C" int tmm_get_ozaki_engine(tmm_context* ctx, int* engine, int* k_block, int64_t* pass_blocks) {
  if (!ctx || !engine || !k_block || !pass_blocks)
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_ozaki_engine: null argument");
  *engine = ctx->oz_engine;
  *k_block = (int)tmm::ozaki_k_block(ctx->oz_engine);
  *pass_blocks = tmm::ozaki_pass_blocks(ctx->oz_engine);
  return TMM_SUCCESS;
}

extern "C" int tmm_set_tile_policy(tmm_context* ctx, int policy) {
  if (!ctx || policy < TMM_TILE_POLICY_REFERENCE || policy > TMM_TILE_POLICY_AUTOTUNE)
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_tile_policy: unknown policy");
  ctx->tile_policy = policy;
  return TMM_SUCCESS;
}

extern "C" int tmm_set_memory_limit(tmm_context* ctx, size_t bytes) {
  if (!ctx) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_memory_limit: null context");
  ctx->memory_limit = bytes;
  return TMM_SUCCESS;
}

extern "C" int tmm_get_stats(tmm_context* ctx, tmm_stats* st) {
  if (!ctx || !st) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_stats: null argument");
  *st = ctx->stats;
  return TMM_SUCCESS;
}

extern "C" int tmm_set_kernel_timing(tmm_context* ctx, int on) {
  if (!ctx) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_set_kernel_timing: null context");
  DeviceGuard dg(ctx->device);
  for (auto& ev : ctx->kt_pending) {  // drop what was recorded so far
    cudaEventSynchronize(ev.second);
    ctx->kt_free.push_back(ev);
  }
  ctx->kt_pending.clear();
  ctx->kt_seconds = 0.0;
  ctx->kt_launches = 0;
  ctx->kt_intervals.clear();
  ctx->ktime = on != 0;
  if (ctx->ktime) {
    // the origin is recorded on the context's first stream before any timed launch
    if (!ctx->kt_origin) TMM_CUDA(ctx, cudaEventCreate(&ctx->kt_origin));
    TMM_CUDA(ctx, cudaEventRecord(ctx->kt_origin, ctx->streams.empty() ? (cudaStream_t)0 : ctx->streams[0]));
  }
  return TMM_SUCCESS;
}

// waits for the recorded launches and folds them into the totals and the interval list
static int drain_kernel_timing(tmm_context* ctx) {
  for (auto& ev : ctx->kt_pending) {
    TMM_CUDA(ctx, cudaEventSynchronize(ev.second));
    float ms = 0.0f, t0 = 0.0f, t1 = 0.0f;
    TMM_CUDA(ctx, cudaEventElapsedTime(&ms, ev.first, ev.second));
    ctx->kt_seconds += 1e-3 * (double)ms;
    ctx->kt_launches++;
    if (ctx->kt_origin && cudaEventElapsedTime(&t0, ctx->kt_origin, ev.first) == cudaSuccess &&
        cudaEventElapsedTime(&t1, ctx->kt_origin, ev.second) == cudaSuccess)
      ctx->kt_intervals.emplace_back(1e-3 * (double)t0, 1e-3 * (double)t1);
    ctx->kt_free.push_back(ev);
  }
  ctx->kt_pending.clear();
  return TMM_SUCCESS;
}

extern "C" int tmm_get_kernel_time(tmm_context* ctx, double* seconds, uint64_t* launches) {
  if (!ctx || !seconds) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_kernel_time: null argument");
  DeviceGuard dg(ctx->device);
  if (int st = drain_kernel_timing(ctx)) return st;
  *seconds = ctx->kt_seconds;
  if (launches) *launches = ctx->kt_launches;
  return TMM_SUCCESS;
}

extern "C" int tmm_get_kernel_busy_time(tmm_context* ctx, double* busy_seconds, double* span_seconds) {
  if (!ctx || !busy_seconds) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_kernel_busy_time: null argument");
  DeviceGuard dg(ctx->device);
  if (int st = drain_kernel_timing(ctx)) return st;
  std::vector<std::pair<double, double>> iv = ctx->kt_intervals;
  std::sort(iv.begin(), iv.end());
  double busy = 0.0, cur0 = 0.0, cur1 = -1.0;
  for (const auto& x : iv) {
    if (x.first > cur1) {  // a gap: close the current run of overlapping launches
      if (cur1 > cur0) busy += cur1 - cur0;
      cur0 = x.first;
      cur1 = x.second;
    } else if (x.second > cur1) {
      cur1 = x.second;
    }
  }
  if (cur1 > cur0) busy += cur1 - cur0;
  *busy_seconds = busy;
  if (span_seconds) *span_seconds = iv.empty() ? 0.0 : cur1 - iv.front().first;
  return TMM_SUCCESS;
}

extern "C" const char* tmm_last_error(tmm_context* ctx) {
  return ctx ? ctx->last_error.c_str() : g_last_error.c_str();
}

extern "C" const char* tmm_status_string(int status) {
  switch (status) {
    case TMM_SUCCESS: return "success";
    case TMM_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case TMM_ERROR_CUDA: return "CUDA error";
    case TMM_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case TMM_ERROR_NOT_SUPPORTED: return "not supported";
    case TMM_ERROR_TIMEOUT: return "device wait timed out";
    default: return "internal error";
  }
}

extern "C" int tmm_get_full_c(tmm_context* ctx, void** ptr, size_t* size, size_t* capacity) {
  if (!ctx || !ptr) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_full_c: null argument");
  *ptr = ctx->full_c.ptr;
  if (size) *size = ctx->full_c_elems;
  if (capacity) *capacity = ctx->full_c.capacity / elem_size(ctx->dtype);
  return TMM_SUCCESS;
}

// ------------------------------------------------------------------ the pipeline
namespace {

// The tcgen05 engine's error word and per-stream FP64 workspaces.
constexpr size_t OZ_ERR_BLOCK = 256;
int reserve_oz_work(tmm_context* ctx, int streams) {
  if (ctx->oz_engine != tmm::OZ_ENGINE_TCGEN05) return TMM_SUCCESS;
  size_t per = (tmm::ozaki_workspace_bytes(ctx->oz_engine) + 255) / 256 * 256;
  bool fresh = ctx->oz_work.ptr == nullptr;
  TMM_CUDA(ctx, ctx->oz_work.reserve(OZ_ERR_BLOCK + (size_t)streams * per));
  if (fresh || ctx->oz_work.bytes) TMM_CUDA(ctx, cudaMemset(ctx->oz_work.ptr, 0, OZ_ERR_BLOCK));
  return TMM_SUCCESS;
}
double* oz_workspace(tmm_context* ctx, int stream_index) {
  if (!ctx->oz_work.ptr) return nullptr;
  size_t per = (tmm::ozaki_workspace_bytes(ctx->oz_engine) + 255) / 256 * 256;
  return (double*)((char*)ctx->oz_work.ptr + OZ_ERR_BLOCK + (size_t)stream_index * per);
}
int* oz_error_word(tmm_context* ctx) { return ctx->oz_work.ptr ? (int*)ctx->oz_work.ptr : nullptr; }
// after synchronisation: a bounded device wait that gave up
int check_oz_error(tmm_context* ctx);

// Float, complex float and complex double on the Ozaki engine (the reference multiplies
// these tiles with cublasSgemm / cublasCgemm / cublasZgemm, src/Tiled-MM/tiled_mm.cpp:226-268):
// per k tile of at most max_tile_k, the real FP64 embedding of op(A) and op(B)
// (tmm_ozaki_embed.cu) is split and multiplied by the real engine into T, then combined
// into C with alpha and beta (beta on the first k tile only), rounded once to the
// context's type.  Scratch of stream slot `slot`; the caller has reserved the engine's
// workspace (reserve_oz_work) for that slot.
int embedded_ozaki(tmm_context* ctx, Op opa, Op opb, int64_t m, int64_t n, int64_t k, const void* alpha,
                   const void* a, int64_t ld_a, const void* b, int64_t ld_b, const void* beta, void* c, int64_t ld_c,
                   cudaStream_t s, int slot) {
  if (m <= 0 || n <= 0) return TMM_SUCCESS;
  const int dt = ctx->dtype;
  const bool cplx = dt == TMM_COMPLEX_FLOAT || dt == TMM_COMPLEX_DOUBLE;
  const int slices = ctx->ozaki_slices > 0 ? ctx->ozaki_slices : tmm::oz_default_slices(dt);
  const int64_t tk = std::max<int64_t>(1, std::min<int64_t>(k, ctx->max_tile_k));
  const int64_t me = cplx ? 2 * m : m, ke = cplx ? 2 * tk : tk;  // embedded sizes
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t ahat = up((size_t)me * (size_t)ke * 8), bhat = up((size_t)ke * (size_t)n * 8);
  const size_t tbuf = up((size_t)me * (size_t)n * 8);
  const size_t sa = up(tmm::ozaki_split_bytes(me, ke, slices)), sb = up(tmm::ozaki_split_bytes(n, ke, slices));
  if ((int)ctx->cz_scratch.size() <= slot) ctx->cz_scratch.resize((size_t)slot + 1);
  tmm::GrowBuffer& buf = ctx->cz_scratch[(size_t)slot];
  TMM_CUDA(ctx, buf.reserve(ahat + bhat + tbuf + sa + sb));
  char* base = (char*)buf.ptr;
  double* Ahat = (double*)base;
  double* Bhat = (double*)(base + ahat);
  double* T = (double*)(base + ahat + bhat);
  char* SA = base + ahat + bhat + tbuf;
  char* SB = SA + sa;
  char one[16] = {0};
  if (dt == TMM_FLOAT || dt == TMM_COMPLEX_FLOAT) *(float*)one = 1.f;
  else *(double*)one = 1.0;
  const size_t es = elem_size(dt);
  if (k == 0) {  // C = beta * C
    TMM_CUDA(ctx, cudaMemsetAsync(T, 0, (size_t)me * (size_t)n * 8, s));
    TMM_CUDA(ctx, tmm::ozaki_combine(dt, m, n, alpha, beta, true, T, c, ld_c, s));
    return TMM_SUCCESS;
  }
  for (int64_t k0 = 0, kt = 0; k0 < k; k0 += tk, ++kt) {
    const int64_t kk = std::min(tk, k - k0), kke = cplx ? 2 * kk : kk;
    const char* ab = (const char*)a + (size_t)(opa == tmm::OP_N ? k0 * ld_a : k0) * es;
    const char* bb = (const char*)b + (size_t)(opb == tmm::OP_N ? k0 : k0 * ld_b) * es;
    tmm::OzakiSplit va = tmm::ozaki_split_view(SA, me, kke, slices, ctx->oz_engine);
    tmm::OzakiSplit vb = tmm::ozaki_split_view(SB, n, kke, slices, ctx->oz_engine);
    // Ahat: me x kke, ld me; Bhat: kke x n, ld kke (lines of the split: rows of Ahat, columns of Bhat)
    cudaError_t e = tmm::ozaki_embed(dt, ab, ld_a, opa, bb, ld_b, opb, m, n, kk, Ahat, Bhat, s);
    if (e == cudaSuccess) e = tmm::ozaki_split(Ahat, me, tmm::OP_N, me, kke, va, s);
    if (e == cudaSuccess) e = tmm::ozaki_split(Bhat, kke, tmm::OP_T, n, kke, vb, s);
    if (e == cudaSuccess) {
      KernelTimer timer(ctx, s);
      e = tmm::ozaki_gemm(va, vb, me, n, 1.0, 0.0, true, T, me, ctx->oz_engine, oz_workspace(ctx, slot),
                          oz_error_word(ctx), s);
      timer.done();
    }
    if (e == cudaSuccess) e = tmm::ozaki_combine(dt, m, n, alpha, kt == 0 ? beta : (const void*)one, true, T, c, ld_c, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "embedded ozaki launch");
    ctx->stats.kernels += 8;  // two embeddings, two two-kernel splits, the product, the combine
  }
  return TMM_SUCCESS;
}

int check_oz_error(tmm_context* ctx) {
  if (!ctx->oz_work.ptr || ctx->oz_engine != tmm::OZ_ENGINE_TCGEN05) return TMM_SUCCESS;
  int word = 0;
  TMM_CUDA(ctx, cudaMemcpy(&word, ctx->oz_work.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (word) {
    cudaMemset(ctx->oz_work.ptr, 0, OZ_ERR_BLOCK);
    return fail(ctx, TMM_ERROR_TIMEOUT, "tcgen05 Ozaki kernel: a pipeline wait timed out");
  }
  return TMM_SUCCESS;
}

struct Plan {
  int64_t m, n, k, tm, tn, tk;
  int engine;
  int64_t ntm, ntn, ntk;
  Op opa, opb;
  size_t es;
  bool ozaki;
  bool embed;  // float / complex on the Ozaki engine: raw tiles, per-tile real FP64 embedding
  int slices;
  size_t a_slot_bytes, b_slot_bytes, c_slot_bytes, staging_bytes;
};

int64_t ntiles(int64_t len, int64_t t) { return len == 0 ? 0 : (len + t - 1) / t; }
int64_t extent(int64_t len, int64_t t, int64_t id) { return std::min(t, len - id * t); }

// Size the tile caches: everything resident when it fits, else one A row
// panel (double-buffered when possible) and the rest for B.
int plan_memory(tmm_context* ctx, const Plan& P, bool copy_back, size_t* n_a, size_t* n_b) {
  size_t freeb = 0, total = 0;
  TMM_CUDA(ctx, cudaMemGetInfo(&freeb, &total));
  size_t held = ctx->pool_a.capacity + ctx->pool_b.capacity + ctx->pool_c.capacity + ctx->staging.capacity;
  size_t avail = (size_t)((double)(freeb + held) * 0.92);
  if (ctx->memory_limit) avail = std::min(avail, ctx->memory_limit);
  size_t fixed = 0;
  if (copy_back) fixed += 2 * (size_t)ctx->n_streams * P.c_slot_bytes;
  else fixed += (size_t)P.m * (size_t)P.n * P.es;  // full C (held outside the cache budget)
  fixed += 3 * P.staging_bytes;
  if (avail <= fixed) return fail(ctx, TMM_ERROR_OUT_OF_MEMORY, "not enough device memory for the C tiles");
  size_t budget = avail - fixed;
  size_t total_a = (size_t)(P.ntm * P.ntk), total_b = (size_t)(P.ntk * P.ntn);
  if (total_a * P.a_slot_bytes + total_b * P.b_slot_bytes <= budget) {
    *n_a = total_a;
    *n_b = total_b;
    return TMM_SUCCESS;
  }
  // A: one panel (+ one panel of prefetch when it fits), at least 2 slots
  size_t want_a = std::min(total_a, (size_t)(2 * P.ntk));
  while (want_a > 2 && want_a * P.a_slot_bytes + 2 * P.b_slot_bytes > budget) --want_a;
  if (want_a < 2) want_a = std::min<size_t>(2, total_a);
  if (want_a * P.a_slot_bytes + std::min<size_t>(2, total_b) * P.b_slot_bytes > budget)
    return fail(ctx, TMM_ERROR_OUT_OF_MEMORY, "not enough device memory for two A and two B tiles");
  size_t want_b = std::min(total_b, (budget - want_a * P.a_slot_bytes) / P.b_slot_bytes);
  *n_a = want_a;
  *n_b = std::max<size_t>(want_b, std::min<size_t>(2, total_b));
  return TMM_SUCCESS;
}

int setup_cache(tmm_context* ctx, tmm::TileCache& c, tmm::GrowBuffer& pool, size_t n, size_t slot_bytes) {
  const size_t sb = (slot_bytes + 255) / 256 * 256;
  TMM_CUDA(ctx, pool.reserve(n * sb));
  while (c.slots.size() > n) {  // drop surplus slots (no work is pending: every call ends synchronised)
    tmm::Slot& s = c.slots.back();
    if (s.ready) cudaEventDestroy(s.ready);
    if (s.last_use) cudaEventDestroy(s.last_use);
    c.slots.pop_back();
  }
  c.slots.resize(n);
  for (size_t i = 0; i < n; ++i) c.slots[i].ptr = (char*)pool.ptr + i * sb;
  int st = make_events(ctx, c);
  if (st) return st;
  c.invalidate();
  return TMM_SUCCESS;
}

struct HostMat {
  const char* ptr;
  int64_t ld;   // elements
  bool direct;  // unregistered host memory that the GPU accesses directly: copied by kernel
};

// true for ordinary (unregistered) host memory on a GPU that reads it through the host page
// tables (the NVLink-C2C systems): a copy-engine copy of it is staged through page-locked
// buffers and returns only when the source is consumed, a copy kernel stays asynchronous
bool host_direct(const tmm_context* ctx, const void* p) {
  if (!ctx->direct_host || !p) return false;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeUnregistered;
}

// 2D copy (height rows of width bytes) on stream s: by kernel when `direct`, else by the
// copy engines
int copy2d(tmm_context* ctx, void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t height,
           cudaStream_t s, bool direct) {
  if (direct) {
    TMM_CUDA(ctx, tmm::copy2d_async(dst, dpitch, src, spitch, width, height, s));
    ctx->stats.kernels++;
    ctx->stats.direct_bytes += (uint64_t)width * (uint64_t)height;
    return TMM_SUCCESS;
  }
  TMM_CUDA(ctx, cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, cudaMemcpyDefault, s));
  return TMM_SUCCESS;
}

// Brings tile `key` (stored sub-block rows r0.., cols c0.. of size rr x cc)
// into the cache; returns the slot.  The copy waits for the evicted tile's
// last reader.  Ozaki tiles are staged raw, then split on the prep stream.
int fetch_tile(tmm_context* ctx, const Plan& P, tmm::TileCache& cache, int64_t key, const HostMat& h,
               int64_t r0, int64_t c0, int64_t rr, int64_t cc, bool lines_are_rows, int* out_slot,
               int* staging_turn, cudaStream_t split_stream) {
  int idx = cache.find(key);
  if (idx >= 0) {
    cache.slots[idx].stamp = ++cache.clock;
    ctx->stats.tiles_reused++;
    *out_slot = idx;
    return TMM_SUCCESS;
  }
  idx = cache.victim();
  tmm::Slot& s = cache.slots[idx];
  if (s.key >= 0) cache.index.erase(s.key);
  const char* src = h.ptr + ((size_t)r0 + (size_t)c0 * (size_t)h.ld) * P.es;
  if (!P.ozaki) {
    if (s.used) TMM_CUDA(ctx, cudaStreamWaitEvent(ctx->h2d, s.last_use, 0));
    int st = copy2d(ctx, s.ptr, (size_t)rr * P.es, src, (size_t)h.ld * P.es, (size_t)rr * P.es, (size_t)cc, ctx->h2d,
                    h.direct);
    if (st) return st;
    TMM_CUDA(ctx, cudaEventRecord(s.ready, ctx->h2d));
  } else {
    // raw tile -> staging buffer (ring of 3) on the copy stream; split -> slot on the stream of
    // the tile's first consumer, after the kernels already queued there: split CTAs resident
    // beside the persistent slice-product kernel would take issue slots from its single-thread
    // MMA issuer, and the split is ~3 % of the work, so running it concurrently gains little
    int turn = (*staging_turn)++ % 3;
    char* stage = (char*)ctx->staging.ptr + (size_t)turn * ((P.staging_bytes + 255) / 256 * 256);
    TMM_CUDA(ctx, cudaStreamWaitEvent(ctx->h2d, ctx->staging_free[turn], 0));
    int st = copy2d(ctx, stage, (size_t)rr * P.es, src, (size_t)h.ld * P.es, (size_t)rr * P.es, (size_t)cc, ctx->h2d,
                    h.direct);
    if (st) return st;
    TMM_CUDA(ctx, cudaEventRecord(s.ready, ctx->h2d));  // reused below as "staged"
    TMM_CUDA(ctx, cudaStreamWaitEvent(split_stream, s.ready, 0));
    if (s.used) TMM_CUDA(ctx, cudaStreamWaitEvent(split_stream, s.last_use, 0));
    // lines along k: for A (lines = rows of op(A)); for B (lines = columns of op(B))
    int64_t lines = lines_are_rows ? rr : cc;   // stored orientation resolved by caller
    int64_t kk = lines_are_rows ? cc : rr;
    Op t = lines_are_rows ? tmm::OP_N : tmm::OP_T;
    tmm::OzakiSplit v = tmm::ozaki_split_view(s.ptr, lines, kk, P.slices, P.engine);
    cudaError_t e = tmm::ozaki_split((const double*)stage, rr, t, lines, kk, v, split_stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "ozaki split launch");
    ctx->stats.kernels++;
    TMM_CUDA(ctx, cudaEventRecord(s.ready, split_stream));
    TMM_CUDA(ctx, cudaEventRecord(ctx->staging_free[turn], split_stream));
  }
  ctx->stats.h2d_bytes += (uint64_t)rr * (uint64_t)cc * P.es;
  ctx->stats.tiles_loaded++;
  s.key = key;
  s.stamp = ++cache.clock;
  cache.index[key] = idx;
  *out_slot = idx;
  return TMM_SUCCESS;
}

int run_gemm(tmm_context* ctx, Plan& P, const void* alpha, const void* a, int64_t lda, const void* b,
             int64_t ldb, const void* beta, void* c, int64_t ldc, bool copy_back) {
  const bool beta_nz = !is_zero(ctx->dtype, beta);
  const int ns = (int)std::max<int64_t>(1, std::min<int64_t>(ctx->n_streams, P.ntm * P.ntn));  // tiled_mm.cpp:284

  // ---- memory
  size_t n_a = 0, n_b = 0;
  int st = plan_memory(ctx, P, copy_back, &n_a, &n_b);
  if (st) return st;
  if (P.ntk > 0) {
    st = setup_cache(ctx, ctx->cache_a, ctx->pool_a, n_a, P.a_slot_bytes);
    if (st) return st;
    st = setup_cache(ctx, ctx->cache_b, ctx->pool_b, n_b, P.b_slot_bytes);
    if (st) return st;
  }
  if (P.embed) {
    st = reserve_oz_work(ctx, ns);
    if (st) return st;
  }
  if (P.ozaki) {
    st = reserve_oz_work(ctx, ns);
    if (st) return st;
    size_t sb = (P.staging_bytes + 255) / 256 * 256;
    TMM_CUDA(ctx, ctx->staging.reserve(3 * sb));
    while (ctx->staging_free.size() < 3) {
      cudaEvent_t e;
      TMM_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ctx->staging_free.push_back(e);
    }
    // staging buffers start free
    for (auto e : ctx->staging_free) TMM_CUDA(ctx, cudaEventRecord(e, ctx->prep));
  }
  if (copy_back) {
    size_t cb = (P.c_slot_bytes + 255) / 256 * 256;
    TMM_CUDA(ctx, ctx->pool_c.reserve(2 * (size_t)ns * cb));
    while ((int)ctx->cslots.size() < 2 * ns) ctx->cslots.push_back(tmm::CSlot());
    for (int i = 0; i < 2 * ns; ++i) {
      if (!ctx->cslots[i].done) TMM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->cslots[i].done, cudaEventDisableTiming));
      ctx->cslots[i].ptr = (char*)ctx->pool_c.ptr + (size_t)i * cb;
      ctx->cslots[i].used = false;
    }
  } else {
    TMM_CUDA(ctx, ctx->full_c.reserve((size_t)P.m * (size_t)P.n * P.es));
    ctx->full_c_elems = (size_t)P.m * (size_t)P.n;
  }

  // everything queued on this context's streams starts after earlier work on them
  HostMat A{(const char*)a, lda, host_direct(ctx, a)}, B{(const char*)b, ldb, host_direct(ctx, b)};
  const bool c_direct = host_direct(ctx, c);
  const char* Ch = (const char*)c;
  int staging_turn = 0;
  char one[16] = {0};  // the scalar 1 of the context's dtype (beta' of later k-tiles)
  switch (ctx->dtype) {
    case TMM_FLOAT: *(float*)one = 1.f; break;
    case TMM_DOUBLE: *(double*)one = 1.0; break;
    case TMM_COMPLEX_FLOAT: ((float*)one)[0] = 1.f; break;
    default: ((double*)one)[0] = 1.0;
  }

  int64_t t = 0;
  for (int64_t i = 0; i < P.ntm; ++i) {
    const int64_t mi = extent(P.m, P.tm, i), r0 = i * P.tm;
    for (int64_t jj = 0; jj < P.ntn; ++jj, ++t) {
      const int64_t j = (i & 1) ? (P.ntn - 1 - jj) : jj;  // snake order: reuse the last B tiles
      const int64_t nj = extent(P.n, P.tn, j), c0 = j * P.tn;
      const int sidx = (int)(t % ns);
      cudaStream_t s = ctx->streams[sidx];
      char* ct;
      int64_t ldct;
      tmm::CSlot* cs = nullptr;
      if (copy_back) {
        cs = &ctx->cslots[(size_t)sidx * 2 + (size_t)((t / ns) & 1)];
        if (cs->used) TMM_CUDA(ctx, cudaStreamWaitEvent(s, cs->done, 0));
        ct = cs->ptr;
        ldct = mi;
      } else {
        ct = (char*)ctx->full_c.ptr + ((size_t)r0 + (size_t)c0 * (size_t)P.m) * P.es;
        ldct = P.m;
      }
      if (beta_nz) {  // the C tile is read only when beta != 0 (tiled_mm.cpp:325-330, 425-431)
        st = copy2d(ctx, ct, (size_t)ldct * P.es, Ch + ((size_t)r0 + (size_t)c0 * (size_t)ldc) * P.es,
                    (size_t)ldc * P.es, (size_t)mi * P.es, (size_t)nj, s, c_direct);
        if (st) return st;
        ctx->stats.h2d_bytes += (uint64_t)mi * (uint64_t)nj * P.es;
      }
      if (P.ntk == 0) {
        st = launch_tile_gemm(ctx, P.opa, P.opb, mi, nj, 0, alpha, nullptr, 1, nullptr, 1, beta, ct, ldct, s);
        if (st) return st;
      }
      for (int64_t kt = 0; kt < P.ntk; ++kt) {
        const int64_t kk = extent(P.k, P.tk, kt), k0 = kt * P.tk;
        int sa = -1, sb = -1;
        // A tile (i, kt): stored block rows/cols depend on op(A)
        if (P.opa == tmm::OP_N)
          st = fetch_tile(ctx, P, ctx->cache_a, i * P.ntk + kt, A, r0, k0, mi, kk, true, &sa, &staging_turn, s);
        else
          st = fetch_tile(ctx, P, ctx->cache_a, i * P.ntk + kt, A, k0, r0, kk, mi, false, &sa, &staging_turn, s);
        if (st) return st;
        if (P.opb == tmm::OP_N)
          st = fetch_tile(ctx, P, ctx->cache_b, kt * P.ntn + j, B, k0, c0, kk, nj, false, &sb, &staging_turn, s);
        else
          st = fetch_tile(ctx, P, ctx->cache_b, kt * P.ntn + j, B, c0, k0, nj, kk, true, &sb, &staging_turn, s);
        if (st) return st;
        tmm::Slot& SA = ctx->cache_a.slots[sa];
        tmm::Slot& SB = ctx->cache_b.slots[sb];
        TMM_CUDA(ctx, cudaStreamWaitEvent(s, SA.ready, 0));
        TMM_CUDA(ctx, cudaStreamWaitEvent(s, SB.ready, 0));
        const void* bk = kt == 0 ? beta : (const void*)one;
        if (!P.ozaki) {
          const int64_t lda_t = P.opa == tmm::OP_N ? mi : kk;
          const int64_t ldb_t = P.opb == tmm::OP_N ? kk : nj;
          st = P.embed ? embedded_ozaki(ctx, P.opa, P.opb, mi, nj, kk, alpha, SA.ptr, lda_t, SB.ptr, ldb_t, bk, ct, ldct, s,
                                    sidx)
                    : launch_tile_gemm(ctx, P.opa, P.opb, mi, nj, kk, alpha, SA.ptr, lda_t, SB.ptr, ldb_t, bk, ct, ldct, s);
          if (st) return st;
        } else {
          tmm::OzakiSplit va = tmm::ozaki_split_view(SA.ptr, mi, kk, P.slices, P.engine);
          tmm::OzakiSplit vb = tmm::ozaki_split_view(SB.ptr, nj, kk, P.slices, P.engine);
          KernelTimer timer(ctx, s);
          cudaError_t e = tmm::ozaki_gemm(va, vb, mi, nj, *(const double*)alpha, *(const double*)beta, kt == 0,
                                          (double*)ct, ldct, P.engine, oz_workspace(ctx, sidx), oz_error_word(ctx), s);
          timer.done();
          if (e != cudaSuccess) return cuda_fail(ctx, e, "ozaki gemm launch");
          ctx->stats.kernels++;
        }
        TMM_CUDA(ctx, cudaEventRecord(SA.last_use, s));
        TMM_CUDA(ctx, cudaEventRecord(SB.last_use, s));
        SA.used = SB.used = true;
      }
      if (copy_back) {  // result stream copies the finished tile back (tiled_mm.cpp:350-358)
        TMM_CUDA(ctx, cudaEventRecord(cs->done, s));
        TMM_CUDA(ctx, cudaStreamWaitEvent(ctx->d2h, cs->done, 0));
        st = copy2d(ctx, (char*)c + ((size_t)r0 + (size_t)c0 * (size_t)ldc) * P.es, (size_t)ldc * P.es, ct,
                    (size_t)ldct * P.es, (size_t)mi * P.es, (size_t)nj, ctx->d2h, c_direct);
        if (st) return st;
        TMM_CUDA(ctx, cudaEventRecord(cs->done, ctx->d2h));
        cs->used = true;
        ctx->stats.d2h_bytes += (uint64_t)mi * (uint64_t)nj * P.es;
      }
    }
  }
  return TMM_SUCCESS;
}

int sync_all(tmm_context* ctx) {
  cudaError_t first = cudaSuccess;
  for (auto s : ctx->streams) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (first == cudaSuccess) first = e;
  }
  for (cudaStream_t s : {ctx->h2d, ctx->prep, ctx->d2h}) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (first == cudaSuccess) first = e;
  }
  if (first != cudaSuccess) return cuda_fail(ctx, first, "stream synchronize");
  return TMM_SUCCESS;
}

}  // namespace

// tmm_gemm on device-resident (or managed) operands: the device entry on the first context
// stream, then a sync.  copy_c_back == false keeps its meaning: the result goes to the
// compact full-C buffer (beta * C read from c) and c is not written.
static int gemm_resident(tmm_context* ctx, char trans_a, char trans_b, int64_t m, int64_t n, int64_t k, const void* alpha,
                  const void* a, int64_t ld_a, const void* b, int64_t ld_b, const void* beta, void* c, int64_t ld_c,
                  bool copy_back, std::chrono::steady_clock::time_point t0) {
  cudaStream_t s = ctx->streams[0];
  void* dst = c;
  int64_t ld_dst = ld_c;
  const size_t es = elem_size(ctx->dtype);
  if (!copy_back) {
    TMM_CUDA(ctx, ctx->full_c.reserve((size_t)m * (size_t)n * es));
    ctx->full_c_elems = (size_t)m * (size_t)n;
    if (!is_zero(ctx->dtype, beta))
      TMM_CUDA(ctx, cudaMemcpy2DAsync(ctx->full_c.ptr, (size_t)m * es, c, (size_t)ld_c * es, (size_t)m * es, (size_t)n,
                                      cudaMemcpyDefault, s));
    dst = ctx->full_c.ptr;
    ld_dst = m;
  }
  int st = tmm_gemm_device(ctx, trans_a, trans_b, m, n, k, alpha, a, ld_a, b, ld_b, beta, dst, ld_dst, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  if (!st && e != cudaSuccess) st = cuda_fail(ctx, e, "cudaStreamSynchronize");
  if (!st && ctx->path == TMM_PATH_OZAKI) st = check_oz_error(ctx);
  ctx->stats.tile_m = (int)std::min<int64_t>(m, INT32_MAX);
  ctx->stats.tile_n = (int)std::min<int64_t>(n, INT32_MAX);
  ctx->stats.tile_k = (int)std::min<int64_t>(std::max<int64_t>(k, 1), ctx->max_tile_k);
  ctx->stats.n_streams = 1;
  ctx->stats.path = (ctx->path == TMM_PATH_OZAKI && ctx->dtype == TMM_DOUBLE) ? TMM_PATH_OZAKI : TMM_PATH_NATIVE;
  ctx->stats.ozaki_slices = ctx->stats.path == TMM_PATH_OZAKI
                                ? (ctx->ozaki_slices > 0 ? ctx->ozaki_slices : tmm::oz_default_slices(ctx->dtype)) : 0;
  ctx->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

extern "C" int tmm_device_status(tmm_context* ctx, void* stream) {
  if (!ctx) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_device_status: null context");
  DeviceGuard dg(ctx->device);
  TMM_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
  int st = check_oz_error(ctx);
  if (!st) st = check_f32_error(ctx);
  return st;
}

extern "C" int tmm_gemm(tmm_context* ctx, char trans_a, char trans_b, int64_t m, int64_t n, int64_t k,
                        const void* alpha, const void* a, int64_t ld_a, const void* b, int64_t ld_b,
                        const void* beta, void* c, int64_t ld_c, int pin_host_buffers, int copy_c_back) {
  if (!ctx) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: null context");
  auto t0 = std::chrono::steady_clock::now();
  ctx->stats = tmm_stats{};
  ctx->stats.direct_host = ctx->direct_host ? 1 : 0;
  Plan P{};
  if (!parse_op(trans_a, ctx->dtype, &P.opa) || !parse_op(trans_b, ctx->dtype, &P.opb))
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: trans must be one of N, T, C");
  if (m < 0 || n < 0 || k < 0) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: negative size");
  if (!alpha || !beta) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: null alpha or beta");
  const int64_t a_rows = P.opa == tmm::OP_N ? m : k, a_cols = P.opa == tmm::OP_N ? k : m;
  const int64_t b_rows = P.opb == tmm::OP_N ? k : n, b_cols = P.opb == tmm::OP_N ? n : k;
  // leading-dimension checks of src/Tiled-MM/tiled_mm.cpp:516-527, enforced here
  if (ld_a < std::max<int64_t>(1, a_rows)) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: ld_a < rows of A");
  if (ld_b < std::max<int64_t>(1, b_rows)) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: ld_b < rows of B");
  if (ld_c < std::max<int64_t>(1, m)) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: ld_c < rows of C");
  if (m == 0 || n == 0) return TMM_SUCCESS;
  const bool beta_nz = !is_zero(ctx->dtype, beta);
  if ((k > 0 && (!a || !b)) || ((copy_c_back || beta_nz) && !c))
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm: null matrix pointer");
  const bool ozaki = ctx->path == TMM_PATH_OZAKI && ctx->dtype == TMM_DOUBLE;
  DeviceGuard dg(ctx->device);

  // ---- every operand already device-accessible: no host link, no pinning, no tiling of m, n
  const bool c_used = copy_c_back || beta_nz;
  if ((k == 0 || (device_accessible(a) && device_accessible(b))) && (!c_used || device_accessible(c)))
    return gemm_resident(ctx, trans_a, trans_b, m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c, copy_c_back != 0,
                         t0);

  // ---- tile sizes (src/Tiled-MM/tiled_mm.cpp:557-560)
  int tm, tn, tk;
  tmm::TuneProblem tune{};
  int tune_index = -1;
  if (ctx->tile_policy == TMM_TILE_POLICY_REFERENCE) {
    tm = optimal_tile_size(m, ctx->cur_tile_m, ctx->max_tile_m);
    tn = optimal_tile_size(n, ctx->cur_tile_n, ctx->max_tile_n);
    tk = optimal_tile_size(std::max<int64_t>(k, 1), ctx->cur_tile_k, ctx->max_tile_k);
  } else if (ctx->tile_policy == TMM_TILE_POLICY_AUTOTUNE) {
    size_t freeb = 0, total = 0;
    if (cudaMemGetInfo(&freeb, &total) != cudaSuccess) return cuda_fail(ctx, cudaGetLastError(), "cudaMemGetInfo");
    size_t budget = freeb + ctx->pool_a.capacity + ctx->pool_b.capacity + ctx->pool_c.capacity + ctx->staging.capacity;
    if (ctx->memory_limit) budget = std::min(budget, ctx->memory_limit);
    tune.dtype = ctx->dtype;
    tune.path = ctx->path;
    tune.engine = ctx->path == TMM_PATH_OZAKI ? ctx->oz_engine : 0;
    tune.slices = ctx->path == TMM_PATH_OZAKI ? (ctx->ozaki_slices > 0 ? ctx->ozaki_slices
                                                                      : tmm::oz_default_slices(ctx->dtype)) : 0;
    tune.m = m;
    tune.n = n;
    tune.k = k;
    tune.ta = trans_a;
    tune.tb = trans_b;
    tune.pinned = pin_host_buffers ? 1 : 0;
    tune.copy_back = copy_c_back ? 1 : 0;
    tune.budget = budget;
    tune.max_tm = ctx->max_tile_m;
    tune.max_tn = ctx->max_tile_n;
    tune.max_tk = ctx->max_tile_k;
    const tmm::TileChoice tc = tmm::autotune_pick(tune, &tune_index, &ctx->stats.autotune_state);
    ctx->last_tune = tune;
    ctx->has_tune = true;
    tm = tc.tm;
    tn = tc.tn;
    tk = tc.tk;
    if (tc.streams > ctx->n_streams) {
      int st0 = tmm_set_num_streams(ctx, tc.streams);
      if (st0) return st0;
    }
  } else {
    tm = (int)std::min<int64_t>(m, ctx->max_tile_m);
    tn = (int)std::min<int64_t>(n, ctx->max_tile_n);
    tk = (int)std::min<int64_t>(std::max<int64_t>(k, 1), ctx->max_tile_k);
  }
  ctx->cur_tile_m = tm;
  ctx->cur_tile_n = tn;
  ctx->cur_tile_k = tk;
  P.m = m; P.n = n; P.k = k; P.tm = tm; P.tn = tn; P.tk = tk;
  P.ntm = ntiles(m, tm); P.ntn = ntiles(n, tn); P.ntk = ntiles(k, tk);
  P.es = elem_size(ctx->dtype);
  P.ozaki = ozaki;
  P.embed = ctx->path == TMM_PATH_OZAKI && tmm::ozaki_embedded_dtype(ctx->dtype);
  P.slices = ctx->ozaki_slices > 0 ? ctx->ozaki_slices : tmm::oz_default_slices(ctx->dtype);
  P.engine = ctx->oz_engine;
  if (ozaki) {
    P.a_slot_bytes = tmm::ozaki_split_bytes(tm, tk, P.slices);
    P.b_slot_bytes = tmm::ozaki_split_bytes(tn, tk, P.slices);
    P.staging_bytes = (size_t)std::max(tm, tn) * (size_t)tk * 8;
  } else {
    P.a_slot_bytes = (size_t)tm * (size_t)tk * P.es;
    P.b_slot_bytes = (size_t)tk * (size_t)tn * P.es;
    P.staging_bytes = 0;
  }
  P.c_slot_bytes = (size_t)tm * (size_t)tn * P.es;

  // ---- pin (src/Tiled-MM/tiled_mm.cpp:529-554)
  Pin pa, pb, pc;
  int st = TMM_SUCCESS;
  if (pin_host_buffers) {
    if (k > 0) {
      st = pin_range(ctx, a, ((size_t)ld_a * (size_t)(a_cols - 1) + (size_t)a_rows) * P.es, &pa);
      if (!st) st = pin_range(ctx, b, ((size_t)ld_b * (size_t)(b_cols - 1) + (size_t)b_rows) * P.es, &pb);
    }
    if (!st && (copy_c_back || beta_nz))
      st = pin_range(ctx, c, ((size_t)ld_c * (size_t)(n - 1) + (size_t)m) * P.es, &pc);
  }
  ctx->stats.tile_m = tm;
  ctx->stats.tile_n = tn;
  ctx->stats.tile_k = tk;
  ctx->stats.n_streams = (int)std::min<int64_t>(ctx->n_streams, P.ntm * P.ntn);
  ctx->stats.path = (ozaki || P.embed) ? TMM_PATH_OZAKI : TMM_PATH_NATIVE;
  ctx->stats.ozaki_slices = (ozaki || P.embed) ? P.slices : 0;
  if (!st) st = run_gemm(ctx, P, alpha, a, ld_a, b, ld_b, beta, c, ld_c, copy_c_back != 0);
  int st2 = sync_all(ctx);  // returns with C final (the reference syncs the device: tiled_mm.cpp:602-604)
  if (!st) st = st2;
  if (!st && (ozaki || P.embed)) st = check_oz_error(ctx);
  if (!st && (ctx->dtype == TMM_FLOAT || ctx->dtype == TMM_COMPLEX_FLOAT)) st = check_f32_error(ctx);
  unpin(pa);
  unpin(pb);
  unpin(pc);
  ctx->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!st && tune_index >= 0) tmm::autotune_report(tune, tune_index, ctx->stats.seconds);
  return st;
}

extern "C" int tmm_get_autotune_report(tmm_context* ctx, char* text, size_t capacity) {
  if (!ctx || !text || capacity == 0) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_get_autotune_report: bad argument");
  const std::string r = ctx->has_tune ? tmm::autotune_explain(ctx->last_tune)
                                      : std::string("no call of this context used the autotuner");
  const size_t len = std::min(r.size(), capacity - 1);
  memcpy(text, r.data(), len);
  text[len] = 0;
  return TMM_SUCCESS;
}

extern "C" int tmm_gemm_device(tmm_context* ctx, char trans_a, char trans_b, int64_t m, int64_t n, int64_t k,
                               const void* alpha, const void* a, int64_t ld_a, const void* b, int64_t ld_b,
                               const void* beta, void* c, int64_t ld_c, void* stream) {
  if (!ctx) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_device: null context");
  ctx->stats = tmm_stats{};
  ctx->stats.direct_host = ctx->direct_host ? 1 : 0;
  Op opa, opb;
  if (!parse_op(trans_a, ctx->dtype, &opa) || !parse_op(trans_b, ctx->dtype, &opb))
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_device: trans must be one of N, T, C");
  if (m < 0 || n < 0 || k < 0 || !alpha || !beta)
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_device: bad size or scalar");
  const int64_t a_rows = opa == tmm::OP_N ? m : k, b_rows = opb == tmm::OP_N ? k : n;
  if (ld_a < std::max<int64_t>(1, a_rows) || ld_b < std::max<int64_t>(1, b_rows) || ld_c < std::max<int64_t>(1, m))
    return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_device: leading dimension too small");
  if (m == 0 || n == 0) return TMM_SUCCESS;
  if ((k > 0 && (!a || !b)) || !c) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_device: null matrix pointer");
  DeviceGuard dg(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream, as everywhere in CUDA
  if (ctx->path == TMM_PATH_OZAKI && ctx->dtype == TMM_DOUBLE && k > 0) {
    // split op(A) and op(B) in k-tiles of at most tile_k (per-k-tile scaling) into scratch, then multiply
    const int slices = ctx->ozaki_slices > 0 ? ctx->ozaki_slices : tmm::oz_default_slices(ctx->dtype);
    const int64_t tk = std::min<int64_t>(k, ctx->max_tile_k);
    const size_t sa = tmm::ozaki_split_bytes(m, tk, slices), sb = tmm::ozaki_split_bytes(n, tk, slices);
    const size_t sa_al = (sa + 255) / 256 * 256;
    TMM_CUDA(ctx, ctx->scratch.reserve(sa_al + sb));
    int st = reserve_oz_work(ctx, 1);
    if (st) return st;
    for (int64_t k0 = 0, kt = 0; k0 < k; k0 += tk, ++kt) {
      const int64_t kk = std::min(tk, k - k0);
      tmm::OzakiSplit va = tmm::ozaki_split_view(ctx->scratch.ptr, m, kk, slices, ctx->oz_engine);
      tmm::OzakiSplit vb = tmm::ozaki_split_view((char*)ctx->scratch.ptr + sa_al, n, kk, slices, ctx->oz_engine);
      const double* ab = opa == tmm::OP_N ? (const double*)a + k0 * ld_a : (const double*)a + k0;
      const double* bb = opb == tmm::OP_N ? (const double*)b + k0 : (const double*)b + k0 * ld_b;
      cudaError_t e = tmm::ozaki_split(ab, ld_a, opa == tmm::OP_N ? tmm::OP_N : tmm::OP_T, m, kk, va, s);
      if (e == cudaSuccess) e = tmm::ozaki_split(bb, ld_b, opb == tmm::OP_N ? tmm::OP_T : tmm::OP_N, n, kk, vb, s);
      if (e == cudaSuccess) {
        KernelTimer timer(ctx, s);
        e = tmm::ozaki_gemm(va, vb, m, n, *(const double*)alpha, *(const double*)beta, kt == 0, (double*)c, ld_c,
                            ctx->oz_engine, oz_workspace(ctx, 0), oz_error_word(ctx), s);
        timer.done();
      }
      if (e != cudaSuccess) return cuda_fail(ctx, e, "ozaki device gemm launch");
      ctx->stats.kernels += 5;  // two two-kernel splits and the product
    }
    return TMM_SUCCESS;
  }
  if (ctx->path == TMM_PATH_OZAKI && tmm::ozaki_embedded_dtype(ctx->dtype)) {
    int st = reserve_oz_work(ctx, 1);
    if (st) return st;
    return embedded_ozaki(ctx, opa, opb, m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c, s, 0);
  }
  return launch_tile_gemm(ctx, opa, opb, m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c, s);
}

// ------------------------------------------------------------------ utilities
extern "C" int tmm_malloc_pinned(size_t bytes, void** p) {
  if (!p) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_malloc_pinned: null output");
  cudaError_t e = cudaHostAlloc(p, bytes ? bytes : 1, cudaHostAllocDefault);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaHostAlloc");
  return TMM_SUCCESS;
}
extern "C" int tmm_free_pinned(void* p) {
  if (!p) return TMM_SUCCESS;
  cudaError_t e = cudaFreeHost(p);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaFreeHost");
  return TMM_SUCCESS;
}
extern "C" int tmm_copy_to_device(const void* h, void* d, size_t bytes) {
  cudaError_t e = cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemcpy H2D");
  return TMM_SUCCESS;
}
extern "C" int tmm_copy_to_host(const void* d, void* h, size_t bytes) {
  cudaError_t e = cudaMemcpy(h, d, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemcpy D2H");
  return TMM_SUCCESS;
}
extern "C" int tmm_memcpy_async(void* dst, const void* src, size_t bytes, void* stream) {
  if ((!dst || !src) && bytes) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_memcpy_async: null pointer");
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemcpyAsync");
  return TMM_SUCCESS;
}
extern "C" int tmm_malloc_device(size_t bytes, void** p) {
  if (!p) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_malloc_device: null output");
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  return TMM_SUCCESS;
}
extern "C" int tmm_free_device(void* p) {
  if (!p) return TMM_SUCCESS;
  cudaError_t e = cudaFree(p);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaFree");
  return TMM_SUCCESS;
}

extern "C" int tmm_fill_host_f64(double* x, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                                 uint64_t seed, uint64_t id, int n_threads) {
  if (!x || rows < 0 || cols < 0 || ld < rows) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_fill_host_f64: bad arguments");
  if (n_threads < 1) n_threads = 1;
  auto work = [&](int t) {
    int64_t c0 = cols * t / n_threads, c1 = cols * (t + 1) / n_threads;
    for (int64_t j = c0; j < c1; ++j)
      for (int64_t i = 0; i < rows; ++i) x[i + j * ld] = tmm_gen_value(kind, param, seed, id, i, j, rows);
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& h : th) h.join();
  return TMM_SUCCESS;
}

extern "C" int tmm_fill_device_f64(double* x, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                                   uint64_t seed, uint64_t id, void* stream) {
  if (!x || rows < 0 || cols < 0 || ld < rows) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_fill_device_f64: bad arguments");
  cudaError_t e = tmm::launch_fill_f64(x, rows, cols, ld, kind, param, seed, id, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "fill kernel launch");
  return TMM_SUCCESS;
}

// Compensated dot products (TwoSum / TwoProduct, Ogita-Rump-Oishi 2005) over
// sampled entries: the FP64-oracle error metric reported with every result.
extern "C" int tmm_error_metric_f64(char trans_a, char trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                                    const double* a, int64_t lda, const double* b, int64_t ldb, double beta,
                                    const double* c0, int64_t ldc0, const double* c, int64_t ldc, int64_t ns,
                                    uint64_t seed, int n_threads, double* metric) {
  if (!metric || !c || m <= 0 || n <= 0 || k < 0 || ns <= 0 || (k > 0 && (!a || !b)) || (beta != 0.0 && !c0))
    return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_error_metric_f64: bad arguments");
  const bool ta = upper(trans_a) != 'N', tb = upper(trans_b) != 'N';
  if (n_threads < 1) n_threads = 1;
  std::vector<double> worst(n_threads, 0.0);
  auto work = [&](int t) {
    for (int64_t s = t; s < ns; s += n_threads) {
      uint64_t h = tmm_splitmix64(seed ^ (uint64_t)s * 0x9E3779B97F4A7C15ull);
      int64_t i = (int64_t)(h % (uint64_t)m), j = (int64_t)((h >> 32) % (uint64_t)n);
      if (s == 0) { i = 0; j = 0; }
      if (s == 1) { i = m - 1; j = n - 1; }
      double sum = 0, err = 0, mag = 0;
      for (int64_t l = 0; l < k; ++l) {
        double x = ta ? a[l + i * lda] : a[i + l * lda];
        double y = tb ? b[j + l * ldb] : b[l + j * ldb];
        double p = x * y, pe = std::fma(x, y, -p);
        double s2 = sum + p, z = s2 - sum, se = (sum - (s2 - z)) + (p - z);
        sum = s2;
        err += pe + se;
        mag += std::fabs(x) * std::fabs(y);
      }
      double hi = alpha * sum, lo = std::fma(alpha, sum, -hi) + alpha * err;
      mag *= std::fabs(alpha);
      if (beta != 0.0) {
        double cv = c0[i + j * ldc0];
        double p = beta * cv, pe = std::fma(beta, cv, -p);
        double s2 = hi + p, z = s2 - hi, se = (hi - (s2 - z)) + (p - z);
        hi = s2;
        lo += se + pe;
        mag += std::fabs(beta) * std::fabs(cv);
      }
      double ref = hi + lo, got = c[i + j * ldc];
      double d = std::fabs(got - ref);
      double r;
      if (d != d) r = INFINITY;
      else if (mag == 0) r = d == 0 ? 0.0 : INFINITY;
      else r = d / ((double)std::max<int64_t>(k, 1) * 1.1102230246251565e-16 * mag);
      if (r > worst[t] || r != r) worst[t] = r;
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& h : th) h.join();
  double w = 0;
  for (double v : worst) w = std::max(w, v);
  *metric = w;
  return TMM_SUCCESS;
}

// ------------------------------------------------------------------ batched path
namespace {

bool page_locked(const void* p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeHost;
}

void drop_batch_graph(tmm_context* ctx) {
  if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
  ctx->batch_exec = nullptr;
  ctx->batch_key.clear();
}

// FP64 problems of a batch on the Ozaki path (context path TMM_PATH_OZAKI).  Each problem is
// split per k tile of at most max_tile_k, as tmm_gemm_device does, so each result equals that
// call's bit for bit; the split planes of all problems live in one arena, and the tcgen05 engine
// multiplies every problem of a chunk in one persistent launch over their tiles
// (ozaki_gemm_tc_grouped).  The problems are cut into chunks of about equal work; with host
// operands, chunk c's copies in run on a copy stream, its splits and grouped launches on a
// compute stream once they have landed, and its copies out on a third stream, so the host
// link in both directions overlaps the products of the other chunks.  The three streams fork
// from the batch stream and join it.  The IMMA engine runs the same pipeline with one launch
// per problem and k tile.
constexpr int BATCH_OZ_CHUNKS = 4;
constexpr int BATCH_OZ_SPLIT_STREAMS = 4;

struct BatchOzRound {  // one grouped launch: the chunk's problems that have a k tile r
  int chunk, round, n_probs, n_items;
  size_t image_off;  // its device records in the batch scratch
};
struct BatchOzPlan {
  std::vector<int> ids;                 // FP64 problems on the engine
  std::vector<int64_t> tk;              // per id: k tile
  std::vector<size_t> a_off, b_off;     // per id: split planes in the arena
  std::vector<int> chunk_of;            // per id
  std::vector<std::vector<int>> chunks;  // positions in ids, per chunk
  std::vector<BatchOzRound> launches;
  int slices = 0;
  size_t work_off = 0, arena_off = 0, arena_bytes = 0;
  int kernels = 0;
};

// slice count of a batch problem's precision: the context's own count for problems of its
// precision, the precision's default for the others
int batch_slices(const tmm_context* ctx, int dtype) {
  const bool ctx_single = ctx->dtype == TMM_FLOAT || ctx->dtype == TMM_COMPLEX_FLOAT;
  const bool single = dtype == TMM_FLOAT;
  return ctx->ozaki_slices > 0 && ctx_single == single ? ctx->ozaki_slices : tmm::oz_default_slices(dtype);
}

// the split views of problem position j of the plan for k tile kt
void batch_oz_views(const tmm_context* ctx, const BatchOzPlan& plan, const tmm::BatchProblem& d, size_t j, int64_t kt,
                    tmm::OzakiSplit* va, tmm::OzakiSplit* vb) {
  char* arena = (char*)ctx->batch_oz_scratch.ptr + plan.arena_off;
  const int64_t kk = std::min(plan.tk[j], d.k - kt * plan.tk[j]);
  *va = tmm::ozaki_split_view(arena + plan.a_off[j], d.m, kk, plan.slices, ctx->oz_engine);
  *vb = tmm::ozaki_split_view(arena + plan.b_off[j], d.n, kk, plan.slices, ctx->oz_engine);
}

int plan_batch_ozaki(tmm_context* ctx, const std::vector<tmm::BatchProblem>& dev, const std::vector<int>& ids,
                     BatchOzPlan* plan, bool* moved) {
  *plan = BatchOzPlan{};
  *moved = false;
  if (ids.empty()) return TMM_SUCCESS;
  BatchOzPlan& P = *plan;
  P.ids = ids;
  P.slices = batch_slices(ctx, TMM_DOUBLE);
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  // arena: both operands' planes of every problem for one k tile
  size_t arena = 0;
  std::vector<double> cost;
  for (int id : ids) {
    const tmm::BatchProblem& d = dev[(size_t)id];
    const int64_t tk = std::min<int64_t>(d.k, ctx->max_tile_k);
    P.tk.push_back(tk);
    P.a_off.push_back(arena);
    arena += up(tmm::ozaki_split_bytes(d.m, tk, P.slices));
    P.b_off.push_back(arena);
    arena += up(tmm::ozaki_split_bytes(d.n, tk, P.slices));
    cost.push_back((double)d.m * (double)d.n * (double)d.k);
  }
  // chunks of about equal work, in problem order
  const double total = std::accumulate(cost.begin(), cost.end(), 0.0);
  const int nch = std::min<int>(BATCH_OZ_CHUNKS, (int)ids.size());
  P.chunks.assign((size_t)nch, {});
  double acc = 0.0;
  for (size_t j = 0; j < ids.size(); ++j) {
    const int c = std::min(nch - 1, (int)(acc / total * nch));
    P.chunks[(size_t)c].push_back((int)j);
    P.chunk_of.push_back(c);
    acc += cost[j];
  }
  P.work_off = 0;
  const size_t work = up(tmm::ozaki_workspace_bytes(ctx->oz_engine));
  P.arena_off = work;
  P.arena_bytes = arena;
  // the grouped launches' device records, per chunk and k-tile round
  std::vector<unsigned char> images;
  void* before = ctx->batch_oz_scratch.ptr;
  // the records hold device addresses inside the scratch: size it first, then build them
  for (int pass = 0; pass < 2; ++pass) {
    images.clear();
    P.launches.clear();
    P.kernels = 0;
    for (int c = 0; c < nch; ++c) {
      int rounds = 0;
      for (int j : P.chunks[(size_t)c]) {
        const tmm::BatchProblem& d = dev[(size_t)ids[(size_t)j]];
        rounds = std::max<int>(rounds, (int)((d.k + P.tk[(size_t)j] - 1) / P.tk[(size_t)j]));
      }
      for (int r = 0; r < rounds; ++r) {
        std::vector<tmm::GroupedProduct> prods;
        for (int j : P.chunks[(size_t)c]) {
          const tmm::BatchProblem& d = dev[(size_t)ids[(size_t)j]];
          if ((int64_t)r * P.tk[(size_t)j] >= d.k) continue;
          tmm::GroupedProduct g;
          batch_oz_views(ctx, P, d, (size_t)j, r, &g.A, &g.B);
          g.m = d.m;
          g.n = d.n;
          g.alpha = d.alpha;
          g.beta = d.beta;
          g.first_k_tile = r == 0;
          g.C = (double*)d.c;
          g.ldc = d.ldc;
          prods.push_back(g);
          P.kernels += 4;  // two two-kernel splits
        }
        BatchOzRound L{c, r, (int)prods.size(), 0, P.arena_off + P.arena_bytes + images.size()};
        if (ctx->oz_engine == tmm::OZ_ENGINE_TCGEN05 && pass == 1) {
          std::vector<unsigned char> img;
          cudaError_t e = tmm::ozaki_tc_grouped_image(prods, (char*)ctx->batch_oz_scratch.ptr + P.arena_off,
                                                      P.arena_bytes, img, &L.n_items);
          if (e != cudaSuccess) return cuda_fail(ctx, e, "batched ozaki plan");
          images.insert(images.end(), img.begin(), img.end());
          images.resize(up(images.size()));
        } else if (ctx->oz_engine == tmm::OZ_ENGINE_TCGEN05) {
          // sizes only: records and tiles of this launch
          size_t tiles = 0;
          for (const auto& g : prods) tiles += (size_t)((g.m + 127) / 128) * (size_t)((g.n + 255) / 256);
          images.resize(up(images.size() + up(prods.size() * 256) + tiles * 16));
        }
        P.kernels += ctx->oz_engine == tmm::OZ_ENGINE_TCGEN05 ? 1 : (int)prods.size();
        P.launches.push_back(L);
      }
    }
    if (pass == 0) TMM_CUDA(ctx, ctx->batch_oz_scratch.reserve(P.arena_off + P.arena_bytes + images.size() + 256));
  }
  *moved = ctx->batch_oz_scratch.ptr != before;
  if (!images.empty())
    TMM_CUDA(ctx, cudaMemcpy((char*)ctx->batch_oz_scratch.ptr + P.arena_off + P.arena_bytes, images.data(),
                             images.size(), cudaMemcpyHostToDevice));
  void* wbefore = ctx->oz_work.ptr;
  int st = reserve_oz_work(ctx, 0);  // the error word; the workspace is in the batch scratch
  if (st) return st;
  if (ctx->oz_work.ptr != wbefore) *moved = true;
  if (!ctx->oz_fork) TMM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->oz_fork, cudaEventDisableTiming));
  // products, copies in, copies out, the split streams
  while (ctx->oz_branches.size() < 3 + (size_t)BATCH_OZ_SPLIT_STREAMS) {
    cudaStream_t bs;
    TMM_CUDA(ctx, cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    ctx->oz_branches.push_back(bs);
  }
  // per chunk: copies landed, products done; the joins; the split fork and joins; the copies
  // of the batch's other problems
  while (ctx->oz_branch_done.size() < 2 * (size_t)BATCH_OZ_CHUNKS + 4 + (size_t)BATCH_OZ_SPLIT_STREAMS) {
    cudaEvent_t ev;
    TMM_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->oz_branch_done.push_back(ev);
  }
  TMM_CUDA(ctx, tmm::ozaki_prepare(ctx->oz_engine));
  return TMM_SUCCESS;
}

// operands of problem d from the caller's host buffers into the arena, and C back
// A column-major block of `cols` columns of `width` bytes between pitches dpitch and spitch:
// one plain copy when both sides are contiguous (the copy engines move a 2D copy row by row,
// and batch problems with short columns -- 64 rows of a float are 256 bytes -- crawl that
// way), else a 2D copy.
cudaError_t copy_block(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t cols,
                       cudaMemcpyKind kind, cudaStream_t s) {
  if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * cols, kind, s);
  return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, cols, kind, s);
}

int copy_problem_in(tmm_context* ctx, const tmm_batch_problem& h, const tmm::BatchProblem& d, cudaStream_t s) {
  const size_t es = h.dtype == TMM_DOUBLE ? 8 : 4;
  if (d.m == 0 || d.n == 0) return TMM_SUCCESS;
  if (d.k > 0) {
    const int64_t ar = d.opa == tmm::OP_N ? d.m : d.k, ac = d.opa == tmm::OP_N ? d.k : d.m;
    const int64_t br = d.opb == tmm::OP_N ? d.k : d.n, bc = d.opb == tmm::OP_N ? d.n : d.k;
    TMM_CUDA(ctx, copy_block((void*)d.a, (size_t)ar * es, h.a, (size_t)h.ld_a * es, (size_t)ar * es, (size_t)ac,
                             cudaMemcpyHostToDevice, s));
    TMM_CUDA(ctx, copy_block((void*)d.b, (size_t)br * es, h.b, (size_t)h.ld_b * es, (size_t)br * es, (size_t)bc,
                             cudaMemcpyHostToDevice, s));
    ctx->stats.h2d_bytes += (uint64_t)(ar * ac + br * bc) * es;
  }
  if (h.beta != 0.0) {
    TMM_CUDA(ctx, copy_block(d.c, (size_t)d.m * es, h.c, (size_t)h.ld_c * es, (size_t)d.m * es, (size_t)d.n,
                             cudaMemcpyHostToDevice, s));
    ctx->stats.h2d_bytes += (uint64_t)(d.m * d.n) * es;
  }
  return TMM_SUCCESS;
}

int copy_problem_out(tmm_context* ctx, const tmm_batch_problem& h, const tmm::BatchProblem& d, cudaStream_t s) {
  const size_t es = h.dtype == TMM_DOUBLE ? 8 : 4;
  if (d.m == 0 || d.n == 0) return TMM_SUCCESS;
  TMM_CUDA(ctx, copy_block(h.c, (size_t)h.ld_c * es, d.c, (size_t)d.m * es, (size_t)d.m * es, (size_t)d.n,
                           cudaMemcpyDeviceToHost, s));
  ctx->stats.d2h_bytes += (uint64_t)(d.m * d.n) * es;
  return TMM_SUCCESS;
}

// Forks the pipeline's three streams from s and queues every chunk (see plan_batch_ozaki):
// with host operands (host != nullptr) copies in, splits and products, copies out;
// join_batch_ozaki makes s wait for the pipeline.
int enqueue_batch_ozaki(tmm_context* ctx, const std::vector<tmm::BatchProblem>& dev, const BatchOzPlan& plan,
                        cudaStream_t s, const tmm_batch_problem* host) {
  if (plan.ids.empty()) return TMM_SUCCESS;
  cudaStream_t cin = ctx->oz_branches[1], comp = ctx->oz_branches[0], cout = ctx->oz_branches[2];
  const size_t nch = plan.chunks.size();
  cudaEvent_t* ev_in = &ctx->oz_branch_done[0];
  cudaEvent_t* ev_done = &ctx->oz_branch_done[(size_t)BATCH_OZ_CHUNKS];
  cudaEvent_t ev_split_fork = ctx->oz_branch_done[2 * (size_t)BATCH_OZ_CHUNKS + 2];
  cudaEvent_t* ev_split_done = &ctx->oz_branch_done[2 * (size_t)BATCH_OZ_CHUNKS + 3];
  TMM_CUDA(ctx, cudaEventRecord(ctx->oz_fork, s));
  TMM_CUDA(ctx, cudaStreamWaitEvent(comp, ctx->oz_fork, 0));
  if (host) {
    TMM_CUDA(ctx, cudaStreamWaitEvent(cin, ctx->oz_fork, 0));
    TMM_CUDA(ctx, cudaStreamWaitEvent(cout, ctx->oz_fork, 0));
  }
  char* scratch = (char*)ctx->batch_oz_scratch.ptr;
  double* work = (double*)(scratch + plan.work_off);
  size_t li = 0;
  for (size_t c = 0; c < nch; ++c) {
    if (host) {
      for (int j : plan.chunks[c]) {
        const int id = plan.ids[(size_t)j];
        if (int st = copy_problem_in(ctx, host[id], dev[(size_t)id], cin)) return st;
      }
      TMM_CUDA(ctx, cudaEventRecord(ev_in[c], cin));
      TMM_CUDA(ctx, cudaStreamWaitEvent(comp, ev_in[c], 0));
    }
    for (; li < plan.launches.size() && plan.launches[li].chunk == (int)c; ++li) {
      const BatchOzRound& L = plan.launches[li];
      std::vector<std::pair<tmm::OzakiSplit, tmm::OzakiSplit>> views;
      std::vector<int> pos;
      // the splits of small problems are latency-bound kernels: they run on BATCH_OZ_SPLIT_STREAMS
      // streams forked from the compute stream and joined before the grouped launch
      TMM_CUDA(ctx, cudaEventRecord(ev_split_fork, comp));
      for (int q = 0; q < BATCH_OZ_SPLIT_STREAMS; ++q)
        TMM_CUDA(ctx, cudaStreamWaitEvent(ctx->oz_branches[3 + (size_t)q], ev_split_fork, 0));
      for (int j : plan.chunks[c]) {
        const tmm::BatchProblem& d = dev[(size_t)plan.ids[(size_t)j]];
        const int64_t k0 = (int64_t)L.round * plan.tk[(size_t)j];
        if (k0 >= d.k) continue;
        tmm::OzakiSplit va, vb;
        batch_oz_views(ctx, plan, d, (size_t)j, L.round, &va, &vb);
        const double* ab = d.opa == tmm::OP_N ? (const double*)d.a + k0 * d.lda : (const double*)d.a + k0;
        const double* bb = d.opb == tmm::OP_N ? (const double*)d.b + k0 : (const double*)d.b + k0 * d.ldb;
        cudaStream_t ss = ctx->oz_branches[3 + pos.size() % BATCH_OZ_SPLIT_STREAMS];
        cudaError_t e = tmm::ozaki_split(ab, d.lda, d.opa == tmm::OP_N ? tmm::OP_N : tmm::OP_T, d.m, va.kk, va, ss);
        if (e == cudaSuccess)
          e = tmm::ozaki_split(bb, d.ldb, d.opb == tmm::OP_N ? tmm::OP_T : tmm::OP_N, d.n, vb.kk, vb, ss);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "batched ozaki split");
        views.emplace_back(va, vb);
        pos.push_back(j);
      }
      for (int q = 0; q < BATCH_OZ_SPLIT_STREAMS; ++q) {
        TMM_CUDA(ctx, cudaEventRecord(ev_split_done[q], ctx->oz_branches[3 + (size_t)q]));
        TMM_CUDA(ctx, cudaStreamWaitEvent(comp, ev_split_done[q], 0));
      }
      cudaError_t e = cudaSuccess;
      if (ctx->oz_engine == tmm::OZ_ENGINE_TCGEN05) {
        e = tmm::ozaki_gemm_tc_grouped(scratch + plan.arena_off, plan.arena_bytes, plan.slices, scratch + L.image_off,
                                       L.n_probs, L.n_items, work, oz_error_word(ctx), comp);
      } else {
        for (size_t q = 0; q < views.size() && e == cudaSuccess; ++q) {
          const tmm::BatchProblem& d = dev[(size_t)plan.ids[(size_t)pos[q]]];
          e = tmm::ozaki_gemm(views[q].first, views[q].second, d.m, d.n, d.alpha, d.beta, L.round == 0, (double*)d.c,
                              d.ldc, ctx->oz_engine, work, oz_error_word(ctx), comp);
        }
      }
      if (e != cudaSuccess) return cuda_fail(ctx, e, "batched ozaki launch");
    }
    TMM_CUDA(ctx, cudaEventRecord(ev_done[c], comp));
    if (host) {
      TMM_CUDA(ctx, cudaStreamWaitEvent(cout, ev_done[c], 0));
      for (int j : plan.chunks[c]) {
        const int id = plan.ids[(size_t)j];
        if (int st = copy_problem_out(ctx, host[id], dev[(size_t)id], cout)) return st;
      }
    }
  }
  ctx->stats.kernels += plan.kernels;
  return TMM_SUCCESS;
}

int join_batch_ozaki(tmm_context* ctx, const BatchOzPlan& plan, cudaStream_t s, bool host) {
  if (plan.ids.empty()) return TMM_SUCCESS;
  cudaEvent_t* fin = &ctx->oz_branch_done[2 * (size_t)BATCH_OZ_CHUNKS];
  TMM_CUDA(ctx, cudaEventRecord(fin[0], ctx->oz_branches[0]));
  TMM_CUDA(ctx, cudaStreamWaitEvent(s, fin[0], 0));
  if (host) {
    TMM_CUDA(ctx, cudaEventRecord(fin[1], ctx->oz_branches[2]));
    TMM_CUDA(ctx, cudaStreamWaitEvent(s, fin[1], 0));
    // the copy-in stream's last work precedes the compute stream's (it waited on it)
  }
  return TMM_SUCCESS;
}

// FP32 problems of a batch on the FP32 tensor-core engine: their bf16 planes (the whole k of
// each problem) in one arena of the context's batch FP32 scratch, after its 256-byte error
// word, and the grouped launch's records after the planes.
struct BatchF32Plan {
  std::vector<int> ids;
  std::vector<size_t> a_off, b_off;  // plane offsets from the scratch base
  size_t arena_off = 256, arena_bytes = 0, image_off = 0;
  int n_probs = 0, n_items = 0;
};

int plan_batch_f32(tmm_context* ctx, const std::vector<tmm::BatchProblem>& dev, const std::vector<int>& ids,
                   BatchF32Plan* plan, bool* moved) {
  *plan = BatchF32Plan{};
  *moved = false;
  if (ids.empty()) return TMM_SUCCESS;
  BatchF32Plan& P = *plan;
  P.ids = ids;
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  size_t arena = 0;
  std::vector<tmm::F32GroupedProduct> prods;
  for (int id : ids) {
    const tmm::BatchProblem& d = dev[(size_t)id];
    P.a_off.push_back(P.arena_off + arena);
    arena += up(tmm::f32tc_plane_bytes(d.m, d.k));
    P.b_off.push_back(P.arena_off + arena);
    arena += up(tmm::f32tc_plane_bytes(d.n, d.k));
    prods.push_back(tmm::F32GroupedProduct{nullptr, nullptr, d.m, d.n, d.k, (float)d.alpha, (float)d.beta,
                                           (float*)d.c, d.ldc});
  }
  P.arena_bytes = arena;
  P.image_off = P.arena_off + arena;
  const bool fresh = ctx->batch_f32_scratch.capacity < P.image_off + up(tmm::f32tc_grouped_image_bound(prods));
  void* before = ctx->batch_f32_scratch.ptr;
  TMM_CUDA(ctx, ctx->batch_f32_scratch.reserve(P.image_off + up(tmm::f32tc_grouped_image_bound(prods))));
  if (fresh) TMM_CUDA(ctx, cudaMemset(ctx->batch_f32_scratch.ptr, 0, 256));  // the error word
  *moved = ctx->batch_f32_scratch.ptr != before;
  char* base = (char*)ctx->batch_f32_scratch.ptr;
  for (size_t j = 0; j < prods.size(); ++j) {
    prods[j].a_planes = base + P.a_off[j];
    prods[j].b_planes = base + P.b_off[j];
  }
  std::vector<unsigned char> img;
  cudaError_t e = tmm::f32tc_grouped_image(prods, base + P.arena_off, P.arena_bytes, img, &P.n_items);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched FP32 plan");
  P.n_probs = (int)prods.size();
  if (!img.empty()) TMM_CUDA(ctx, cudaMemcpy(base + P.image_off, img.data(), img.size(), cudaMemcpyHostToDevice));
  TMM_CUDA(ctx, tmm::f32tc_prepare());
  return TMM_SUCCESS;
}

// Lanes: BATCH_LANES streams that fork from stream s (lanes_fork), take work round robin,
// and join back into s (lanes_join).  Small kernels and copies queued on one stream run one
// after another, each after the previous one's launch latency; spread over the lanes their
// latencies overlap (the 512 FP32 splits and 256 copies back of a 512-problem batch: 57.7
// against 58.5 ms per call).
constexpr int BATCH_LANES = 4;

int ensure_batch_lanes(tmm_context* ctx) {
  while (ctx->batch_lanes.size() < (size_t)BATCH_LANES) {
    cudaStream_t ls;
    TMM_CUDA(ctx, cudaStreamCreateWithFlags(&ls, cudaStreamNonBlocking));
    ctx->batch_lanes.push_back(ls);
  }
  while (ctx->batch_lane_events.size() < 1 + (size_t)BATCH_LANES) {
    cudaEvent_t ev;
    TMM_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->batch_lane_events.push_back(ev);
  }
  return TMM_SUCCESS;
}

int lanes_fork(tmm_context* ctx, cudaStream_t s) {
  TMM_CUDA(ctx, cudaEventRecord(ctx->batch_lane_events[0], s));
  for (int q = 0; q < BATCH_LANES; ++q) TMM_CUDA(ctx, cudaStreamWaitEvent(ctx->batch_lanes[(size_t)q], ctx->batch_lane_events[0], 0));
  return TMM_SUCCESS;
}

int lanes_join(tmm_context* ctx, cudaStream_t s) {
  for (int q = 0; q < BATCH_LANES; ++q) {
    TMM_CUDA(ctx, cudaEventRecord(ctx->batch_lane_events[1 + (size_t)q], ctx->batch_lanes[(size_t)q]));
    TMM_CUDA(ctx, cudaStreamWaitEvent(s, ctx->batch_lane_events[1 + (size_t)q], 0));
  }
  return TMM_SUCCESS;
}

// splits (on the lanes) and the grouped launch on stream t (operands already in place)
int enqueue_batch_f32(tmm_context* ctx, const std::vector<tmm::BatchProblem>& dev, const BatchF32Plan& P,
                      cudaStream_t t) {
  if (P.ids.empty()) return TMM_SUCCESS;
  char* base = (char*)ctx->batch_f32_scratch.ptr;
  if (int st = lanes_fork(ctx, t)) return st;
  for (size_t j = 0; j < P.ids.size(); ++j) {
    const tmm::BatchProblem& d = dev[(size_t)P.ids[j]];
    cudaStream_t ls = ctx->batch_lanes[j % BATCH_LANES];
    // lines of op(A): its rows (adjacent when A is not transposed); of op(B): its columns
    cudaError_t e = tmm::f32tc_split_lines((const float*)d.a, d.lda, d.opa == tmm::OP_N, d.m, d.k, base + P.a_off[j], ls);
    if (e == cudaSuccess)
      e = tmm::f32tc_split_lines((const float*)d.b, d.ldb, d.opb != tmm::OP_N, d.n, d.k, base + P.b_off[j], ls);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batched FP32 split");
  }
  if (int st = lanes_join(ctx, t)) return st;
  cudaError_t e = tmm::f32tc_gemm_grouped(base + P.arena_off, P.arena_bytes, base + P.image_off, P.n_probs, P.n_items,
                                          (int*)base, t);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched FP32 launch");
  ctx->stats.kernels += 2 * P.ids.size() + 1;
  return TMM_SUCCESS;
}

// the FP32 problems' work on the batch's second stream, forked from and joined into s
int fork_batch_f32(tmm_context* ctx, const std::vector<tmm::BatchProblem>& dev, const BatchF32Plan& P, cudaStream_t s,
                   bool join) {
  if (P.ids.empty()) return TMM_SUCCESS;
  if (!join) {
    TMM_CUDA(ctx, cudaEventRecord(ctx->batch_f32_fork, s));
    TMM_CUDA(ctx, cudaStreamWaitEvent(ctx->batch_f32_stream, ctx->batch_f32_fork, 0));
    return enqueue_batch_f32(ctx, dev, P, ctx->batch_f32_stream);
  }
  TMM_CUDA(ctx, cudaEventRecord(ctx->batch_f32_join, ctx->batch_f32_stream));
  TMM_CUDA(ctx, cudaStreamWaitEvent(s, ctx->batch_f32_join, 0));
  return TMM_SUCCESS;
}

// copies in, the persistent launch, copies out (host operands)
int enqueue_batch(tmm_context* ctx, const std::vector<tmm::BatchProblem>& dev, const tmm_batch_problem* host,
                  int count, int n_work, int n_f64, int any_k0, const BatchOzPlan& oz, const BatchF32Plan& f32,
                  cudaStream_t s) {
  const size_t rec = tmm::batch_problem_record_bytes();
  const void* dprobs = ctx->batch_meta.ptr;
  const void* dwork = (const char*)ctx->batch_meta.ptr + (rec * (size_t)count + 255) / 256 * 256;
  std::vector<char> on_branch((size_t)count, 0);
  for (int id : oz.ids) on_branch[(size_t)id] = 1;
  // the Ozaki pipeline first: it moves its own operands; the other problems' operands follow
  // its chunks on the same copy stream, so that the engine's chunks are not kept waiting
  int st = enqueue_batch_ozaki(ctx, dev, oz, s, host);
  if (st) return st;
  const bool after_oz = !oz.ids.empty();
  cudaStream_t cs = after_oz ? ctx->oz_branches[1] : s;
  for (int i = 0; i < count; ++i)
    if (!on_branch[(size_t)i] && (st = copy_problem_in(ctx, host[i], dev[i], cs))) return st;
  if (after_oz) {
    cudaEvent_t ev = ctx->oz_branch_done[2 * (size_t)BATCH_OZ_CHUNKS + 3 + (size_t)BATCH_OZ_SPLIT_STREAMS];
    TMM_CUDA(ctx, cudaEventRecord(ev, cs));
    TMM_CUDA(ctx, cudaStreamWaitEvent(s, ev, 0));
  }
  if ((st = fork_batch_f32(ctx, dev, f32, s, false))) return st;
  cudaError_t e = tmm::batch_launch(dprobs, count, dwork, n_f64, n_work - n_f64, any_k0, s, ctx->batch_aux,
                                    ctx->batch_fork, ctx->batch_join);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched kernel launch");
  ctx->stats.kernels += (n_f64 > 0) + (n_work - n_f64 > 0) + (any_k0 ? 1 : 0);
  if ((st = fork_batch_f32(ctx, dev, f32, s, true))) return st;
  if ((st = lanes_fork(ctx, s))) return st;
  for (int i = 0, q = 0; i < count; ++i)
    if (!on_branch[(size_t)i] && (st = copy_problem_out(ctx, host[i], dev[i], ctx->batch_lanes[(size_t)(q++ % BATCH_LANES)])))
      return st;
  if ((st = lanes_join(ctx, s))) return st;
  return join_batch_ozaki(ctx, oz, s, true);
}

}  // namespace

extern "C" int tmm_gemm_batched(tmm_context* ctx, int count, const tmm_batch_problem* probs, int device_operands) {
  if (!ctx) return fail(nullptr, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_batched: null context");
  auto t0 = std::chrono::steady_clock::now();
  ctx->stats = tmm_stats{};
  ctx->stats.direct_host = ctx->direct_host ? 1 : 0;
  if (count < 0 || (count > 0 && !probs)) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_batched: bad count");
  if (count == 0) return TMM_SUCCESS;
  DeviceGuard dg(ctx->device);
  std::vector<tmm::BatchProblem> dev((size_t)count);
  size_t arena = 0;
  int any_k0 = 0;
  for (int i = 0; i < count; ++i) {
    const tmm_batch_problem& h = probs[i];
    tmm::BatchProblem& d = dev[i];
    if (h.dtype != TMM_FLOAT && h.dtype != TMM_DOUBLE)
      return fail(ctx, TMM_ERROR_NOT_SUPPORTED, "tmm_gemm_batched: problems must be TMM_FLOAT or TMM_DOUBLE");
    if (!parse_op(h.trans_a, h.dtype, &d.opa) || !parse_op(h.trans_b, h.dtype, &d.opb))
      return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_batched: trans must be one of N, T, C");
    if (h.m < 0 || h.n < 0 || h.k < 0) return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_batched: negative size");
    const int64_t ar = d.opa == tmm::OP_N ? h.m : h.k, br = d.opb == tmm::OP_N ? h.k : h.n;
    if (h.ld_a < std::max<int64_t>(1, ar) || h.ld_b < std::max<int64_t>(1, br) || h.ld_c < std::max<int64_t>(1, h.m))
      return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_batched: leading dimension too small");
    if (h.m > 0 && h.n > 0 && (!h.c || (h.k > 0 && (!h.a || !h.b))))
      return fail(ctx, TMM_ERROR_INVALID_ARGUMENT, "tmm_gemm_batched: null matrix pointer");
    d.dtype = h.dtype;
    d.m = h.m;
    d.n = h.n;
    d.k = h.k;
    d.alpha = h.alpha;
    d.beta = h.beta;
    d.variant = (h.m > 0 && h.n > 0 && h.k > 0) ? tmm::autotune_batch_variant(h.dtype, h.m, h.n, h.k) : 0;
    if (h.k == 0 && h.m > 0 && h.n > 0) any_k0 = 1;
    if (device_operands) {
      d.a = h.a;
      d.b = h.b;
      d.c = h.c;
      d.lda = h.ld_a;
      d.ldb = h.ld_b;
      d.ldc = h.ld_c;
    } else {  // packed, compact leading dimensions in the arena (offsets filled below)
      const size_t es = h.dtype == TMM_DOUBLE ? 8 : 4;
      d.lda = std::max<int64_t>(1, ar);
      d.ldb = std::max<int64_t>(1, br);
      d.ldc = std::max<int64_t>(1, h.m);
      arena += ((size_t)(h.m * h.k) * es + 255) / 256 * 256;
      arena += ((size_t)(h.k * h.n) * es + 255) / 256 * 256;
      arena += ((size_t)(h.m * h.n) * es + 255) / 256 * 256;
    }
  }
  cudaStream_t s = ctx->streams[0];
  if (!device_operands) {
    void* before = ctx->batch_arena.ptr;
    TMM_CUDA(ctx, ctx->batch_arena.reserve(arena ? arena : 256));
    if (ctx->batch_arena.ptr != before) drop_batch_graph(ctx);
    char* p = (char*)ctx->batch_arena.ptr;
    for (int i = 0; i < count; ++i) {
      tmm::BatchProblem& d = dev[i];
      const size_t es = d.dtype == TMM_DOUBLE ? 8 : 4;
      d.a = p;
      p += ((size_t)(d.m * d.k) * es + 255) / 256 * 256;
      d.b = p;
      p += ((size_t)(d.k * d.n) * es + 255) / 256 * 256;
      d.c = p;
      p += ((size_t)(d.m * d.n) * es + 255) / 256 * 256;
    }
  }
  // on the Ozaki path FP64 problems with k > 0 leave the grouped kernels' list (their records
  // stay, empty) for the engine's grouped launches
  std::vector<int> oz_ids, f32_ids;
  std::vector<tmm::BatchProblem> grouped = dev;
  if (ctx->path == TMM_PATH_OZAKI)
    for (int i = 0; i < count; ++i)
      if (dev[i].m > 0 && dev[i].n > 0 && dev[i].k > 0 && dev[i].dtype == TMM_DOUBLE) {
        oz_ids.push_back(i);
        grouped[i].m = grouped[i].n = 0;
      }
  // FP32 problems with k > 0 run on the FP32 tensor-core engine in one grouped launch
  // (TMM_F32_KERNEL=simt: the grouped FFMA kernel)
  if (!ctx->f32_simt)
    for (int i = 0; i < count; ++i)
      if (dev[i].m > 0 && dev[i].n > 0 && dev[i].k > 0 && dev[i].dtype == TMM_FLOAT) {
        f32_ids.push_back(i);
        grouped[i].m = grouped[i].n = 0;
      }
  BatchF32Plan f32;
  {
    bool moved = false;
    int st0 = plan_batch_f32(ctx, dev, f32_ids, &f32, &moved);
    if (st0) return st0;
    if (moved) drop_batch_graph(ctx);
  }
  BatchOzPlan oz;
  {
    bool moved = false;
    int st0 = plan_batch_ozaki(ctx, dev, oz_ids, &oz, &moved);
    if (st0) return st0;
    if (moved) drop_batch_graph(ctx);
  }
  std::vector<unsigned char> pb, wb;
  int n_work = 0, n_f64 = 0;
  tmm::batch_plan(grouped, pb, wb, &n_work, &n_f64);
  if (!ctx->batch_aux) {
    TMM_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->batch_aux, cudaStreamNonBlocking));
    TMM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->batch_fork, cudaEventDisableTiming));
    TMM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->batch_join, cudaEventDisableTiming));
  }
  if (!ctx->batch_f32_stream) {
    TMM_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->batch_f32_stream, cudaStreamNonBlocking));
    TMM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->batch_f32_fork, cudaEventDisableTiming));
    TMM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->batch_f32_join, cudaEventDisableTiming));
  }
  if (int st0 = ensure_batch_lanes(ctx)) return st0;
  const int kernels = (n_f64 > 0) + (n_work - n_f64 > 0) + any_k0 + oz.kernels +
                      (f32.ids.empty() ? 0 : 2 * (int)f32.ids.size() + 1);
  const size_t pb_al = (pb.size() + 255) / 256 * 256;
  {
    void* before = ctx->batch_meta.ptr;
    TMM_CUDA(ctx, ctx->batch_meta.reserve(pb_al + wb.size() + 256));
    if (ctx->batch_meta.ptr != before) drop_batch_graph(ctx);
  }
  // the layout key: every field of every problem, plus the chosen variants
  std::vector<unsigned char> key((const unsigned char*)probs, (const unsigned char*)probs + sizeof(tmm_batch_problem) * count);
  for (auto& d : dev) key.push_back((unsigned char)d.variant);
  for (int v : {ctx->path, oz.slices, ctx->oz_engine, ctx->max_tile_k, (int)ctx->f32_simt}) {
    const unsigned char* vb = (const unsigned char*)&v;
    key.insert(key.end(), vb, vb + sizeof(v));
  }
  int st = TMM_SUCCESS;
  if (!device_operands && ctx->batch_exec && key == ctx->batch_key) {
    TMM_CUDA(ctx, cudaGraphLaunch(ctx->batch_exec, s));
    ctx->stats.batch_graph = 2;
    ctx->stats.kernels = kernels;
    for (int i = 0; i < count; ++i) {  // same traffic as the captured copies
      const size_t es = dev[i].dtype == TMM_DOUBLE ? 8 : 4;
      if (dev[i].m == 0 || dev[i].n == 0) continue;
      if (dev[i].k > 0) ctx->stats.h2d_bytes += (uint64_t)(dev[i].m * dev[i].k + dev[i].k * dev[i].n) * es;
      if (probs[i].beta != 0.0) ctx->stats.h2d_bytes += (uint64_t)(dev[i].m * dev[i].n) * es;
      ctx->stats.d2h_bytes += (uint64_t)(dev[i].m * dev[i].n) * es;
    }
  } else {
    TMM_CUDA(ctx, cudaMemcpy(ctx->batch_meta.ptr, pb.data(), pb.size(), cudaMemcpyHostToDevice));
    if (!wb.empty())
      TMM_CUDA(ctx, cudaMemcpy((char*)ctx->batch_meta.ptr + pb_al, wb.data(), wb.size(), cudaMemcpyHostToDevice));
    if (device_operands) {
      st = enqueue_batch_ozaki(ctx, dev, oz, s, nullptr);
      if (st) return st;
      if ((st = fork_batch_f32(ctx, dev, f32, s, false))) return st;
      cudaError_t e = tmm::batch_launch(ctx->batch_meta.ptr, count, (char*)ctx->batch_meta.ptr + pb_al, n_f64,
                                        n_work - n_f64, any_k0, s, ctx->batch_aux, ctx->batch_fork, ctx->batch_join);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "batched kernel launch");
      if ((st = fork_batch_f32(ctx, dev, f32, s, true))) return st;
      st = join_batch_ozaki(ctx, oz, s, false);
      if (st) return st;
      ctx->stats.kernels = kernels;
    } else {
      bool pinned = true;
      for (int i = 0; i < count && pinned; ++i) {
        const tmm_batch_problem& h = probs[i];
        if (h.m == 0 || h.n == 0) continue;
        pinned = page_locked(h.c) && (h.k == 0 || (page_locked(h.a) && page_locked(h.b)));
      }
      if (pinned) {
        drop_batch_graph(ctx);
        TMM_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        st = enqueue_batch(ctx, dev, probs, count, n_work, n_f64, any_k0, oz, f32, s);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (st) {
          if (graph) cudaGraphDestroy(graph);
          return st;
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&ctx->batch_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
          ctx->batch_exec = nullptr;
          return cuda_fail(ctx, e, "cudaGraphInstantiate");
        }
        ctx->batch_key = key;
        TMM_CUDA(ctx, cudaGraphLaunch(ctx->batch_exec, s));
        ctx->stats.batch_graph = 1;
      } else {
        st = enqueue_batch(ctx, dev, probs, count, n_work, n_f64, any_k0, oz, f32, s);
        if (st) return st;
      }
    }
  }
  TMM_CUDA(ctx, cudaStreamSynchronize(s));
  if (!st && !oz_ids.empty()) {
    ctx->stats.path = TMM_PATH_OZAKI;
    ctx->stats.ozaki_slices = oz.slices;
    st = check_oz_error(ctx);
  }
  if (!st && !f32_ids.empty()) st = check_f32_error(ctx);
  ctx->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return st;
}
