/*
 * tmm_c_api.h — C ABI of the GB300 (sm_103a) out-of-core tiled GEMM.
 *
 * This is the drop-in boundary: plain pointers, sizes and status codes, no
 * CUDA or C++ types in the signatures.  The C++ headers under
 * include/Tiled-MM/ (the reference's public API: gpu::make_context,
 * gpu::gemm, mm_handle::get_full_device_buffer_c, ...) are thin inline
 * wrappers over these entry points, and any FFI (ctypes, cgo, JNI) can bind
 * them directly.  Each entry point names the reference interface it replaces
 * (file:line in eth-cscs/Tiled-MM).
 *
 * Semantics kept from the reference:
 *   - C = alpha * op(A) * op(B) + beta * C, column-major, op in {N, T, C}
 *     (lower case accepted: toupper, src/Tiled-MM/tiled_mm.cpp:503-504);
 *   - host pointers; the call is synchronous (returns when C is final);
 *   - beta == 0 never reads C (src/Tiled-MM/tiled_mm.cpp:325, 425);
 *   - pin_host_buffers registers A, B (and C when copy_c_back || beta != 0)
 *     for the call's duration (src/Tiled-MM/tiled_mm.cpp:529-554, 606-623);
 *   - copy_c_back == 0 leaves the result on the device in a compact m x n
 *     column-major buffer (ld = m) returned by tmm_get_full_c
 *     (src/Tiled-MM/mm_handle.cpp:162-165, tests/test-multiply.cpp:339);
 *   - device buffers grow and are never shrunk by a call
 *     (src/Tiled-MM/device_vector.hpp:93-107);
 *   - the tile-size policy of src/Tiled-MM/mm_handle.cpp:89-133 is the
 *     default (TMM_TILE_POLICY_REFERENCE).
 * Deliberate deviations from the reference:
 *   - 64-bit sizes, leading dimensions and offsets (the reference's int
 *     offsets overflow past 2^31 elements);
 *   - invalid arguments are reported (the reference constructs but never
 *     throws them, src/Tiled-MM/tiled_mm.cpp:516-527);
 *   - stream synchronisation of this context's streams instead of a
 *     device-wide cudaDeviceSynchronize (src/Tiled-MM/tiled_mm.cpp:602-604);
 *   - an already-registered host buffer is used as is (and left registered).
 */
#ifndef TMM_C_API_H
#define TMM_C_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tmm_context tmm_context;

/* Scalar types of the reference's explicit instantiations
 * (src/Tiled-MM/tiled_mm.cpp:626-668, src/Tiled-MM/mm_handle.cpp:167-170). */
enum tmm_dtype {
  TMM_FLOAT = 0,
  TMM_DOUBLE = 1,
  TMM_COMPLEX_FLOAT = 2, /* std::complex<float>: {re, im} pairs */
  TMM_COMPLEX_DOUBLE = 3 /* std::complex<double> */
};

enum tmm_status {
  TMM_SUCCESS = 0,
  TMM_ERROR_INVALID_ARGUMENT = 1,
  TMM_ERROR_CUDA = 2,
  TMM_ERROR_OUT_OF_MEMORY = 3,
  TMM_ERROR_NOT_SUPPORTED = 4,
  TMM_ERROR_INTERNAL = 5,
  TMM_ERROR_TIMEOUT = 6
};

/* Multiplication paths for TMM_DOUBLE. */
enum tmm_path {
  TMM_PATH_NATIVE = 0, /* FP64 tensor-core (DMMA) tile kernel */
  TMM_PATH_OZAKI = 1   /* split-precision emulation on tcgen05 low-precision tensor cores */
};

/* Tile-size policies. */
enum tmm_tile_policy {
  TMM_TILE_POLICY_REFERENCE = 0, /* src/Tiled-MM/mm_handle.cpp:89-133 (divisor policy) */
  TMM_TILE_POLICY_FIXED = 1,     /* use the context's max tile sizes, clipped to the matrix */
  TMM_TILE_POLICY_AUTOTUNE = 2   /* the autotuner's choice per (dtype, path, size class) */
};

/* ------------------------------------------------------------------ context */

/* Replaces gpu::make_context<Scalar>(streams, max_tile_m, max_tile_n, max_tile_k)
 * (src/Tiled-MM/mm_handle.hpp:60-69) and mm_handle::mm_handle
 * (src/Tiled-MM/mm_handle.cpp:11-29).  Creates the streams on the caller's
 * current device; allocates no device memory (buffers are sized lazily by the
 * first gemm, as in the reference). */
int tmm_create(int dtype, int n_streams, int max_tile_m, int max_tile_n, int max_tile_k,
               tmm_context** ctx);

/* Replaces mm_handle::~mm_handle / gpu_context::~gpu_context
 * (src/Tiled-MM/mm_handle.cpp:32-34, src/Tiled-MM/gpu_context.cpp:59-63). */
int tmm_destroy(tmm_context* ctx);

/* ------------------------------------------------------------------ GEMM */

/* Replaces gpu::gemm<Scalar>(mm_handle&, trans_a, trans_b, m, n, k, alpha, a,
 * ld_a, b, ld_b, beta, c, ld_c, pin_host_buffers, copy_c_back)
 * (src/Tiled-MM/tiled_mm.hpp:69-79, src/Tiled-MM/tiled_mm.cpp:492-624).
 * alpha and beta point to one scalar of the context's dtype. */
int tmm_gemm(tmm_context* ctx, char trans_a, char trans_b, int64_t m, int64_t n, int64_t k,
             const void* alpha, const void* a, int64_t ld_a, const void* b, int64_t ld_b,
             const void* beta, void* c, int64_t ld_c, int pin_host_buffers, int copy_c_back);

/* Same product on operands already in device memory (no host copies), on the
 * given CUDA stream (a cudaStream_t; NULL is the legacy default stream).
 * Returns after the work is enqueued; the caller synchronises the stream.
 * No reference counterpart: it is the device-pointer entry of the tile
 * kernel that src/Tiled-MM/tiled_mm.cpp:200-217 reaches through cuBLAS. */
int tmm_gemm_device(tmm_context* ctx, char trans_a, char trans_b, int64_t m, int64_t n, int64_t k,
                    const void* alpha, const void* a_dev, int64_t ld_a, const void* b_dev, int64_t ld_b,
                    const void* beta, void* c_dev, int64_t ld_c, void* stream);

/* No counterpart in the reference (its calls are synchronous and report every failure).
 * Device-side status of the asynchronous work this context has enqueued through
 * tmm_gemm_device: waits for `stream` (a cudaStream_t; NULL: legacy default stream), then
 * returns TMM_ERROR_TIMEOUT if a tensor-core kernel of this context gave up a pipeline wait
 * (after about a second; its C is then incomplete) since the last check, TMM_SUCCESS
 * otherwise, and clears what it read.  The synchronous calls check this themselves. */
int tmm_device_status(tmm_context* ctx, void* stream);

/* No counterpart in the reference.  The Ozaki (emulated FP64) product on
 * device operands for callers that cannot allocate device memory while they
 * run -- a framework whose caching allocator already owns the GPU, or a
 * latency-critical caller that cannot take cudaFree's device-wide sync.  It
 * calls no cudaMalloc/cudaFree: its scratch is one fixed 96 MiB array of
 * device memory inside the library, held by every GPU that loads the library
 * until exit.  Up to slices * (round256(m) + round256(n)) * k_tile bytes of
 * digits per k step fit (k_tile = 0 picks the largest that fits, a multiple of
 * 128); larger requests fail with TMM_ERROR_INVALID_ARGUMENT and a message in
 * tmm_last_error(NULL).  All calls share the array: calls that overlap on the
 * GPU race.  The first call on a device looks up the array's device address;
 * make it before any stream capture.  Enqueues on `stream` (NULL: legacy
 * default stream) and returns; results equal tmm_gemm_device's with the
 * tcgen05 engine, the same slice count and max_tile_k = k_tile (k_tile is an
 * upper bound: a k_tile beyond k means one k step).  A tensor-core wait that
 * gives up on the GPU (after about a second; C is then incomplete) is
 * reported by tmm_ozaki_noalloc_status, not by this call. */
int tmm_ozaki_gemm_device_noalloc(char trans_a, char trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                                  const double* a_dev, int64_t ld_a, const double* b_dev, int64_t ld_b,
                                  double beta, double* c_dev, int64_t ld_c, int slices, int64_t k_tile,
                                  void* stream);

/* No counterpart in the reference.  Device-side status of the allocation-free
 * entry above: waits for `stream` (a cudaStream_t; NULL: legacy default
 * stream), then returns TMM_ERROR_TIMEOUT if a call on the current device gave
 * up waiting inside the tensor-core pipeline since the last status check, and
 * TMM_SUCCESS otherwise; clears the word it read.  Allocates nothing. */
int tmm_ozaki_noalloc_status(void* stream);

/* One problem of a batch (tmm_gemm_batched). */
typedef struct tmm_batch_problem {
  int dtype;             /* TMM_FLOAT or TMM_DOUBLE */
  char trans_a, trans_b; /* 'N', 'T' or 'C' */
  int64_t m, n, k;
  double alpha, beta;    /* rounded to float for TMM_FLOAT problems */
  const void* a;
  int64_t ld_a;
  const void* b;
  int64_t ld_b;
  void* c;
  int64_t ld_c;
} tmm_batch_problem;

/* New, no reference counterpart (its users call gpu::gemm once per problem,
 * src/Tiled-MM/tiled_mm.cpp:492-624): `count` GEMMs of any shapes, FP64 and
 * FP32 mixed, in one persistent kernel launch over a work list of (problem,
 * C tile) items, tile shapes per size class from the autotuner.  Operands are
 * host pointers (device_operands == 0: copied in, results copied back; when
 * every host buffer is page-locked the copies and the launch are captured
 * once into a CUDA graph keyed by the batch layout and replayed by later calls
 * with the same layout) or device pointers (device_operands != 0).
 * Synchronous; semantics per problem as tmm_gemm with copy_c_back. */
int tmm_gemm_batched(tmm_context* ctx, int count, const tmm_batch_problem* problems, int device_operands);

/* Replaces mm_handle::get_full_device_buffer_c() (src/Tiled-MM/mm_handle.cpp:162-165)
 * and its device_vector::data()/size()/capacity() (src/Tiled-MM/device_vector.hpp:67-80):
 * the device pointer of the compact (ld = m) result left by copy_c_back == 0. */
int tmm_get_full_c(tmm_context* ctx, void** device_ptr, size_t* size_elems, size_t* capacity_elems);

/* ------------------------------------------------------------------ streams, events, device buffers */

/* gpu_context::get_stream(stream_id) (src/Tiled-MM/gpu_context.cpp:27-32): the context's
 * compute stream stream_id (a cudaStream_t), 0 <= stream_id < the stream count; out of range
 * gives TMM_ERROR_INVALID_ARGUMENT. */
int tmm_get_stream(tmm_context* ctx, int stream_id, void** stream);
/* gpu_context::get_result_stream() (src/Tiled-MM/gpu_context.cpp:55-57): the stream results
 * return to the host on. */
int tmm_get_result_stream(tmm_context* ctx, void** stream);
/* device_buffer::data() / stream_buffer(stream_id) of the handle's A, B or C buffer
 * (src/Tiled-MM/device_buffer.hpp:19-21, 49-63): which is 'a', 'b' or 'c'; stream_id -1 gives
 * the buffer's base.  C: the first result-tile slot of compute stream stream_id.  A and B: this
 * library caches device tiles instead of keeping one slot per stream, so the pointer is that of
 * cache slot stream_id.  NULL until the first gemm has sized the buffers. */
int tmm_get_device_buffer(tmm_context* ctx, char which, int stream_id, void** ptr);

/* device_stream / device_event (src/Tiled-MM/device_stream.hpp:8-75,
 * src/Tiled-MM/device_event.hpp:9-80) over the current device: a non-blocking stream, an event
 * (timing enabled, so that time_since works), recording, host and stream waits, elapsed seconds. */
int tmm_stream_create(void** stream);
int tmm_stream_destroy(void* stream);
int tmm_event_create(void** event);
int tmm_event_destroy(void* event);
int tmm_event_record(void* event, void* stream);
int tmm_event_synchronize(void* event);
int tmm_event_elapsed(void* start, void* end, double* seconds);
int tmm_stream_wait_event(void* stream, void* event);

/* ------------------------------------------------------------------ handle settings */

/* mm_handle::set_num_streams / get_num_streams (src/Tiled-MM/mm_handle.cpp:37-50). */
int tmm_set_num_streams(tmm_context* ctx, int n_streams);
int tmm_get_num_streams(tmm_context* ctx, int* n_streams);

/* mm_handle::set_tile_sizes (src/Tiled-MM/mm_handle.cpp:58-71): records the
 * current tile sizes (and grows the tile buffers on next use). */
int tmm_set_tile_sizes(tmm_context* ctx, int tile_m, int tile_n, int tile_k);
/* device_buffer::get_tile_sizes of the C and A buffers (src/Tiled-MM/device_buffer.hpp:181-184):
 * the tile sizes used by the last call (tile_m, tile_n from C; tile_k from A). */
int tmm_get_tile_sizes(tmm_context* ctx, int* tile_m, int* tile_n, int* tile_k);

/* mm_handle::set_full_sizes (src/Tiled-MM/mm_handle.cpp:74-80): grow the full-C buffer to m*n. */
int tmm_set_full_sizes(tmm_context* ctx, int64_t m, int64_t n, int64_t k);

/* mm_handle::optimal_tile_sizes (src/Tiled-MM/mm_handle.cpp:117-133). */
int tmm_optimal_tile_sizes(tmm_context* ctx, int64_t m, int64_t n, int64_t k, int* tile_m, int* tile_n,
                           int* tile_k);

/* mm_handle::get_max_tile_sizes (src/Tiled-MM/mm_handle.cpp:112-115). */
int tmm_get_max_tile_sizes(tmm_context* ctx, int* tile_m, int* tile_n, int* tile_k);

/* mm_handle::set_streams_and_tiles (src/Tiled-MM/mm_handle.cpp:135-145). */
int tmm_set_streams_and_tiles(tmm_context* ctx, int n_streams, int tile_m, int tile_n, int tile_k);

/* New: multiplication path and the Ozaki slice count (slices <= 0 selects the default:
 * 13 for double and complex double, 6 for float and complex float).  On TMM_PATH_OZAKI,
 * double contexts split their cached tiles; float, complex float and complex double
 * contexts cache raw tiles and multiply each tile's real FP64 embedding (complex:
 * [[Re A, -Im A], [Im A, Re A]] x [Re B; Im B]) on the same engine, alpha and beta applied
 * in double and the result rounded once to the context's type. */
int tmm_set_path(tmm_context* ctx, int path, int ozaki_slices);
int tmm_get_path(tmm_context* ctx, int* path, int* ozaki_slices);

/* New: the engine behind TMM_PATH_OZAKI (TMM_OZAKI_IMMA: mma.sync int8 -> int32;
 * TMM_OZAKI_TCGEN05: tcgen05.mma kind::f8f6f4 e4m3 -> FP32 in tensor memory, the
 * default of new contexts; the environment variable TMM_OZAKI_ENGINE=imma|tcgen05
 * overrides it), its k-block (elements) and the k-blocks accumulated exactly between
 * two FP64 recombination steps. */
enum tmm_ozaki_engine { TMM_OZAKI_IMMA = 0, TMM_OZAKI_TCGEN05 = 1 };
int tmm_set_ozaki_engine(tmm_context* ctx, int engine);
int tmm_get_ozaki_engine(tmm_context* ctx, int* engine, int* k_block, int64_t* pass_blocks);

/* New: tile policy (enum tmm_tile_policy).  TMM_TILE_POLICY_AUTOTUNE times a few candidate
 * tile sets (sizes that fit the device memory, k tiles halved and quartered, m and n tiles
 * halved) per size class -- dtype, path, engine, slices, log2 of m, n and k, trans, pinning,
 * copy-back -- over the first calls of the class (each call computes the whole product with
 * one candidate), then uses the fastest; TMM_AUTOTUNE_CACHE names a file that keeps the
 * choices across processes.  It replaces the reference's divisor rule
 * (src/Tiled-MM/mm_handle.cpp:89-133), which stays the default policy. */
int tmm_set_tile_policy(tmm_context* ctx, int policy);
/* New: the autotuner's measurements for the size class of this context's last autotuned call
 * (candidates, their FP64-equivalent TFLOP/s, the chosen one), as text into text[capacity]. */
int tmm_get_autotune_report(tmm_context* ctx, char* text, size_t capacity);

/* New: cap on the device memory the context may hold (0 = no cap beyond what
 * is free on the device).  Smaller caps force out-of-core tiling. */
int tmm_set_memory_limit(tmm_context* ctx, size_t bytes);

/* ------------------------------------------------------------------ diagnostics */

typedef struct tmm_stats {
  uint64_t h2d_bytes;     /* host -> device bytes of the last call */
  uint64_t d2h_bytes;     /* device -> host bytes of the last call */
  uint64_t kernels;       /* kernel launches of the last call */
  uint64_t tiles_loaded;  /* A/B tiles copied to the device */
  uint64_t tiles_reused;  /* A/B tile uses served from device-resident tiles */
  int tile_m, tile_n, tile_k, n_streams;
  int path, ozaki_slices;
  double seconds;         /* host wall time of the last call */
  int batch_graph;        /* last tmm_gemm_batched: 0 no graph, 1 captured, 2 replayed */
  int direct_host;        /* TMM_DIRECT_HOST=1 and the GPU reads and writes pageable host memory through
                             the host page tables: unregistered host tiles are copied by kernel */
  uint64_t direct_bytes;  /* bytes of the last call copied by kernel between unregistered host memory and
                             the device (the rest of h2d_bytes / d2h_bytes went through the copy engines) */
  int autotune_state;     /* TMM_TILE_POLICY_AUTOTUNE: 1 the call ran an untimed candidate of its size class,
                             2 the fastest measured candidate, 3 a choice read from TMM_AUTOTUNE_CACHE;
                             0 another policy */
} tmm_stats;

int tmm_get_stats(tmm_context* ctx, tmm_stats* stats);

/* Timing of the engine kernels (the tile GEMM of the native path, the slice-product
 * kernel of the Ozaki path), for profiling; no counterpart in the reference.  While on,
 * every engine launch is bracketed by two CUDA events recorded on its stream.
 * tmm_set_kernel_timing clears the totals; tmm_get_kernel_time waits for the recorded
 * launches and returns the summed device time (seconds) and the number of launches. */
int tmm_set_kernel_timing(tmm_context* ctx, int on);
int tmm_get_kernel_time(tmm_context* ctx, double* seconds, uint64_t* launches);
/* The same launches as device busy time: the length of the union of their [start, end]
 * intervals (launches on several streams that overlap count once) and the span from the
 * first start to the last end, in seconds, since timing was switched on. */
int tmm_get_kernel_busy_time(tmm_context* ctx, double* busy_seconds, double* span_seconds);

/* Message of the last failure of this context (ctx == NULL: of the calling
 * thread's last context-free call).  Never NULL. */
const char* tmm_last_error(tmm_context* ctx);
const char* tmm_status_string(int status);

/* ------------------------------------------------------------------ utilities */

/* gpu::malloc_pinned (src/Tiled-MM/util.hpp:64-72): page-locked host memory. */
int tmm_malloc_pinned(size_t bytes, void** ptr);
int tmm_free_pinned(void* ptr);
/* gpu::copy_to_device / copy_to_host (src/Tiled-MM/util.hpp:79-88). */
int tmm_copy_to_device(const void* host, void* device, size_t bytes);
int tmm_copy_to_host(const void* device, void* host, size_t bytes);
/* gpu::copy_to_device_async / copy_to_host_async (src/Tiled-MM/util.hpp:90-118): direction
 * inferred from the pointers (unified addressing); stream is a cudaStream_t or NULL. */
int tmm_memcpy_async(void* dst, const void* src, size_t bytes, void* stream);
/* gpu::malloc_device (src/Tiled-MM/util.hpp:56-62) and its release. */
int tmm_malloc_device(size_t bytes, void** ptr);
int tmm_free_device(void* ptr);

/* Seeded synthetic matrices (kind: see tiled-mm_gb300/csrc/tmm_datagen.h).
 * The host and device generators give identical values element by element. */
int tmm_fill_host_f64(double* x, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                      uint64_t seed, uint64_t id, int n_threads);
int tmm_fill_device_f64(double* x, int64_t rows, int64_t cols, int64_t ld, int kind, double param,
                        uint64_t seed, uint64_t id, void* stream);

/* Componentwise error metric of a computed FP64 GEMM on sampled entries:
 * max |C(i,j) - C*(i,j)| / (k * 2^-53 * (|alpha| |op(A)||op(B)| + |beta| |C0|)(i,j)),
 * with C* evaluated in twice-working precision (compensated dot product).
 * c0 is the input C (may be NULL when beta == 0), c the result. */
int tmm_error_metric_f64(char trans_a, char trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                         const double* a, int64_t ld_a, const double* b, int64_t ld_b, double beta,
                         const double* c0, int64_t ld_c0, const double* c, int64_t ld_c, int64_t n_samples,
                         uint64_t seed, int n_threads, double* metric);

/* ------------------------------------------------------------------ cublasXt-style entry
 * The call shape of the reference's comparison program against cublasXt
 * (examples/cublasXt-multiply.cpp:153-167: cublasXtCreate, cublasXtDeviceSelect,
 * cublasXtSetBlockDim, cublasXt?gemm on host pointers), on the tiled path of this library:
 * one block dimension for all three tile sizes (default 4096), trans arguments as
 * cublasOperation_t values (0 = N, 1 = T, 2 = C), host or device pointers, page-locking
 * for the call and C copied back, synchronous.  The current device is used.
 * tmm_xt_set_path selects the path of all four calls (slices <= 0: each type's default). */
typedef struct tmm_xt tmm_xt;
int tmm_xt_create(tmm_xt** handle);
int tmm_xt_destroy(tmm_xt* handle);
int tmm_xt_set_block_dim(tmm_xt* handle, int block_dim);
int tmm_xt_get_block_dim(tmm_xt* handle, int* block_dim);
int tmm_xt_set_path(tmm_xt* handle, int path, int ozaki_slices);
const char* tmm_xt_last_error(tmm_xt* handle);
int tmm_xt_sgemm(tmm_xt* handle, int transa, int transb, int64_t m, int64_t n, int64_t k, const float* alpha,
                 const float* a, int64_t ld_a, const float* b, int64_t ld_b, const float* beta, float* c,
                 int64_t ld_c);
int tmm_xt_dgemm(tmm_xt* handle, int transa, int transb, int64_t m, int64_t n, int64_t k, const double* alpha,
                 const double* a, int64_t ld_a, const double* b, int64_t ld_b, const double* beta, double* c,
                 int64_t ld_c);
/* complex float / complex double: interleaved (re, im) pairs, as std::complex */
int tmm_xt_cgemm(tmm_xt* handle, int transa, int transb, int64_t m, int64_t n, int64_t k, const void* alpha,
                 const void* a, int64_t ld_a, const void* b, int64_t ld_b, const void* beta, void* c, int64_t ld_c);
int tmm_xt_zgemm(tmm_xt* handle, int transa, int transb, int64_t m, int64_t n, int64_t k, const void* alpha,
                 const void* a, int64_t ld_a, const void* b, int64_t ld_b, const void* beta, void* c, int64_t ld_c);

#ifdef __cplusplus
}
#endif

#endif /* TMM_C_API_H */
