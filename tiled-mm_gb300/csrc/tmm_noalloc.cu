// Allocation-free variant of the Ozaki (emulated FP64) GEMM on device operands.
//
// Who needs it: callers that must not call cudaMalloc/cudaFree while they run
// -- for example a framework whose caching allocator already owns the GPU's
// memory (a fresh cudaMalloc would fail or fragment it), or a latency-critical
// caller that cannot accept the device-wide synchronisation cudaFree implies.
// The regular entry points grow their scratch buffers on demand; this one never
// allocates: its scratch (digit planes, the tensor-core engine's FP64
// accumulators and its error word) is one fixed array in device memory,
// declared below, that every GPU which loads this library holds until the
// process exits.
//
// Limits: the array is TMM_NOALLOC_SCRATCH_BYTES (96 MiB + 256 bytes): 40 MiB of
// FP64 accumulators (one 128 x 256 slot per SM, up to 160 SMs) and 56 MiB of
// digit planes, enough for slices * (round256(m) + round256(n)) * k_tile bytes
// of one k step, k_tile a multiple of 128.  Requests that do not fit (or
// slices outside 1..20, or a device with more than 160 SMs) are rejected with
// TMM_ERROR_INVALID_ARGUMENT and a message from tmm_last_error(NULL).
//
// Sharing: every call on every stream of a device uses the same array and the
// array keeps the last call's contents, so calls that overlap on the GPU race
// and corrupt each other; serialise them (one stream, or events).
//
// Errors found on the GPU: the call returns once its work is enqueued, so a
// tensor-core wait that gives up (after about a second; C is then incomplete)
// can only be reported later.  It sets an error word in the array that stays
// set until tmm_ozaki_noalloc_status reads it: that call waits for the given
// stream, returns TMM_ERROR_TIMEOUT if any call on this device since the last
// status check gave up (TMM_SUCCESS otherwise) and clears the word.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current (in host code the
// array's name is only a host-side stand-in, never a device address).  Make
// that first call before any stream capture begins.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/tmm_c_api.h"
#include "tmm_ozaki.h"

namespace {

constexpr size_t NOALLOC_ERR_BYTES = 256;
constexpr size_t NOALLOC_MAX_SMS = 160;
constexpr size_t NOALLOC_WORK_BYTES = NOALLOC_MAX_SMS * 128 * 256 * sizeof(double);  // 40 MiB
constexpr size_t NOALLOC_DIGIT_BYTES = (size_t)56 << 20;                            // 56 MiB
constexpr size_t TMM_NOALLOC_SCRATCH_BYTES = NOALLOC_ERR_BYTES + NOALLOC_WORK_BYTES + NOALLOC_DIGIT_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[TMM_NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void* g_scratch_ptr[MAX_DEVICES] = {nullptr};

int reject(int status, const std::string& msg) {
  tmm::set_last_error_message(msg.c_str());  // read back with tmm_last_error(NULL)
  return status;
}

// The array's device address on the current device (looked up once per device, with
// that device current: in host code the array's name is a host-side stand-in).
int scratch_base(const char* who, unsigned char** base) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
    return reject(TMM_ERROR_CUDA, std::string(who) + ": no current CUDA device");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return reject(TMM_ERROR_CUDA, std::string(who) + ": cudaGetSymbolAddress: " + cudaGetErrorString(e));
    }
    g_scratch_ptr[dev] = p;
  }
  *base = (unsigned char*)g_scratch_ptr[dev];
  return TMM_SUCCESS;
}

}  // namespace

extern "C" int tmm_ozaki_gemm_device_noalloc(char trans_a, char trans_b, int64_t m, int64_t n, int64_t k,
                                             double alpha, const double* a, int64_t ld_a, const double* b,
                                             int64_t ld_b, double beta, double* c, int64_t ld_c, int slices,
                                             int64_t k_tile, void* stream) {
  using namespace tmm;
  auto op_of = [](char t, Op* o) {
    switch (t) {
      case 'N': case 'n': *o = OP_N; return true;
      case 'T': case 't': case 'C': case 'c': *o = OP_T; return true;
      default: return false;
    }
  };
  Op opa, opb;
  if (!op_of(trans_a, &opa) || !op_of(trans_b, &opb))
    return reject(TMM_ERROR_INVALID_ARGUMENT, "tmm_ozaki_gemm_device_noalloc: trans must be one of N, T, C");
  if (m < 0 || n < 0 || k < 0 || slices < 1 || slices > OZ_MAX_SLICES || k_tile < 0)
    return reject(TMM_ERROR_INVALID_ARGUMENT, "tmm_ozaki_gemm_device_noalloc: bad size, slice count or k_tile");
  const int64_t a_rows = opa == OP_N ? m : k, b_rows = opb == OP_N ? k : n;
  if (ld_a < (a_rows > 1 ? a_rows : 1) || ld_b < (b_rows > 1 ? b_rows : 1) || ld_c < (m > 1 ? m : 1))
    return reject(TMM_ERROR_INVALID_ARGUMENT, "tmm_ozaki_gemm_device_noalloc: leading dimension too small");
  if (m == 0 || n == 0) return TMM_SUCCESS;
  if (!c || (k > 0 && (!a || !b)))
    return reject(TMM_ERROR_INVALID_ARGUMENT, "tmm_ozaki_gemm_device_noalloc: null matrix pointer");

  // ---- fit the request into the fixed digit region (m and n are bounded first, so that
  // the byte counts below cannot overflow: one 128-wide k step of one slice of m + n lines
  // must fit)
  if (m > (int64_t)(NOALLOC_DIGIT_BYTES / OZ_K_ALIGN) || n > (int64_t)(NOALLOC_DIGIT_BYTES / OZ_K_ALIGN)) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "tmm_ozaki_gemm_device_noalloc: m=%lld, n=%lld: one 128-wide k step needs more digit bytes than the "
             "fixed %zu-byte scratch holds",
             (long long)m, (long long)n, NOALLOC_DIGIT_BYTES);
    return reject(TMM_ERROR_INVALID_ARGUMENT, buf);
  }
  const int64_t rows_total = oz_round_up(m, OZ_ROW_ALIGN) + oz_round_up(n, OZ_ROW_ALIGN);
  const int64_t per_k = (int64_t)slices * rows_total;  // digit bytes per k element
  const int64_t exp_bytes = 2 * 256 + rows_total * (int64_t)sizeof(int32_t) + 2048;  // exponents + alignment
  const int64_t k_room = ((int64_t)NOALLOC_DIGIT_BYTES - exp_bytes) / per_k / OZ_K_ALIGN * OZ_K_ALIGN;
  if (k_room < OZ_K_ALIGN) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "tmm_ozaki_gemm_device_noalloc: m=%lld, n=%lld with %d slices need %lld bytes of digits per 128 k, "
             "more than the fixed %zu-byte scratch holds",
             (long long)m, (long long)n, slices, (long long)(per_k * OZ_K_ALIGN + exp_bytes), NOALLOC_DIGIT_BYTES);
    return reject(TMM_ERROR_INVALID_ARGUMENT, buf);
  }
  // k_tile is an upper bound, as max_tile_k is for the regular entry: a k_tile beyond k is k
  int64_t kt = k_tile > 0 ? (k_tile < k ? k_tile : k) : (k < k_room ? k : k_room);
  if (kt <= 0) kt = 1;
  if (oz_round_up(kt, OZ_K_ALIGN) > k_room) {
    char buf[256];
    snprintf(buf, sizeof buf, "tmm_ozaki_gemm_device_noalloc: k_tile=%lld exceeds the %lld that the fixed scratch "
                              "holds for m=%lld, n=%lld, %d slices",
             (long long)kt, (long long)k_room, (long long)m, (long long)n, slices);
    return reject(TMM_ERROR_INVALID_ARGUMENT, buf);
  }

  // ---- once per device: the array's device address
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
    return reject(TMM_ERROR_CUDA, "tmm_ozaki_gemm_device_noalloc: no current CUDA device");
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0 ||
      (size_t)sms > NOALLOC_MAX_SMS || ozaki_tc_workspace_bytes() > NOALLOC_WORK_BYTES)
    return reject(TMM_ERROR_NOT_SUPPORTED, "tmm_ozaki_gemm_device_noalloc: device has more SMs than the fixed "
                                           "accumulator slots cover");
  unsigned char* base = nullptr;
  if (int st = scratch_base("tmm_ozaki_gemm_device_noalloc", &base)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // the error word stays set until tmm_ozaki_noalloc_status reads and clears it
  int* err = (int*)base;
  double* work = (double*)(base + NOALLOC_ERR_BYTES);
  unsigned char* digits = base + NOALLOC_ERR_BYTES + NOALLOC_WORK_BYTES;

  if (k == 0) {
    // C = beta * C with the product empty: one pass of the split-product path is not needed
    e = launch_scale_f64(m, n, beta, c, ld_c, s);
    return e == cudaSuccess ? TMM_SUCCESS : reject(TMM_ERROR_CUDA, "tmm_ozaki_gemm_device_noalloc: launch failed");
  }
  const size_t sa = ozaki_split_bytes(m, kt, slices);
  const size_t sa_al = (sa + 255) / 256 * 256;
  for (int64_t k0 = 0, t = 0; k0 < k; k0 += kt, ++t) {
    const int64_t kk = (k - k0) < kt ? (k - k0) : kt;
    OzakiSplit va = ozaki_split_view(digits, m, kk, slices, OZ_ENGINE_TCGEN05);
    OzakiSplit vb = ozaki_split_view(digits + sa_al, n, kk, slices, OZ_ENGINE_TCGEN05);
    const double* ab = opa == OP_N ? a + k0 * ld_a : a + k0;
    const double* bb = opb == OP_N ? b + k0 : b + k0 * ld_b;
    e = ozaki_split(ab, ld_a, opa == OP_N ? OP_N : OP_T, m, kk, va, s);
    if (e == cudaSuccess) e = ozaki_split(bb, ld_b, opb == OP_N ? OP_T : OP_N, n, kk, vb, s);
    if (e == cudaSuccess) e = ozaki_gemm_tc(va, vb, m, n, alpha, beta, t == 0, c, ld_c, work, err, s);
    if (e != cudaSuccess)
      return reject(TMM_ERROR_CUDA, std::string("tmm_ozaki_gemm_device_noalloc: launch failed: ") + cudaGetErrorString(e));
  }
  return TMM_SUCCESS;
}

extern "C" int tmm_ozaki_noalloc_status(void* stream) {
  unsigned char* base = nullptr;
  if (int st = scratch_base("tmm_ozaki_noalloc_status", &base)) return st;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  int word = 0;
  // a plain copy of 4 bytes into this stack variable and a 4-byte clear: nothing is allocated
  if (e == cudaSuccess) e = cudaMemcpy(&word, base, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && word) e = cudaMemset(base, 0, sizeof(int));
  if (e != cudaSuccess)
    return reject(TMM_ERROR_CUDA, std::string("tmm_ozaki_noalloc_status: ") + cudaGetErrorString(e));
  if (word)
    return reject(TMM_ERROR_TIMEOUT, "tmm_ozaki_noalloc_status: a tensor-core pipeline wait gave up in an earlier "
                                     "call on this device; its C is incomplete");
  return TMM_SUCCESS;
}
