// Internal interface of the Ozaki split-precision FP64 engine (not part of the C ABI).
//
// A double tile op(X) (lines x kk along k) is split into s digit planes of
// small integers |d| <= 16 stored one byte per digit, K-major, plus one
// power-of-two exponent per line (digit layouts: see OzakiSplit); the product
// of two split tiles is a sum of exact integer tile GEMMs on the tensor cores,
// recombined in FP64 with the alpha/beta epilogue fused.  tmm_ozaki.cu holds
// the algorithm and its published sources.
#pragma once
#include <cuda_runtime.h>

#include <vector>
#include <stdint.h>

#include "tmm_c_api.h"
#include "tmm_kernels.h"

namespace tmm {

constexpr int OZ_ROW_ALIGN = 256;  // lines are padded to the GEMM tiles (128 x 256)
constexpr int OZ_K_ALIGN = 128;    // k is padded to whole k-blocks (bytes)
constexpr int OZ_DIGIT_BITS = 5;   // |d| <= 2^(w-1) = 16: exact in int8 and in e4m3
constexpr int OZ_MAX_SLICES = 20;
// Line exponent of a line (row of op(A), column of op(B)) holding an Inf or a NaN: the frexp
// exponent of the largest finite magnitude is at most 1024, and the line maximum taken over
// the IEEE bits of |x| puts any non-finite value above every finite one.  The product's
// entries in such a row or column are NaN (IEEE arithmetic would give +-Inf for some of them).
constexpr int OZ_EXP_NONFINITE = 1025;
constexpr int OZ_DEFAULT_SLICES = 13;
// float and complex float contexts: 6 slices (30 bits per line) leave the product within a
// few units of FP32 rounding, below the error of an FP32-accumulating GEMM
constexpr int OZ_DEFAULT_SLICES_FLOAT = 6;
inline int oz_default_slices(int dtype) {
  return dtype == TMM_FLOAT || dtype == TMM_COMPLEX_FLOAT ? OZ_DEFAULT_SLICES_FLOAT : OZ_DEFAULT_SLICES;
}

// digit byte encodings
enum OzEnc : int { OZ_ENC_INT8 = 0, OZ_ENC_E4M3 = 1 };
// slice-product engines
enum OzEngine : int { OZ_ENGINE_IMMA = 0, OZ_ENGINE_TCGEN05 = 1 };

// Digit layouts.  Plain (IMMA engine): [s][rows_pad][k_pad], line-major.
// Blocked (tcgen05 engine): [s][rows_pad/128][k_pad/128][128 lines][128 bytes]:
// the 128-line x 128-byte box a tensor-core stage loads is one contiguous 16 KB
// block of HBM (in the plain layout it is 128 segments of 128 bytes, k_pad apart,
// nearly every one opening its own DRAM page).
constexpr int OZ_BLOCK = 128;

struct OzakiSplit {
  uint8_t* digits = nullptr;  // plain or blocked (above)
  int32_t* exps = nullptr;    // [rows_pad]
  int64_t rows = 0, kk = 0, rows_pad = 0, k_pad = 0;
  int slices = 0;
  int enc = OZ_ENC_INT8;
  int blocked = 0;
};

// byte offset of digit (line r, element l) in slice 0 of a split (add p * rows_pad * k_pad for slice p)
inline __host__ __device__ size_t oz_digit_offset(int64_t r, int64_t l, int64_t k_pad, int blocked) {
  if (!blocked) return (size_t)r * (size_t)k_pad + (size_t)l;
  return ((size_t)(r / OZ_BLOCK) * (size_t)(k_pad / OZ_BLOCK) + (size_t)(l / OZ_BLOCK)) * (OZ_BLOCK * OZ_BLOCK) +
         (size_t)(r % OZ_BLOCK) * OZ_BLOCK + (size_t)(l % OZ_BLOCK);
}

inline int64_t oz_round_up(int64_t v, int64_t q) { return (v + q - 1) / q * q; }

// default engine of new contexts (environment TMM_OZAKI_ENGINE=imma|tcgen05 overrides)
int ozaki_default_engine();
inline int ozaki_encoding(int engine) { return engine == OZ_ENGINE_TCGEN05 ? OZ_ENC_E4M3 : OZ_ENC_INT8; }

// bytes needed by a split tile of rows x kk
size_t ozaki_split_bytes(int64_t rows, int64_t kk, int slices);
// lay out a split tile in a buffer of ozaki_split_bytes bytes, digits encoded for `engine`
OzakiSplit ozaki_split_view(void* base, int64_t rows, int64_t kk, int slices, int engine);

// Split `rows` lines of a device FP64 operand into `out`:
//   trans == OP_N: line r, element l = X[r + l * ld];   otherwise X[l + r * ld].
cudaError_t ozaki_split(const double* X, int64_t ld, Op trans, int64_t rows, int64_t kk, const OzakiSplit& out,
                        cudaStream_t s);

// C (m x n, ldc) = alpha * A_split * B_split^T + beta' * C, beta' = beta on the
// first k-tile (C not read when beta == 0) and 1 afterwards.
// work: ozaki_workspace_bytes(engine) of device memory private to this launch; err: a device
// word that a timed-out wait sets (tcgen05 engine).
cudaError_t ozaki_gemm(const OzakiSplit& A, const OzakiSplit& B, int64_t m, int64_t n, double alpha,
                       double beta, bool first_k_tile, double* C, int64_t ldc, int engine, double* work, int* err,
                       cudaStream_t s);

size_t ozaki_workspace_bytes(int engine);
// workspace that one launch for an m x n product uses (at most ozaki_workspace_bytes)
size_t ozaki_workspace_bytes_for(int engine, int64_t m, int64_t n);
// one-time launch setup of the engine (attributes, occupancy, driver entry points), so
// that later launches can be captured into a CUDA graph
cudaError_t ozaki_prepare(int engine);
// k-blocks (of the engine's k-block size) accumulated between two FP64 drains
int64_t ozaki_pass_blocks(int engine);
int64_t ozaki_k_block(int engine);

// Float, complex float and complex double on the engine (tmm_ozaki_embed.cu).  embed writes
// the real FP64 embedding of op(A) and op(B) (op C conjugates): for float Ahat = op(A)
// (m x k, ld m) and Bhat = op(B) (k x n, ld k); for complex Ahat = [[Re, -Im], [Im, Re]]
// of op(A) (2m x 2k, ld 2m) and Bhat = [Re; Im] of op(B) (2k x n, ld 2k), whose real
// product T (2m x n) holds Re C on top of Im C.  combine writes C = alpha T + beta' C in
// double, rounded once to the context's type (beta' = beta on the first k-tile, C not
// read when it is zero; 1 after); alpha and beta point to scalars of the context's type.
bool ozaki_embedded_dtype(int dtype);
cudaError_t ozaki_embed(int dtype, const void* A, int64_t lda, Op opa, const void* B, int64_t ldb, Op opb, int64_t m,
                        int64_t n, int64_t k, double* Ahat, double* Bhat, cudaStream_t s);
cudaError_t ozaki_combine(int dtype, int64_t m, int64_t n, const void* alpha, const void* beta, bool first,
                          const double* Tm, void* C, int64_t ldc, cudaStream_t s);

// sets the message that tmm_last_error(NULL) returns on the calling thread (tmm_core.cpp)
void set_last_error_message(const char* msg);

// tcgen05 engine (tmm_tcgen05.cu)
size_t ozaki_tc_workspace_bytes();
size_t ozaki_tc_workspace_bytes_for(int64_t m, int64_t n);
cudaError_t ozaki_tc_prepare();
int64_t ozaki_tc_pass_blocks();
int ozaki_tc_k_block();
cudaError_t ozaki_gemm_tc(const OzakiSplit& A, const OzakiSplit& B, int64_t m, int64_t n, double alpha, double beta,
                          bool first_k_tile, double* C, int64_t ldc, double* work, int* err, cudaStream_t s);

// One persistent launch over the tiles of several products (a batch's FP64 problems on the
// Ozaki path): product i multiplies the split planes A, B (tcgen05 blocked layout, the same
// slice count, all inside one arena) into C with its own alpha, beta and first-k-tile flag,
// exactly as ozaki_gemm_tc would on its own.  ozaki_tc_grouped_image writes the launch's
// device records (problems, then the tile list, largest problems first) into out, to be
// copied to device memory at dev_image; ozaki_gemm_tc_grouped launches on them.  work:
// ozaki_tc_workspace_bytes() bytes.
struct GroupedProduct {
  OzakiSplit A, B;
  int64_t m, n;
  double alpha, beta;
  bool first_k_tile;
  double* C;
  int64_t ldc;
};
cudaError_t ozaki_tc_grouped_image(const std::vector<GroupedProduct>& prods, const void* arena, size_t arena_bytes,
                                   std::vector<unsigned char>& out, int* n_items);
cudaError_t ozaki_gemm_tc_grouped(const void* arena, size_t arena_bytes, int slices, const void* dev_image, int n_probs,
                                  int n_items, double* work, int* err, cudaStream_t s);

}  // namespace tmm
