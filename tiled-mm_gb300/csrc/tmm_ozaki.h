// Internal interface of the Ozaki split-precision FP64 engine (not part of the C ABI).
//
// A double tile op(X) (lines x kk along k) is split into s digit planes of
// small integers |d| <= 16 stored one byte per digit, K-major
// [s][rows_pad][k_pad], plus one power-of-two exponent per line; the product
// of two split tiles is a sum of exact integer tile GEMMs on the tensor cores,
// recombined in FP64 with the alpha/beta epilogue fused.  tmm_ozaki.cu holds
// the algorithm and its published sources.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tmm_kernels.h"

namespace tmm {

constexpr int OZ_ROW_ALIGN = 128;  // lines are padded to the GEMM tile
constexpr int OZ_K_ALIGN = 128;    // k is padded to whole k-blocks (bytes)
constexpr int OZ_DIGIT_BITS = 5;   // |d| <= 2^(w-1) = 16: exact in int8 and in e4m3
constexpr int OZ_MAX_SLICES = 20;
constexpr int OZ_DEFAULT_SLICES = 13;

// digit byte encodings
enum OzEnc : int { OZ_ENC_INT8 = 0, OZ_ENC_E4M3 = 1 };
// slice-product engines
enum OzEngine : int { OZ_ENGINE_IMMA = 0, OZ_ENGINE_TCGEN05 = 1 };

struct OzakiSplit {
  uint8_t* digits = nullptr;  // [s][rows_pad][k_pad]
  int32_t* exps = nullptr;    // [rows_pad]
  int64_t rows = 0, kk = 0, rows_pad = 0, k_pad = 0;
  int slices = 0;
  int enc = OZ_ENC_INT8;
};

inline int64_t oz_round_up(int64_t v, int64_t q) { return (v + q - 1) / q * q; }

// the engine used by ozaki_split/ozaki_gemm (environment TMM_OZAKI_ENGINE=imma|tcgen05)
int ozaki_engine();
int ozaki_encoding();

// bytes needed by a split tile of rows x kk
size_t ozaki_split_bytes(int64_t rows, int64_t kk, int slices);
// lay out a split tile in a buffer of ozaki_split_bytes bytes (encoding of the current engine)
OzakiSplit ozaki_split_view(void* base, int64_t rows, int64_t kk, int slices);

// Split `rows` lines of a device FP64 operand into `out`:
//   trans == OP_N: line r, element l = X[r + l * ld];   otherwise X[l + r * ld].
cudaError_t ozaki_split(const double* X, int64_t ld, Op trans, int64_t rows, int64_t kk, const OzakiSplit& out,
                        cudaStream_t s);

// C (m x n, ldc) = alpha * A_split * B_split^T + beta' * C, beta' = beta on the
// first k-tile (C not read when beta == 0) and 1 afterwards.
cudaError_t ozaki_gemm(const OzakiSplit& A, const OzakiSplit& B, int64_t m, int64_t n, double alpha,
                       double beta, bool first_k_tile, double* C, int64_t ldc, cudaStream_t s);

// k-blocks (of the engine's k-block size) accumulated between two FP64 drains
int64_t ozaki_pass_blocks();
int64_t ozaki_k_block();

}  // namespace tmm
