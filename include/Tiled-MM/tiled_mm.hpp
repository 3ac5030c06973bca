// Drop-in for src/Tiled-MM/tiled_mm.hpp of eth-cscs/Tiled-MM:
//   C = alpha * op(A) * op(B) + beta * C from host pointers, column-major,
//   op in {N, T, C}, on one GPU (tiled_mm.hpp:69-79).
// Same signature and default arguments; the work is done by the GB300
// library through the C ABI (include/tmm_c_api.h).  Sizes are 64-bit inside.
#pragma once
#include "mm_handle.hpp"

namespace gpu {

template <typename Scalar>
void gemm(mm_handle<Scalar>& handle, char trans_a, char trans_b, int m, int n, int k, Scalar alpha, Scalar* a,
          int ld_a, Scalar* b, int ld_b, Scalar beta, Scalar* c, int ld_c, bool pin_host_buffers = true,
          bool copy_c_back = true) {
  int st = tmm_gemm(handle.native(), trans_a, trans_b, m, n, k, &alpha, a, ld_a, b, ld_b, &beta, c, ld_c,
                    pin_host_buffers ? 1 : 0, copy_c_back ? 1 : 0);
  check_tmm_status(st, handle.native());
  handle.after_gemm();
}

}  // namespace gpu
