// Drop-in for src/Tiled-MM/tiled_mm.hpp of eth-cscs/Tiled-MM:
//   C = alpha * op(A) * op(B) + beta * C from host pointers, column-major,
//   op in {N, T, C}, on one GPU (tiled_mm.hpp:69-79).
// Same declaration and default arguments.  As in the reference, the template is
// defined in the compiled library, which carries its explicit instantiations
// for float, double, std::complex<float> and std::complex<double>
// (tiled_mm.cpp:626-668); link with libtiledmm_gb300 (CMake: the imported target
// Tiled-MM::Tiled-MM of find_package(Tiled-MM)).  The work is done by the GB300
// kernels behind the C ABI (include/tmm_c_api.h); sizes are 64-bit inside.
#pragma once
#include <complex>

#include "mm_handle.hpp"

namespace gpu {

template <typename Scalar>
void gemm(mm_handle<Scalar>& handle, char trans_a, char trans_b, int m, int n, int k, Scalar alpha, Scalar* a,
          int ld_a, Scalar* b, int ld_b, Scalar beta, Scalar* c, int ld_c, bool pin_host_buffers = true,
          bool copy_c_back = true);

extern template void gemm<float>(mm_handle<float>&, char, char, int, int, int, float, float*, int, float*, int, float,
                                 float*, int, bool, bool);
extern template void gemm<double>(mm_handle<double>&, char, char, int, int, int, double, double*, int, double*, int,
                                  double, double*, int, bool, bool);
extern template void gemm<std::complex<float>>(mm_handle<std::complex<float>>&, char, char, int, int, int,
                                               std::complex<float>, std::complex<float>*, int, std::complex<float>*,
                                               int, std::complex<float>, std::complex<float>*, int, bool, bool);
extern template void gemm<std::complex<double>>(mm_handle<std::complex<double>>&, char, char, int, int, int,
                                                std::complex<double>, std::complex<double>*, int,
                                                std::complex<double>*, int, std::complex<double>,
                                                std::complex<double>*, int, bool, bool);

}  // namespace gpu
