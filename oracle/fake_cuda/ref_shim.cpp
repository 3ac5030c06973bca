// ORACLE test infrastructure: a C entry point into the reference's own host
// code (src/Tiled-MM, compiled unmodified against oracle/fake_cuda), so that
// Python tests can run the reference's gpu::gemm on the CPU.
#include <Tiled-MM/tiled_mm.hpp>
#include <Tiled-MM/tiled_matrix.hpp>

#include <complex>
#include <cstdint>
#include <cstring>
#include <exception>

namespace gpu {
// defined in src/Tiled-MM/mm_handle.cpp:89 with external linkage, not declared in a header
int optimal_tile_size(int dim, int curr_tile_size, int max_tile_size);
}

namespace {
template <typename T>
int run(char ta, char tb, int m, int n, int k, const void* alpha, void* a, int lda, void* b, int ldb,
        const void* beta, void* c, int ldc, int streams, int tm, int tn, int tk, int pin, int copy_c_back,
        void* full_c_out, int* tiles_out) {
  try {
    auto ctx = gpu::make_context<T>(streams, tm, tn, tk);
    gpu::gemm<T>(*ctx, ta, tb, m, n, k, *(const T*)alpha, (T*)a, lda, (T*)b, ldb, *(const T*)beta, (T*)c, ldc,
                 pin != 0, copy_c_back != 0);
    if (tiles_out) {
      auto t = ctx->get_device_buffer_c().get_tile_sizes();
      tiles_out[0] = t.rows();
      tiles_out[1] = t.cols();
      tiles_out[2] = ctx->get_device_buffer_a().get_tile_sizes().cols();
    }
    if (!copy_c_back && full_c_out) {
      auto& fc = ctx->get_full_device_buffer_c();
      std::memcpy(full_c_out, fc.data(), sizeof(T) * (size_t)m * (size_t)n);
    }
  } catch (const std::exception&) {
    return -1;
  }
  return 0;
}
}  // namespace

extern "C" {
int ref_optimal_tile_size(int dim, int curr, int max_tile) { return gpu::optimal_tile_size(dim, curr, max_tile); }

// tiled_matrix geometry of a rows x cols matrix cut in tr x tc tiles:
// out = {n_tiles_row, n_tiles_col, tile_rows(coord), tile_cols(coord), tile_offset(coord)}
void ref_tiled_matrix_info(int rows, int cols, int ld, int tr, int tc, int ci, int cj, long long* out5) {
  gpu::tiled_matrix<double> t(nullptr, rows, cols, ld, gpu::tile_dim(tr, tc));
  out5[0] = t.num_tiles_row();
  out5[1] = t.num_tiles_col();
  auto d = t.tile_dimensions(gpu::tile_coord(ci, cj));
  out5[2] = d.rows();
  out5[3] = d.cols();
  out5[4] = t.tile_offset(gpu::tile_coord(ci, cj));
}

// dtype: 0 float, 1 double, 2 complex<float>, 3 complex<double>
int ref_gemm(int dtype, char ta, char tb, int m, int n, int k, const void* alpha, void* a, int lda, void* b,
             int ldb, const void* beta, void* c, int ldc, int streams, int tm, int tn, int tk, int pin,
             int copy_c_back, void* full_c_out, int* tiles_out) {
  switch (dtype) {
    case 0: return run<float>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, streams, tm, tn, tk, pin, copy_c_back, full_c_out, tiles_out);
    case 1: return run<double>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, streams, tm, tn, tk, pin, copy_c_back, full_c_out, tiles_out);
    case 2: return run<std::complex<float>>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, streams, tm, tn, tk, pin, copy_c_back, full_c_out, tiles_out);
    case 3: return run<std::complex<double>>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, streams, tm, tn, tk, pin, copy_c_back, full_c_out, tiles_out);
  }
  return -1;
}
}
