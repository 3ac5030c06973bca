// C++ parity driver for the drop-in API: the reference's test program
// semantics (tests/test-multiply.cpp) against include/Tiled-MM/*.hpp.
//
// Inputs are the reference test's known-answer integers 0..9 from one
// std::mt19937(42), drawn for A, B, C (test-multiply.cpp:58-66).  The check
// value is a host triple loop (exact for these integers while 81 k < 2^53);
// both copy modes are run and compared with |x - y| <= 1e-6
// (test-multiply.cpp:89-98, 298-346).  Exit status 0 when CORRECT.
//
//   test_multiply_gb300 m n k tile_m tile_n tile_k n_streams trans alpha beta [ld_pad] [ozaki_slices]
#include <Tiled-MM/tiled_mm.hpp>
#include <Tiled-MM/util.hpp>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

int main(int argc, char** argv) {
  if (argc < 11) {
    std::fprintf(stderr, "usage: %s m n k tile_m tile_n tile_k n_streams trans alpha beta [ld_pad] [ozaki_slices]\n", argv[0]);
    return 2;
  }
  int m = std::atoi(argv[1]), n = std::atoi(argv[2]), k = std::atoi(argv[3]);
  int tm = std::atoi(argv[4]), tn = std::atoi(argv[5]), tk = std::atoi(argv[6]);
  int streams = std::atoi(argv[7]);
  std::string trans = argv[8];
  double alpha = std::atof(argv[9]), beta = std::atof(argv[10]);
  int pad = argc > 11 ? std::atoi(argv[11]) : 0;
  int slices = argc > 12 ? std::atoi(argv[12]) : 0;
  char ta = std::toupper(trans[0]), tb = std::toupper(trans[1]);
  int a_m = ta == 'N' ? m : k, a_n = ta == 'N' ? k : m;
  int b_m = tb == 'N' ? k : n, b_n = tb == 'N' ? n : k;
  int ld_a = a_m + pad, ld_b = b_m + pad, ld_c = m + pad;

  size_t na = (size_t)ld_a * a_n, nb = (size_t)ld_b * b_n, nc = (size_t)ld_c * n;
  double* a = gpu::malloc_pinned<double>(na, 1);
  double* b = gpu::malloc_pinned<double>(nb, 1);
  double* c = gpu::malloc_pinned<double>(nc, 0);
  std::vector<double> c2(nc), cref(nc);
  std::mt19937 rng(42);
  std::uniform_int_distribution<int> dist(0, 9);
  for (size_t i = 0; i < na; ++i) a[i] = dist(rng);
  for (size_t i = 0; i < nb; ++i) b[i] = dist(rng);
  for (size_t i = 0; i < nc; ++i) c[i] = dist(rng);
  std::vector<double> corig(c, c + nc);
  for (size_t i = 0; i < nc; ++i) c2[i] = cref[i] = c[i];

  // host check value
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0;
      for (int l = 0; l < k; ++l) {
        double x = ta == 'N' ? a[i + (size_t)l * ld_a] : a[l + (size_t)i * ld_a];
        double y = tb == 'N' ? b[l + (size_t)j * ld_b] : b[j + (size_t)l * ld_b];
        s += x * y;
      }
      double& r = cref[i + (size_t)j * ld_c];
      r = alpha * s + (beta != 0 ? beta * r : 0.0);
    }

  auto ctx = gpu::make_context<double>(streams, tm, tn, tk);
  if (slices > 0) ctx->set_path(TMM_PATH_OZAKI, slices);
  gpu::gemm(*ctx, ta, tb, m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c, false, true);
  bool correct = true;
  for (int j = 0; j < n && correct; ++j)
    for (int i = 0; i < m; ++i)
      if (std::fabs(c[i + (size_t)j * ld_c] - cref[i + (size_t)j * ld_c]) > 1e-6) { correct = false; break; }
  std::printf("copy_c_back=1 %s\n", correct ? "ok" : "MISMATCH");

  gpu::gemm(*ctx, ta, tb, m, n, k, alpha, a, ld_a, b, ld_b, beta, c2.data(), ld_c, true, false);
  std::vector<double> full((size_t)m * n);
  auto& dv = ctx->get_full_device_buffer_c();
  if (dv.size() != (size_t)m * n) correct = false;
  gpu::copy_to_host(dv.data(), full.data(), (size_t)m * n);
  bool correct2 = true;
  for (int j = 0; j < n && correct2; ++j)
    for (int i = 0; i < m; ++i)
      if (std::fabs(full[i + (size_t)j * m] - cref[i + (size_t)j * ld_c]) > 1e-6) { correct2 = false; break; }
  std::printf("copy_c_back=0 %s\n", correct2 ? "ok" : "MISMATCH");
  for (size_t i = 0; i < nc; ++i)
    if (c2[i] != corig[i]) correct2 = false;  // host C untouched without copy-back
  auto t = ctx->get_device_buffer_c().get_tile_sizes();
  std::printf("tiles %d %d %d\n", t.rows(), t.cols(), ctx->get_device_buffer_a().get_tile_sizes().cols());
  correct = correct && correct2;
  std::printf("The result is %s\n", correct ? "CORRECT" : "NOT CORRECT");
  gpu::free_pinned(a);
  gpu::free_pinned(b);
  gpu::free_pinned(c);
  return !correct;
}
