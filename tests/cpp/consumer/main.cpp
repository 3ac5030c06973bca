// Uses the drop-in API the way a caller of the reference does: gpu::gemm for
// the four scalar types (explicit instantiations in the library), the handle's
// context streams and events, and its device buffers.
#include <Tiled-MM/tiled_mm.hpp>
#include <Tiled-MM/util.hpp>

#include <complex>
#include <cstdio>

#ifndef TILED_MM_CUDA
#error "the Tiled-MM target exports TILED_MM_CUDA"
#endif

template <typename T>
int run(int n) {
  auto ctx = gpu::make_context<T>(2, 64, 64, 64);
  T* a = gpu::malloc_pinned<T>((size_t)n * n, T(1));
  T* b = gpu::malloc_pinned<T>((size_t)n * n, T(1));
  T* c = gpu::malloc_pinned<T>((size_t)n * n, T(0));
  gpu::gemm<T>(*ctx, 'N', 'N', n, n, n, T(1), a, n, b, n, T(0), c, n);
  auto& gctx = ctx->get_gpu_context();
  auto e0 = gctx.enqueue_event(0);
  auto& rs = gctx.get_result_stream();
  auto e1 = rs.enqueue_event();
  e1.wait();
  (void)gctx.get_stream(1);
  (void)ctx->get_device_buffer_c().stream_buffer(1);
  const bool ok = c[0] == T(n);
  gpu::free_pinned(a);
  gpu::free_pinned(b);
  gpu::free_pinned(c);
  return ok ? 0 : 1;
}

int main() {
  int bad = run<float>(100) + run<double>(100) + run<std::complex<float>>(100) + run<std::complex<double>>(100);
  std::printf(bad ? "FAILED\n" : "consumer OK\n");
  return bad;
}
