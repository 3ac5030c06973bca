// Drop-in for src/Tiled-MM/mm_handle.hpp of eth-cscs/Tiled-MM: the handle
// owns a C-ABI context (streams, tile caches, full-C buffer) for one scalar
// type; same constructor, setters, getters and make_context overloads
// (mm_handle.hpp:11-76).  Non-copyable and non-movable, as in the reference.
#pragma once
#include <complex>
#include <memory>
#include <tuple>

#include "device_buffer.hpp"
#include "device_vector.hpp"
#include "gpu_context.hpp"
#include "tile_dim.hpp"
#include "util.hpp"

namespace gpu {

template <typename Scalar> struct tmm_dtype_of;
template <> struct tmm_dtype_of<float> { static constexpr int value = TMM_FLOAT; };
template <> struct tmm_dtype_of<double> { static constexpr int value = TMM_DOUBLE; };
template <> struct tmm_dtype_of<std::complex<float>> { static constexpr int value = TMM_COMPLEX_FLOAT; };
template <> struct tmm_dtype_of<std::complex<double>> { static constexpr int value = TMM_COMPLEX_DOUBLE; };

template <typename Scalar>
class mm_handle {
 public:
  // creates the streams; device memory is sized lazily by the first gemm (mm_handle.cpp:11-29)
  mm_handle(int streams, int max_tile_m, int max_tile_n, int max_tile_k)
      : ctx_(create(streams, max_tile_m, max_tile_n, max_tile_k)), gpu_ctx_(ctx_), a_buff_(ctx_, 'a', streams),
        b_buff_(ctx_, 'b', streams), c_buff_(ctx_, 'c', streams) {}
  ~mm_handle() { tmm_destroy(ctx_); }

  mm_handle(mm_handle&&) = delete;
  mm_handle(const mm_handle&) = delete;
  mm_handle& operator=(const mm_handle&& other) = delete;

  void set_num_streams(int streams) {
    gpu_ctx_.set_num_streams(streams);
    a_buff_.set_num_streams(streams);
    b_buff_.set_num_streams(streams);
    c_buff_.set_num_streams(streams);
  }
  int get_num_streams() {
    int n = 0;
    check_tmm_status(tmm_get_num_streams(ctx_, &n), ctx_);
    return n;
  }
  gpu_context& get_gpu_context() { return gpu_ctx_; }

  void set_tile_sizes(int tile_m, int tile_n, int tile_k) {
    check_tmm_status(tmm_set_tile_sizes(ctx_, tile_m, tile_n, tile_k), ctx_);
    sync_tiles();
  }
  void set_tile_sizes(int tile) { set_tile_sizes(tile, tile, tile); }
  void set_full_sizes(int m, int n, int k) {
    check_tmm_status(tmm_set_full_sizes(ctx_, m, n, k), ctx_);
    refresh_full_c();
  }
  std::tuple<int, int, int> optimal_tile_sizes(int m, int n, int k) {
    int a, b, c;
    check_tmm_status(tmm_optimal_tile_sizes(ctx_, m, n, k, &a, &b, &c), ctx_);
    return std::tuple<int, int, int>(a, b, c);
  }
  std::tuple<int, int, int> get_max_tile_sizes() {
    int a, b, c;
    check_tmm_status(tmm_get_max_tile_sizes(ctx_, &a, &b, &c), ctx_);
    return std::tuple<int, int, int>(a, b, c);
  }
  void set_streams_and_tiles(int streams, int tile_m, int tile_n, int tile_k) {
    check_tmm_status(tmm_set_streams_and_tiles(ctx_, streams, tile_m, tile_n, tile_k), ctx_);
    a_buff_.set_num_streams(streams);
    b_buff_.set_num_streams(streams);
    c_buff_.set_num_streams(streams);
    sync_tiles();
  }

  device_buffer<Scalar>& get_device_buffer_a() { return a_buff_; }
  device_buffer<Scalar>& get_device_buffer_b() { return b_buff_; }
  device_buffer<Scalar>& get_device_buffer_c() { return c_buff_; }
  device_vector<Scalar>& get_full_device_buffer_c() {
    refresh_full_c();
    return full_c_;
  }

  // additions: the underlying C-ABI context, the multiplication path, the tile policy
  tmm_context* native() { return ctx_; }
  void set_path(int path, int ozaki_slices = 0) { check_tmm_status(tmm_set_path(ctx_, path, ozaki_slices), ctx_); }
  void set_tile_policy(int policy) { check_tmm_status(tmm_set_tile_policy(ctx_, policy), ctx_); }

  // called by gpu::gemm after each multiplication
  void after_gemm() {
    sync_tiles();
    refresh_full_c();
  }

 private:
  static tmm_context* create(int streams, int tm, int tn, int tk) {
    tmm_context* c = nullptr;
    check_tmm_status(tmm_create(tmm_dtype_of<Scalar>::value, streams, tm, tn, tk, &c));
    return c;
  }
  void sync_tiles() {
    int tm, tn, tk;
    check_tmm_status(tmm_get_tile_sizes(ctx_, &tm, &tn, &tk), ctx_);
    a_buff_.set_tile_sizes(tile_dim(tm, tk));
    b_buff_.set_tile_sizes(tile_dim(tk, tn));
    c_buff_.set_tile_sizes(tile_dim(tm, tn));
  }
  void refresh_full_c() {
    void* p = nullptr;
    std::size_t size = 0, cap = 0;
    check_tmm_status(tmm_get_full_c(ctx_, &p, &size, &cap), ctx_);
    full_c_.set_view(static_cast<Scalar*>(p), size, cap);
  }

  tmm_context* ctx_;
  gpu_context gpu_ctx_;
  device_buffer<Scalar> a_buff_, b_buff_, c_buff_;
  device_vector<Scalar> full_c_;
};

// mm_handle.hpp:60-69
template <typename Scalar>
std::unique_ptr<mm_handle<Scalar>> make_context(int streams, int max_tile_m, int max_tile_n, int max_tile_k) {
  return std::unique_ptr<mm_handle<Scalar>>(new mm_handle<Scalar>(streams, max_tile_m, max_tile_n, max_tile_k));
}

// mm_handle.hpp:70-76: 2 streams, tiles of 5000
template <typename Scalar = double>
std::unique_ptr<mm_handle<Scalar>> make_context() {
  return make_context<Scalar>(2, 5000, 5000, 5000);
}

}  // namespace gpu
