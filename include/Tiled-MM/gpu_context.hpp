// Drop-in for src/Tiled-MM/gpu_context.hpp: the streams of a handle
// (gpu_context.hpp:13-42, gpu_context.cpp:6-57).  The streams are owned by the
// C-ABI context; get_stream / get_device_stream / get_result_stream return
// them (the device_stream objects are views), enqueue_event records on one.
// The reference's get_blas_handle has no counterpart: this library calls no
// BLAS (every tile product is its own kernel).
#pragma once
#include <memory>
#include <stdexcept>
#include <vector>

#include "device_stream.hpp"

namespace gpu {

class gpu_context {
 public:
  explicit gpu_context(tmm_context* ctx) : ctx_(ctx) {}
  gpu_context(gpu_context&&) = delete;
  gpu_context(gpu_context&) = delete;

  int get_num_streams() const {
    int n = 0;
    check_tmm_status(tmm_get_num_streams(ctx_, &n), ctx_);
    return n;
  }
  void set_num_streams(int n) {
    check_tmm_status(tmm_set_num_streams(ctx_, n), ctx_);
    views_.clear();
  }

  // compute stream stream_id (gpu_context.cpp:27-32): out of range throws, as in the reference
  cudaStream_t get_stream(int stream_id) const {
    void* s = nullptr;
    if (tmm_get_stream(ctx_, stream_id, &s) != TMM_SUCCESS)
      throw std::runtime_error("index of gpu blas handle has to be in the range [0, n_streams)");
    return static_cast<cudaStream_t>(s);
  }
  device_stream& get_device_stream(int stream_id) {
    const int n = get_num_streams();
    if (stream_id < 0 || stream_id >= n)
      throw std::runtime_error("index of gpu blas handle has to be in the range [0, n_streams)");
    if ((int)views_.size() != n) {
      views_.clear();
      for (int i = 0; i < n; ++i) views_.push_back(device_stream::view(get_stream(i)));
    }
    return views_[(size_t)stream_id];
  }
  device_event enqueue_event(int stream_id) const {
    device_event e;
    check_tmm_status(tmm_event_record(e.get(), get_stream(stream_id)), ctx_);
    return e;
  }
  // the stream results return to the host on (gpu_context.cpp:55-57)
  device_stream& get_result_stream() {
    if (!result_) {
      void* s = nullptr;
      check_tmm_status(tmm_get_result_stream(ctx_, &s), ctx_);
      result_.reset(new device_stream(device_stream::view(static_cast<cudaStream_t>(s))));
    }
    return *result_;
  }

 private:
  tmm_context* ctx_;
  std::vector<device_stream> views_;
  std::unique_ptr<device_stream> result_;
};

}  // namespace gpu
