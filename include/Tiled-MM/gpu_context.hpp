// Drop-in for src/Tiled-MM/gpu_context.hpp, reduced to the stream count
// (gpu_context.cpp:45-53); the streams are owned by the C-ABI context.
#pragma once
#include "util.hpp"

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
  void set_num_streams(int n) { check_tmm_status(tmm_set_num_streams(ctx_, n), ctx_); }

 private:
  tmm_context* ctx_;
};

}  // namespace gpu
