// Drop-in for src/Tiled-MM/device_buffer.hpp: the device tiles of one operand
// of a handle (device_buffer.hpp:14-83) -- tile sizes, stream count,
// stream_buffer(i) and data() -- read from the C-ABI context, which owns the
// memory.  C: the first result-tile slot of compute stream i.  A and B: this
// library keeps device tile caches (a tile is copied once and reused) instead
// of one slot per stream, so stream_buffer(i) is cache slot i.  A pointer is
// nullptr until the first gemm has sized the buffers.
#pragma once
#include <memory>

#include "tile_dim.hpp"
#include "util.hpp"

namespace gpu {

template <typename T>
class device_buffer {
 public:
  device_buffer() = default;
  explicit device_buffer(int streams) : n_streams_(streams) {}
  device_buffer(tmm_context* ctx, char which, int streams) : ctx_(ctx), which_(which), n_streams_(streams) {}

  T* stream_buffer(int stream_id) {
    if (stream_id < 0 || stream_id >= n_streams_)
      throw std::runtime_error("stream id in device buffer has to be in the range [0, n_streams)");
    return lookup(stream_id);
  }
  T* data() { return lookup(-1); }

  void set_num_streams(int s) { n_streams_ = s; }
  int get_num_streams() const { return n_streams_; }
  void set_tile_sizes(tile_dim t) { tile_ = t; }
  tile_dim get_tile_sizes() const { return tile_; }
  void set_streams_and_tiles(int streams, tile_dim t) {
    n_streams_ = streams;
    tile_ = t;
  }

 private:
  T* lookup(int stream_id) {
    if (!ctx_) return nullptr;
    void* p = nullptr;
    check_tmm_status(tmm_get_device_buffer(ctx_, which_, stream_id, &p), ctx_);
    return static_cast<T*>(p);
  }
  tmm_context* ctx_ = nullptr;
  char which_ = 'c';
  int n_streams_ = 0;
  tile_dim tile_;
};

}  // namespace gpu
