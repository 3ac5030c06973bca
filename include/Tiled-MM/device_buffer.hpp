// Drop-in for src/Tiled-MM/device_buffer.hpp, reduced to what callers read:
// the tile sizes the handle's buffers were last sized for
// (device_buffer.hpp:181-184).  The device tiles themselves are owned by the
// context's tile caches.
#pragma once
#include "tile_dim.hpp"

namespace gpu {

template <typename T>
class device_buffer {
 public:
  device_buffer() = default;
  explicit device_buffer(int streams) : n_streams_(streams) {}
  tile_dim get_tile_sizes() const { return tile_; }
  void set_tile_sizes(tile_dim t) { tile_ = t; }
  void set_num_streams(int s) { n_streams_ = s; }
  int get_num_streams() const { return n_streams_; }

 private:
  int n_streams_ = 0;
  tile_dim tile_;
};

}  // namespace gpu
