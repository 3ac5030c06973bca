// Drop-in for src/Tiled-MM/tile_dim.hpp: rows x cols of a tile (64-bit size).
#pragma once
#include <cstdint>

namespace gpu {

class tile_dim {
 public:
  tile_dim() = default;
  tile_dim(int n_rows, int n_cols) : n_rows_(n_rows), n_cols_(n_cols) {}
  int rows() const { return n_rows_; }
  int cols() const { return n_cols_; }
  void set_rows(int r) { n_rows_ = r; }
  void set_cols(int c) { n_cols_ = c; }
  std::int64_t size() const { return (std::int64_t)n_rows_ * (std::int64_t)n_cols_; }

 private:
  int n_rows_ = 0;
  int n_cols_ = 0;
};

}  // namespace gpu
