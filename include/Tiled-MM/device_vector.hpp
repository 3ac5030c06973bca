// Drop-in for src/Tiled-MM/device_vector.hpp: a grow-only device array
// (capacity 1.2x when it grows, device_vector.hpp:93-107).  An instance
// returned by mm_handle::get_full_device_buffer_c() is a view of the
// context's full-C buffer and does not own it.
#pragma once
#include <cmath>
#include <cstddef>

#include "util.hpp"

namespace gpu {

template <typename mm_scalar> class mm_handle;

template <typename T>
class device_vector {
 public:
  device_vector() = default;
  explicit device_vector(std::size_t n) { resize(n); }
  device_vector(device_vector&) = delete;
  device_vector& operator=(device_vector&) = delete;
  device_vector& operator=(device_vector&& other) {
    if (this != &other) {
      release();
      data_ = other.data_;
      size_ = other.size_;
      capacity_ = other.capacity_;
      owning_ = other.owning_;
      other.data_ = nullptr;
      other.size_ = other.capacity_ = 0;
    }
    return *this;
  }
  ~device_vector() { release(); }

  T* data() { return data_; }
  std::size_t size() { return size_; }
  std::size_t capacity() { return capacity_; }

  void resize(std::size_t size) {
    if (size == 0) return;
    if (size > capacity_) {
      if (!owning_) throw std::runtime_error("device_vector: cannot resize a view of the context's C buffer");
      release();
      capacity_ = (std::size_t)std::ceil(1.2 * (double)size);
      data_ = malloc_device<T>(capacity_);
    }
    size_ = size;
  }

 private:
  template <typename S> friend class mm_handle;
  void set_view(T* p, std::size_t size, std::size_t capacity) {
    owning_ = false;
    data_ = p;
    size_ = size;
    capacity_ = capacity;
  }
  void release() {
    if (owning_ && data_) tmm_free_device(data_);
    data_ = nullptr;
    size_ = capacity_ = 0;
  }
  T* data_ = nullptr;
  std::size_t size_ = 0;
  std::size_t capacity_ = 0;
  bool owning_ = true;
};

}  // namespace gpu
