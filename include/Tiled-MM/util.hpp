// Drop-in for src/Tiled-MM/util.hpp of eth-cscs/Tiled-MM: status checks that
// throw std::runtime_error("GPU ERROR") (util.hpp:13-36) and the memory
// helpers users call (util.hpp:56-118), implemented over the C ABI.
#pragma once
#include <algorithm>
#include <cstddef>
#include <iostream>
#include <stdexcept>
#include <string>

#include "../tmm_c_api.h"

namespace gpu {

inline void check_tmm_status(int status, tmm_context* ctx = nullptr) {
  if (status != TMM_SUCCESS) {
    std::cerr << "error: GPU API call : " << tmm_status_string(status) << ": " << tmm_last_error(ctx) << std::endl;
    throw std::runtime_error("GPU ERROR");
  }
}

// allocate space on the GPU for n instances of T (util.hpp:56-62)
template <typename T>
T* malloc_device(std::size_t n) {
  void* p = nullptr;
  check_tmm_status(tmm_malloc_device(n * sizeof(T), &p));
  return static_cast<T*>(p);
}

template <typename T>
void free_device(T* p) {
  check_tmm_status(tmm_free_device(p));
}

// page-locked host allocation filled with value (util.hpp:64-72)
template <typename T>
T* malloc_pinned(std::size_t n, T value = T()) {
  void* p = nullptr;
  check_tmm_status(tmm_malloc_pinned(n * sizeof(T), &p));
  T* t = static_cast<T*>(p);
  std::fill(t, t + n, value);
  return t;
}

template <typename T>
void free_pinned(T* p) {
  check_tmm_status(tmm_free_pinned(p));
}

// copy n*T host -> device / device -> host (util.hpp:79-88)
template <typename T>
void copy_to_device(const T* from, T* to, std::size_t n) {
  check_tmm_status(tmm_copy_to_device(from, to, n * sizeof(T)));
}

template <typename T>
void copy_to_host(const T* from, T* to, std::size_t n) {
  check_tmm_status(tmm_copy_to_host(from, to, n * sizeof(T)));
}

// asynchronous copies on a CUDA stream (cudaStream_t passed as void*; NULL = default stream)
// (util.hpp:90-118)
template <typename T>
void copy_to_device_async(const T* from, T* to, std::size_t n, void* stream = nullptr) {
  check_tmm_status(tmm_memcpy_async(to, from, n * sizeof(T), stream));
}

template <typename T>
void copy_to_host_async(const T* from, T* to, std::size_t n, void* stream = nullptr) {
  check_tmm_status(tmm_memcpy_async(to, from, n * sizeof(T), stream));
}

}  // namespace gpu
