// Drop-in for src/Tiled-MM/device_stream.hpp: a move-only CUDA stream
// (device_stream.hpp:8-75) -- stream(), enqueue_event(), wait_on_event().  A
// default-constructed device_stream owns a new non-blocking stream, as in the
// reference; the ones gpu_context hands out are views of the context's own
// streams and do not destroy them.
#pragma once
#include "device_event.hpp"

typedef struct CUstream_st* cudaStream_t;

namespace gpu {

class device_stream {
 public:
  device_stream() {
    void* s = nullptr;
    check_tmm_status(tmm_stream_create(&s));
    stream_ = static_cast<cudaStream_t>(s);
    owning_ = true;
  }
  ~device_stream() {
    if (owning_) tmm_stream_destroy(stream_);
  }
  device_stream(device_stream&& other) : stream_(other.stream_), owning_(other.owning_) { other.owning_ = false; }
  device_stream& operator=(device_stream&& other) {
    if (this != &other) {
      if (owning_) tmm_stream_destroy(stream_);
      stream_ = other.stream_;
      owning_ = other.owning_;
      other.owning_ = false;
    }
    return *this;
  }
  device_stream(device_stream&) = delete;
  device_stream& operator=(device_stream&) = delete;

  cudaStream_t stream() const { return stream_; }

  // an event recorded on this stream now
  device_event enqueue_event() const {
    device_event e;
    check_tmm_status(tmm_event_record(e.get(), stream_));
    return e;
  }
  // later work on this stream waits for e
  void wait_on_event(device_event& e) const { check_tmm_status(tmm_stream_wait_event(stream_, e.get())); }

  // a non-owning view of a stream owned elsewhere (the C-ABI context)
  static device_stream view(cudaStream_t s) { return device_stream(s); }

 private:
  explicit device_stream(cudaStream_t s) : stream_(s), owning_(false) {}
  cudaStream_t stream_ = nullptr;
  bool owning_ = false;
};

}  // namespace gpu
