// Drop-in for src/Tiled-MM/device_event.hpp: a move-only CUDA event
// (device_event.hpp:9-80) -- get(), wait(), time_since() -- created and driven
// through the C ABI.  cudaEvent_t is the CUDA runtime's own handle type,
// declared here the way the runtime declares it, so that this header needs no
// CUDA headers and works beside them.
#pragma once
#include "util.hpp"

typedef struct CUevent_st* cudaEvent_t;

namespace gpu {

class device_event {
 public:
  device_event() {
    void* e = nullptr;
    check_tmm_status(tmm_event_create(&e));
    event_ = static_cast<cudaEvent_t>(e);
    valid_ = true;
  }
  ~device_event() {
    if (valid_) tmm_event_destroy(event_);
  }
  device_event(device_event&& other) : valid_(other.valid_), event_(other.event_) { other.valid_ = false; }
  device_event& operator=(device_event&& other) {
    if (this != &other) {
      if (valid_) tmm_event_destroy(event_);
      event_ = other.event_;
      valid_ = other.valid_;
      other.valid_ = false;
    }
    return *this;
  }
  device_event(device_event&) = delete;
  device_event& operator=(device_event&) = delete;

  // the underlying cudaEvent_t
  cudaEvent_t& get() { return event_; }
  // host waits for the event
  void wait() { check_tmm_status(tmm_event_synchronize(event_)); }
  // seconds between `other` and this event
  double time_since(device_event& other) {
    double s = 0.0;
    check_tmm_status(tmm_event_elapsed(other.get(), event_, &s));
    return s;
  }

 private:
  bool valid_ = false;
  cudaEvent_t event_ = nullptr;
};

}  // namespace gpu
