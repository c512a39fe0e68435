// devices.hpp -- device selection and the execution queue.
//
// Mirrors include/helpers/devices.hpp of quantumz-io/oneSolver
// (devices::construct_device_selector, devices.hpp:27-42) and stands in for
// the sycl::queue the reference's solvers take. "gpu" selects the CUDA
// backend; "cpu" and "host" name the reference's SYCL CPU devices, which this
// build does not have (there is no CPU fallback), and any other string is an
// unknown device type, as in the reference.
#ifndef ONESOLVER_DEVICES_HPP_
#define ONESOLVER_DEVICES_HPP_

#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>

#include "onesolver.h"

namespace os {

// Throw the library's last error for a failed call.
inline void check(os_status st) {
  if (st == OS_OK) return;
  const char *msg = os_last_error();
  std::string m = msg ? msg : "";
  if (st == OS_INVALID_ARG || st == OS_PARSE_ERROR) throw std::invalid_argument(m);
  throw std::runtime_error(std::string(os_status_string(st)) + ": " + m);
}

// One CUDA device and stream (replaces sycl::queue).
class Queue {
public:
  explicit Queue(int device = 0) : device_(device) { check(os_ctx_create(device, &ctx_)); }
  Queue(const Queue &) = delete;
  Queue &operator=(const Queue &) = delete;
  ~Queue() {
    if (ctx_) os_ctx_destroy(ctx_);
  }
  os_ctx *ctx() const { return ctx_; }
  int device() const { return device_; }
  std::string device_name() const {
    char buf[256];
    check(os_device_name(device_, buf, sizeof buf));
    return buf;
  }

private:
  int device_;
  os_ctx *ctx_ = nullptr;
};

}  // namespace os

namespace devices {

struct device_selector {
  int device;
};
using device_selector_ptr = std::unique_ptr<device_selector>;

// construct_device_selector (devices.hpp:27-42): "gpu" -> CUDA device 0;
// "cpu"/"host" -> std::runtime_error (no CPU backend in this library); any
// other string -> std::invalid_argument("Unknown device type: ...").
inline device_selector_ptr construct_device_selector(std::string device_type) {
  int dev = -1;
  os_status st = os_select_device(device_type.c_str(), &dev);
  if (st == OS_INVALID_ARG) {
    std::ostringstream error_stream;
    error_stream << "Unknown device type: " << device_type;
    throw std::invalid_argument(error_stream.str());
  }
  os::check(st);
  return device_selector_ptr(new device_selector{dev});
}

}  // namespace devices

#endif  // ONESOLVER_DEVICES_HPP_
