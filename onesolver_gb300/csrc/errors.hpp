// errors.hpp -- status handling shared by the CUDA and the host-only parts
// of the C ABI: the thread-local error detail and the exception-to-status
// guard used at every entry point.
#ifndef ONESOLVER_ERRORS_HPP_
#define ONESOLVER_ERRORS_HPP_

#include <cstdarg>
#include <new>
#include <stdexcept>
#include <string>

#include "onesolver.h"

namespace os {

// Set the thread-local error detail and return the status.
os_status fail(os_status st, const char *fmt, ...);

// Exception used inside the library; converted to a status at the ABI.
struct Error : std::runtime_error {
  os_status status;
  Error(os_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] void throw_error(os_status st, const char *fmt, ...);

#define OS_REQUIRE(cond, ...)                                                  \
  do {                                                                         \
    if (!(cond)) ::os::throw_error(OS_INVALID_ARG, __VA_ARGS__);               \
  } while (0)

// Run f, turning exceptions into a status with the error detail recorded.
template <class F> os_status guard(F &&f) {
  try {
    f();
    return OS_OK;
  } catch (const Error &e) {
    return fail(e.status, "%s", e.what());
  } catch (const std::bad_alloc &) {
    return fail(OS_INVALID_ARG, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(OS_INVALID_ARG, "%s", e.what());
  } catch (...) {
    return fail(OS_INVALID_ARG, "unknown error");
  }
}

}  // namespace os

#endif  // ONESOLVER_ERRORS_HPP_
