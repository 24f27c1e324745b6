// guard.h -- no C++ exception crosses the C ABI.  An entry point whose host
// code allocates through the standard library (vectors, strings, new) runs
// its body through guarded(), which turns an exception into an error status
// and the thread's error string instead of terminating the caller's process.
#pragma once
#include <exception>
#include <new>
#include "cageo.h"

namespace cageo {
void set_error(const char* fmt, ...);

template <typename Body>
cageo_status guarded(const char* what, Body&& body) noexcept {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    set_error("%s: out of host memory", what);
  } catch (const std::exception& e) {
    set_error("%s: %s", what, e.what());
  } catch (...) {
    set_error("%s: unexpected host exception", what);
  }
  return CAGEO_ERR_HOST;
}
}  // namespace cageo
