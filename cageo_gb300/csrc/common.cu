// common.cu -- error state, scratch allocation, version.
#include <cstdarg>
#include <cstring>
#include "common.cuh"

namespace cageo {

static thread_local char g_last_error[512] = "no error";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

cageo_status cuda_fail(cudaError_t e, const char* what) {
  set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
  return CAGEO_ERR_CUDA;
}

cageo_status Scratch::acquire(void* given, size_t given_bytes, size_t need,
                              cudaStream_t s) {
  stream = s;
  if (given) {
    if (given_bytes < need) {
      set_error("workspace of %zu bytes is smaller than the %zu bytes needed",
                given_bytes, need);
      return CAGEO_ERR_ARGUMENT;
    }
    if ((uintptr_t)given % 256 != 0) {
      set_error("workspace must start on a 256-byte boundary (as cudaMalloc returns)");
      return CAGEO_ERR_ARGUMENT;
    }
    ptr = given;
    owned = false;
    return CAGEO_OK;
  }
  cudaError_t e = cudaMallocAsync(&ptr, need ? need : 16, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(workspace)");
  owned = true;
  return CAGEO_OK;
}

Scratch::~Scratch() {
  if (owned && ptr) cudaFreeAsync(ptr, stream);
}

}  // namespace cageo

extern "C" const char* cageo_version(void) { return "cageo-gb300 0.1 (sm_103a)"; }

extern "C" const char* cageo_last_error_string(void) {
  return cageo::g_last_error;
}
