// pitfill_static.cu -- pit filling that allocates nothing.
//
// cageo_pitfill needs about 5 bytes of device scratch per cell, which it
// takes from the caller's workspace or allocates with cudaMallocAsync.
// Some callers can do neither: a host application that has reserved the
// GPU's memory for its own allocator and forbids plug-ins from calling
// cudaMalloc, or a loop that must not pay an allocation's latency or
// implicit synchronization.  cageo_pitfill_static serves them from a fixed
// scratch array compiled into this library instead.
//
// The array is a file-scope __device__ variable of kStaticFillBytes
// (64 MiB): every GPU that loads the library holds it until the process
// exits.  It fits the fill workspace of grids up to 2048 x 2048 cells
// (about 52 MiB there); larger grids are refused.  All calls share it and it
// keeps the last call's contents, so each call first clears the parts that
// must start at zero; calls that overlap on the GPU (other streams, other
// host threads) race on it and must be serialized by the caller.
#include <mutex>
#include "common.cuh"
#include "pitfill.cuh"

namespace cageo {

constexpr size_t kStaticFillBytes = (size_t)64 << 20;

static __device__ __align__(256) unsigned char g_static_fill_scratch[kStaticFillBytes];

// Host code cannot use the array's name as a device address; its address
// on each device is looked up once, with that device current.
static void* g_static_fill_addr[kMaxDevices] = {};
static std::mutex g_static_fill_mutex;

static cageo_status static_fill_scratch(void** out) {
  int dev = 0;
  CAGEO_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device %d is beyond the %d devices this library tracks", dev, kMaxDevices);
    return CAGEO_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_static_fill_mutex);
  if (!g_static_fill_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_fill_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static fill scratch)");
    g_static_fill_addr[dev] = p;
  }
  *out = g_static_fill_addr[dev];
  return CAGEO_OK;
}

}  // namespace cageo

using namespace cageo;

extern "C" size_t cageo_pitfill_static_max_bytes(void) { return kStaticFillBytes; }

extern "C" cageo_status cageo_pitfill_static(float* d_dem, float* d_filled, int W, int H,
                                             float nodata_dem, int mode, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_dem && d_filled && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(W <= 65535 && H <= 65535, "width and height must be <= 65535");
  CAGEO_CHECK_ARG(d_dem != d_filled, "the filled grid must not alias the DEM");
  CAGEO_CHECK_ARG(mode == CAGEO_FILL_CPU_COMPAT || mode == CAGEO_FILL_EXACT, "fill mode");
  const size_t need = fill_workspace_bytes(W, H);
  if (need > kStaticFillBytes) {
    set_error("a %d x %d grid needs %zu bytes of fill scratch; the static scratch holds %zu "
              "(grids up to 2048 x 2048): use cageo_pitfill with a workspace",
              W, H, need, kStaticFillBytes);
    return CAGEO_ERR_ARGUMENT;
  }
  void* base = nullptr;
  cageo_status st = static_fill_scratch(&base);
  if (st) return st;
  FillWork w = fill_carve(base, W, H);
  if ((st = fill_reset_scalars(w, stream))) return st;
  if (mode == CAGEO_FILL_EXACT) {
    if ((st = fill_run_exact(d_dem, d_filled, w, nodata_dem, nullptr, stream))) return st;
  } else {
    if ((st = fill_quantize_min(d_dem, w, nodata_dem, stream))) return st;
    if ((st = fill_run(d_dem, d_filled, w, nodata_dem, stream))) return st;
  }
  CAGEO_CUDA(cudaStreamSynchronize(stream));
  return fill_check_status(w, nullptr);
}
