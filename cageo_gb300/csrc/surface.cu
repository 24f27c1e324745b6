// surface.cu -- A4 realistic DEM and A5 stream burning.
//
// Stream burning (src/streamburning/StreamBurningAlgorithmCPUOpenMP.h:32-82)
// visits the offsets within the bevel radius nearest first (sorted by
// (d^2, y, x), src/streamburning/StreamBurningAlgorithm.h:140-167) and
// scales a cell by dist/bevel at the first offset that holds a stream cell
// whose elevation is not NODATA; stream cells themselves become 0.  The
// reference runs it in place, so the elevation it tests belongs to a
// neighbour that may already have been zeroed.  The stage kernel here
// resolves that the way a raster-order pass does: neighbours before the
// cell in raster order test 0, later ones their input value.
//
// The pipeline instead precomputes, once per stream raster, a per-cell code
// (front.cuh): the nearest-stream distance class and the stream bits.  That
// code equals the stage result whenever no stream cell's realistic elevation
// equals NODATA and NODATA is not 0; the front kernel flags any realization
// where that does not hold and the pipeline recomputes it with the stage
// kernels.
#include <algorithm>
#include <cmath>
#include <vector>
#include "common.cuh"
#include "front.cuh"
#include "stage_math.cuh"

namespace cageo {

struct BurnOffsets {
  int count;
  signed char dx[120], dy[120];
  unsigned char cls[120];                    // 1-based distance class
  float factor[kMaxBurnClasses + 1];         // factor[cls] = dist / bevel
};

// Offsets sorted like the reference; the factor arithmetic is the
// reference's: sqrt of a float sum of squares, divided by the int radius.
BurnOffsets make_burn_offsets(int bevel) {
  struct E { int d, x, y; };
  std::vector<E> v;
  for (int y = -bevel; y <= bevel; y++)
    for (int x = -bevel; x <= bevel; x++) {
      if (x == 0 && y == 0) continue;
      if (x * x + y * y <= bevel * bevel) v.push_back({x * x + y * y, x, y});
    }
  std::stable_sort(v.begin(), v.end(), [](const E& a, const E& b) {
    if (a.d != b.d) return a.d < b.d;
    if (a.y != b.y) return a.y < b.y;
    return a.x < b.x;
  });
  BurnOffsets o{};
  o.count = (int)v.size();
  int cls = 0, last = -1;
  for (int i = 0; i < o.count; i++) {
    if (v[i].d != last) {
      cls++;
      last = v[i].d;
      volatile float xd = (float)(-v[i].x), yd = (float)(-v[i].y);
      volatile float s = xd * xd + yd * yd;
      volatile float dist = std::sqrt((float)s);
      o.factor[cls] = dist / (float)bevel;
    }
    o.dx[i] = (signed char)v[i].x;
    o.dy[i] = (signed char)v[i].y;
    o.cls[i] = (unsigned char)cls;
  }
  return o;
}

__global__ void realistic_kernel(const float* __restrict__ dem, float* __restrict__ field,
                                 int64_t n, float nodata) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) field[i] = realistic_value(dem[i], field[i], nodata);
}

// General stage kernel: reads `src` (the input elevations), writes `dst`.
__global__ void burn_stage_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                  const float* __restrict__ streams, int W, int H,
                                  float nodata_dem, float nodata_stream, BurnOffsets o) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  int64_t i = (int64_t)y * W + x;
  float v = streams[i] != nodata_stream ? 0.0f : src[i];
  for (int k = 0; k < o.count; k++) {
    int nx = x + o.dx[k], ny = y + o.dy[k];
    if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
    int64_t n = (int64_t)ny * W + nx;
    if (streams[n] == nodata_stream) continue;
    float e = n < i ? 0.0f : src[n];
    if (e != nodata_dem) {
      v = __fmul_rn(v, o.factor[o.cls[k]]);
      break;
    }
  }
  dst[i] = v;
}

// Pipeline code: nearest burning stream within the radius (all stream
// elevations assumed non-NODATA) plus the stream bits.
__global__ void burn_code_kernel(const float* __restrict__ streams, uint8_t* __restrict__ code,
                                 int W, int H, float nodata_stream, BurnOffsets o) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  int64_t i = (int64_t)y * W + x;
  float s = streams[i];
  uint8_t c = 0;
  if (s != nodata_stream) c |= kCodeBurnStream;
  if (s >= 0.0f) c |= kCodeTraceStream;
  for (int k = 0; k < o.count; k++) {
    int nx = x + o.dx[k], ny = y + o.dy[k];
    if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
    if (streams[(int64_t)ny * W + nx] != nodata_stream) {
      c |= o.cls[k];
      break;
    }
  }
  code[i] = c;
}

cageo_status launch_burn_code(const float* streams, uint8_t* code, int W, int H,
                              float nodata_stream, int bevel, float* factor_out,
                              cudaStream_t s) {
  BurnOffsets o = make_burn_offsets(bevel);
  for (int k = 0; k <= kMaxBurnClasses; k++) factor_out[k] = o.factor[k];
  dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
  burn_code_kernel<<<g, b, 0, s>>>(streams, code, W, H, nodata_stream, o);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status launch_realistic(const float* dem, float* field, int64_t n, float nodata,
                              cudaStream_t s) {
  realistic_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dem, field, n, nodata);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status launch_burn_stage(const float* src, float* dst, const float* streams, int W,
                               int H, int bevel, float nodata_dem, float nodata_stream,
                               cudaStream_t s) {
  BurnOffsets o = make_burn_offsets(bevel);
  dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
  burn_stage_kernel<<<g, b, 0, s>>>(src, dst, streams, W, H, nodata_dem, nodata_stream, o);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

// Byte image of a count grid for the JPEG output
// (src/utils/tobytearray/ToByteArrayAlgorithmCPUOpenMP.h:33-52):
// (uint8) rintf(255 * ((v - min) / max)) with the grid's min and max.
__global__ void minmax_kernel(const float* __restrict__ in, int64_t n, unsigned int* mm) {
  float lo = kInf, hi = -kInf;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = in[i];
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  unsigned int a = float_to_ordered(lo), b = float_to_ordered(hi);
  a = __reduce_min_sync(0xffffffffu, a);
  b = __reduce_max_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], a);
    atomicMax(&mm[1], b);
  }
}

__global__ void to_bytes_kernel(const float* __restrict__ in, uint8_t* __restrict__ out,
                                int64_t n, const unsigned int* mm) {
  const float lo = ordered_to_float(mm[0]), hi = ordered_to_float(mm[1]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float s = __fmul_rn(255.0f, __fdiv_rn(__fsub_rn(in[i], lo), hi));
    // Out-of-range or NaN results (an all-zero grid divides by 0) give 0.
    const float r = rintf(s);
    out[i] = (r >= 0.0f && r <= 255.0f) ? (uint8_t)r : (uint8_t)0;
  }
}

__global__ void minmax_init_kernel(unsigned int* mm) {
  mm[0] = 0xffffffffu;
  mm[1] = 0u;
}

cageo_status launch_to_bytes(const float* in, uint8_t* out, int64_t n, unsigned int* mm,
                             cudaStream_t s) {
  minmax_init_kernel<<<1, 1, 0, s>>>(mm);
  minmax_kernel<<<1024, 256, 0, s>>>(in, n, mm);
  to_bytes_kernel<<<1024, 256, 0, s>>>(in, out, n, mm);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

}  // namespace cageo

using namespace cageo;

extern "C" cageo_status cageo_to_bytes(const float* d_in, uint8_t* d_out, int W, int H,
                                       cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_in && d_out && valid_dims(W, H), "pointers and size");
  Scratch ws;
  cageo_status st = ws.acquire(nullptr, 0, 2 * sizeof(unsigned int), stream);
  if (st) return st;
  return launch_to_bytes(d_in, d_out, (int64_t)W * H, (unsigned int*)ws.ptr, stream);
}

extern "C" cageo_status cageo_realistic_dem(const float* d_dem, float* d_field, int W, int H,
                                            float nodata_dem, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_dem && d_field && valid_dims(W, H), "pointers and size");
  return launch_realistic(d_dem, d_field, (int64_t)W * H, nodata_dem, stream);
}

extern "C" cageo_status cageo_stream_burn(float* d_dem, const float* d_streams, int W, int H,
                                          int bevel_radius, float nodata_dem,
                                          float nodata_stream, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_dem && d_streams && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(bevel_radius >= 1 && bevel_radius <= 5, "bevel radius must be 1..5");
  Scratch ws;
  size_t bytes = (size_t)W * H * sizeof(float);
  cageo_status st = ws.acquire(nullptr, 0, bytes, stream);
  if (st) return st;
  CAGEO_CUDA(cudaMemcpyAsync(ws.ptr, d_dem, bytes, cudaMemcpyDeviceToDevice, stream));
  return launch_burn_stage((const float*)ws.ptr, d_dem, d_streams, W, H, bevel_radius,
                           nodata_dem, nodata_stream, stream);
}
