// pipeline.cu -- the Monte Carlo loop of src/main.cpp:180-283 as one object
// that owns its device buffers.
//
// A realization is: noise (Philox) -> fused convolution + realistic DEM +
// burning + quantization (front) -> pit fill -> routing -> tracing ->
// border counts.  In exact mode the front does not quantize and the fill,
// routing and tracing follow the reference's GPU path instead of its CPU
// path.  The launch sequence of one realization reads the
// realization number from device memory, so it is captured once in a CUDA
// graph and replayed; the data-dependent loops (fill passes, flat BFS
// layers, pointer jumps) run inside persistent kernels and need no host
// round trip.  Counts accumulate in uint32.
//
// The fused front uses a burn code precomputed from the stream raster.  It
// flags a realization where that code may differ from the reference's
// in-place burning (a stream cell whose realistic elevation equals NODATA);
// such a realization is not counted by the fast path and is recomputed with
// the stage kernels, which follow the reference step by step.  With a
// NODATA of 0 every realization takes the stage path.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include <unistd.h>
#include "common.cuh"
#include "guard.h"
#include "front.cuh"
#include "pitfill.cuh"
#include "routing.cuh"

namespace cageo {
cageo_status launch_noise(float* d, int64_t n, uint64_t seed, uint32_t realization,
                          const uint32_t* dreal, float mean, float sd, cudaStream_t s);
cageo_status launch_front(const float* noise, int W, int H, int model, const float* filt,
                          int r, const FrontParams& fp, cudaStream_t s, int tile);
bool conv_tile_applies(int model, int r, int tile);
cageo_status launch_burn_code(const float* streams, uint8_t* code, int W, int H,
                              float nodata_stream, int bevel, float* factor_out,
                              cudaStream_t s);
cageo_status launch_realistic(const float* dem, float* field, int64_t n, float nodata,
                              cudaStream_t s);
cageo_status launch_burn_stage(const float* src, float* dst, const float* streams, int W,
                               int H, int bevel, float nodata_dem, float nodata_stream,
                               cudaStream_t s);
cageo_status launch_to_bytes(const float* in, uint8_t* out, int64_t n, unsigned int* mm,
                             cudaStream_t s);
cageo_status ws_infer(const float* params, const float* v, float* warm, float* depth, int W,
                      int H, float nodata, float threshold, cudaStream_t s);

// End of a step of `count` realizations: record the realizations of a
// flagged step (none of them was counted), clear the flag and advance the
// device realization counter.
__global__ void realization_end_kernel(uint32_t* real, int* anomaly, uint32_t* redo,
                                       unsigned int* nredo, unsigned int count) {
  if (threadIdx.x == 0) {
    if (*anomaly) {
      const unsigned int k = atomicAdd(nredo, count);
      for (unsigned int j = 0; j < count && k + j < 4096; j++) redo[k + j] = *real + j;
      *anomaly = 0;
    }
    *real += count;
  }
}

// Order-independent 64-bit digest of a float grid: the wrapping sum over
// cells of a SplitMix64 finalizer of (cell index, value bits).  The
// checkpoint records it so that a resume onto other input grids is refused.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void grid_digest_kernel(const float* __restrict__ g, int64_t n,
                                   unsigned long long salt, unsigned long long* out) {
  unsigned long long h = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    h += mix64(((unsigned long long)i * 0x9E3779B97F4A7C15ull) ^
               ((unsigned long long)__float_as_uint(g[i]) << 32) ^ salt);
  for (int o = 16; o; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

__global__ void counts_to_float_kernel(const uint32_t* __restrict__ c, float* __restrict__ f,
                                       int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = (float)c[i];
}

}  // namespace cageo

using namespace cageo;

struct cageo_pipeline {
  cageo_pipeline_config cfg{};
  int W = 0, H = 0;
  int64_t N = 0;
  int radius = 0;
  cudaStream_t stream = nullptr;
  float *dem = nullptr, *streams = nullptr, *noise = nullptr, *q = nullptr, *filled = nullptr,
        *filter = nullptr, *tmp = nullptr;
  uint8_t* code = nullptr;
  int8_t* dir = nullptr;
  int *flatdist = nullptr, *label = nullptr;
  uint32_t* counts = nullptr;
  void *fill_ws = nullptr, *route_ws = nullptr, *trace_ws = nullptr;
  FillWork fw;
  RouteWork rw;
  TraceWork tw;
  // device scalars: [0] realization counter, [1] anomaly, [2] nredo, [3..] redo list
  uint32_t* dscal = nullptr;
  FrontParams fp{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_ok = false;
  int64_t stats[25] = {};
  // Learned warm start (exact mode only): parameters, warm surface, and the
  // fill's warm-start counters accumulated on the device (9 entries, see
  // fill_accumulate_warm_stats).
  float* ws_params = nullptr;
  float* warm = nullptr;
  unsigned long long* ws_acc = nullptr;
  float ws_threshold = 0.0f;
  // Digest of the DEM and stream grids (grid_digest_kernel), for checkpoints.
  unsigned long long input_digest = 0;
  // Batched steps (cageo_pipeline_set_batch): `batch` realizations share one
  // fill over a stack of their q grids (qb, filledb: batch * N floats, fill
  // workspace fwb for W x batch*H), each slab's minimum of q in slab_min.
  int batch = 1;
  int conv_tile = 0;  // the fused front's convolution tile shape (kConvTiles)
  float *qb = nullptr, *filledb = nullptr;
  void* fill_ws_b = nullptr;
  unsigned int* slab_min = nullptr;
  FillWork fwb;
  // Routing over the stack as well: directions and flat distances of all
  // slabs, routing workspace for W x batch*H.
  int8_t* dirb = nullptr;
  int* flatdistb = nullptr;
  void* route_ws_b = nullptr;
  RouteWork rwb;
  cudaGraph_t graph_b = nullptr;
  cudaGraphExec_t exec_b = nullptr;
  bool last_batched = false;  // the last realization ran in a batched step
};

namespace {

void free_batch(cageo_pipeline* p) {
  if (p->exec_b) cudaGraphExecDestroy(p->exec_b);
  if (p->graph_b) cudaGraphDestroy(p->graph_b);
  p->exec_b = nullptr;
  p->graph_b = nullptr;
  void* bufs[] = {p->qb, p->filledb, p->fill_ws_b, p->slab_min, p->dirb, p->flatdistb,
                  p->route_ws_b};
  for (void* b : bufs)
    if (b) cudaFree(b);
  p->qb = p->filledb = nullptr;
  p->fill_ws_b = nullptr;
  p->slab_min = nullptr;
  p->dirb = nullptr;
  p->flatdistb = nullptr;
  p->route_ws_b = nullptr;
  p->batch = 1;
}

void free_all(cageo_pipeline* p) {
  free_batch(p);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  void* bufs[] = {p->dem, p->streams, p->noise, p->q, p->filled, p->filter, p->tmp, p->code,
                  p->dir, p->flatdist, p->label, p->counts, p->fill_ws, p->route_ws,
                  p->trace_ws, p->dscal, p->ws_params, p->warm, p->ws_acc};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (p->stream) cudaStreamDestroy(p->stream);
}

bool exact_mode(const cageo_pipeline* p) { return p->cfg.fill_mode == CAGEO_FILL_EXACT; }

// Fill, routing and tracing of the current realization in the pipeline's
// mode; p->q holds the (quantized or raw) burned realistic DEM.
// With the learned warm start (exact mode), the network's warm surface is
// inferred from q first; the fill verifies and repairs it itself.
cageo_status enqueue_fill(cageo_pipeline* p) {
  if (!exact_mode(p)) return fill_run(p->q, p->filled, p->fw, p->cfg.nodata_dem, p->stream);
  if (!p->ws_params)
    return fill_run_exact(p->q, p->filled, p->fw, p->cfg.nodata_dem, nullptr, p->stream);
  cageo_status st = ws_infer(p->ws_params, p->q, p->warm, nullptr, p->W, p->H, p->cfg.nodata_dem,
                             p->ws_threshold, p->stream);
  if (st) return st;
  if ((st = fill_run_exact(p->q, p->filled, p->fw, p->cfg.nodata_dem, p->warm, p->stream)))
    return st;
  return fill_accumulate_warm_stats(p->fw, p->ws_acc, p->stream);
}

cageo_status enqueue_route(cageo_pipeline* p) {
  return route_run(p->filled, p->dir, p->flatdist, p->rw, p->stream,
                   exact_mode(p) ? CAGEO_ROUTE_GPU_ORDER : CAGEO_ROUTE_CPU_COMPAT,
                   p->cfg.nodata_dem);
}

int trace_mode(const cageo_pipeline* p) {
  return exact_mode(p) ? CAGEO_TRACE_DEAD_END_ERROR : CAGEO_TRACE_CPU_COMPAT;
}

// Tracing with labels (the learned path reads them before the border).
cageo_status enqueue_trace(cageo_pipeline* p) {
  return trace_run(p->dir, p->streams, p->label, p->tw, p->stream, trace_mode(p), true);
}

// Tracing whose labels are decoded by the border pass (one pass fewer);
// gate: skip the accumulation when set (null: always accumulate).
cageo_status enqueue_trace_border(cageo_pipeline* p, const int* gate) {
  cageo_status st = trace_run(p->dir, p->streams, p->label, p->tw, p->stream, trace_mode(p),
                              false);
  if (st) return st;
  return border_u32_from_state(p->tw, p->label, p->counts, gate,
                               trace_mode(p), p->stream);
}

// Launch sequence of one realization on the fast path.  The realization
// number is read from dscal[0] by the noise kernel.
cageo_status enqueue_fast(cageo_pipeline* p) {
  cudaStream_t s = p->stream;
  const cageo_pipeline_config& c = p->cfg;
  cageo_status st;
  if ((st = fill_reset_scalars(p->fw, s))) return st;
  if (p->fw.front_init && (st = fill_clear_seeds(p->fw, s))) return st;
  if ((st = launch_noise(p->noise, p->N, c.seed, 0, p->dscal, c.error_mean, c.error_stddev, s)))
    return st;
  if ((st = launch_front(p->noise, p->W, p->H, c.filter_model, p->filter, p->radius, p->fp, s,
                         p->conv_tile)))
    return st;
  if ((st = enqueue_fill(p))) return st;
  if ((st = enqueue_route(p))) return st;
  if ((st = enqueue_trace_border(p, (const int*)p->dscal + 1))) return st;
  realization_end_kernel<<<1, 32, 0, s>>>(p->dscal, (int*)p->dscal + 1, p->dscal + 3,
                                          p->dscal + 2, 1u);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

// Launch sequence of one batched step: `p->batch` realizations from the
// device counter on.  Noise and the fused front run per realization, each
// into its slab of the stacked q grid (with its own minimum); one fill
// covers the whole stack (slabs cannot exchange values: see FillWork), and
// so does the routing (flat cells are interior: their neighbours lie in
// their own slab); tracing and the border counts run per slab.  The results
// equal `batch` single realizations bit for bit.
cageo_status enqueue_batch(cageo_pipeline* p) {
  cudaStream_t s = p->stream;
  const cageo_pipeline_config& c = p->cfg;
  const int K = p->batch;
  cageo_status st;
  if ((st = fill_reset_scalars(p->fwb, s))) return st;
  if ((st = fill_clear_seeds(p->fwb, s))) return st;
  CAGEO_CUDA(cudaMemsetAsync(p->slab_min, 0xff, sizeof(unsigned int) * K, s));
  for (int k = 0; k < K; k++) {
    if ((st = launch_noise(p->noise, p->N, c.seed, (uint32_t)k, p->dscal, c.error_mean,
                           c.error_stddev, s)))
      return st;
    FrontParams fp = p->fp;
    fp.q = p->qb + (size_t)k * p->N;
    fp.min_ord = p->slab_min + k;
    fp.flags = p->fwb.flags + (size_t)k * p->N;
    fp.start = p->filledb + (size_t)k * p->N;
    fp.tseed = p->fwb.tseed;
    fp.tiles_x = p->fwb.tiles_x;
    fp.row0 = k * p->H;
    if ((st = launch_front(p->noise, p->W, p->H, c.filter_model, p->filter, p->radius, fp, s,
                           p->conv_tile)))
      return st;
  }
  if ((st = fill_run(p->qb, p->filledb, p->fwb, c.nodata_dem, s))) return st;
  if ((st = route_run(p->filledb, p->dirb, p->flatdistb, p->rwb, s, CAGEO_ROUTE_CPU_COMPAT,
                      c.nodata_dem)))
    return st;
  for (int k = 0; k < K; k++) {
    const int8_t* dir = p->dirb + 2 * (size_t)k * p->N;
    if ((st = trace_run(dir, p->streams, p->label, p->tw, s, CAGEO_TRACE_CPU_COMPAT, false)))
      return st;
    if ((st = border_u32_from_state(p->tw, p->label, p->counts, (const int*)p->dscal + 1,
                                    CAGEO_TRACE_CPU_COMPAT, s)))
      return st;
  }
  realization_end_kernel<<<1, 32, 0, s>>>(p->dscal, (int*)p->dscal + 1, p->dscal + 3,
                                          p->dscal + 2, (unsigned int)K);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

// Reference-order stage sequence for one realization (exact burning).
cageo_status run_stage_path(cageo_pipeline* p, uint32_t r) {
  cudaStream_t s = p->stream;
  const cageo_pipeline_config& c = p->cfg;
  cageo_status st;
  if ((st = fill_reset_scalars(p->fw, s))) return st;
  if ((st = launch_noise(p->noise, p->N, c.seed, r, nullptr, c.error_mean, c.error_stddev, s)))
    return st;
  if ((st = cageo_convolve(p->noise, p->tmp, p->W, p->H, c.filter_model, p->filter, p->radius, s)))
    return st;
  if ((st = launch_realistic(p->dem, p->tmp, p->N, c.nodata_dem, s))) return st;
  if ((st = launch_burn_stage(p->tmp, p->q, p->streams, p->W, p->H, c.bevel_radius, c.nodata_dem,
                              c.nodata_stream, s)))
    return st;
  if (!exact_mode(p) && (st = fill_quantize_min(p->q, p->fw, c.nodata_dem, s))) return st;
  // The stage kernels do not set up the fill: fill_run does it in full.
  const bool fused = p->fw.front_init;
  p->fw.front_init = false;
  st = enqueue_fill(p);
  p->fw.front_init = fused;
  if (st) return st;
  if ((st = enqueue_route(p))) return st;
  if ((st = enqueue_trace_border(p, nullptr))) return st;
  return CAGEO_OK;
}

// Largest filter radius a pipeline accepts (per-call filters included).
constexpr int kMaxRunRadius = 64;

template <typename T>
cageo_status dalloc(T** ptr, size_t bytes) {
  CAGEO_CUDA(cudaMalloc((void**)ptr, bytes ? bytes : 16));
  return CAGEO_OK;
}

cageo_status create_common(cageo_pipeline** out, const cageo_pipeline_config* cfg,
                           const float* dem, const float* streams, cudaMemcpyKind kind) {
  CAGEO_CHECK_ARG(out && cfg && dem && streams, "null argument");
  const int W = cfg->width, H = cfg->height;
  CAGEO_CHECK_ARG(valid_dims(W, H) && W >= 2 && H >= 2, "grid size");
  CAGEO_CHECK_ARG(W <= 65535 && H <= 65535, "width and height must be <= 65535");
  CAGEO_CHECK_ARG(cfg->filter_model == CAGEO_FILTER_GAUSSIAN ||
                      cfg->filter_model == CAGEO_FILTER_EXPONENTIAL,
                  "filter model");
  CAGEO_CHECK_ARG(cfg->bevel_radius >= 1 && cfg->bevel_radius <= 5, "bevel radius must be 1..5");
  CAGEO_CHECK_ARG(cfg->fill_mode == CAGEO_FILL_CPU_COMPAT || cfg->fill_mode == CAGEO_FILL_EXACT,
                  "fill mode");
  CAGEO_CHECK_ARG(cfg->cell_size > 0 && cfg->practical_range > 0, "range and cell size");
  const int r = cageo_filter_radius(cfg->practical_range, cfg->cell_size);
  CAGEO_CHECK_ARG(r >= 0 && r < W && r < H, "filter radius must be below the grid size");
  CAGEO_CHECK_ARG(r <= kMaxRunRadius, "filter radius above 64");
  const int L = 2 * r + 1;
  const int taps = cfg->filter_model == CAGEO_FILTER_GAUSSIAN ? L : L * L;
  std::vector<float> hf(taps);
  cageo_status st = cageo_filter_build(cfg->filter_model, cfg->practical_range, cfg->cell_size,
                                       r, hf.data());
  if (st) return st;
  auto* p = new (std::nothrow) cageo_pipeline();
  if (!p) {
    set_error("out of host memory for the pipeline object");
    return CAGEO_ERR_HOST;
  }
  p->cfg = *cfg;
  p->W = W;
  p->H = H;
  p->N = (int64_t)W * H;
  p->radius = r;
  auto fail = [&](cageo_status s) {
    free_all(p);
    delete p;
    return s;
  };
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(cuda_fail(cudaGetLastError(), "cudaStreamCreate"));
  const size_t fb = sizeof(float) * p->N;
  if ((st = dalloc(&p->dem, fb)) || (st = dalloc(&p->streams, fb)) ||
      (st = dalloc(&p->noise, fb)) || (st = dalloc(&p->q, fb)) || (st = dalloc(&p->filled, fb)) ||
      (st = dalloc(&p->tmp, fb)) ||
      (st = dalloc(&p->filter, sizeof(float) * (2 * kMaxRunRadius + 1) * (2 * kMaxRunRadius + 1))) ||
      (st = dalloc(&p->code, (size_t)p->N)) || (st = dalloc(&p->dir, 2 * (size_t)p->N)) ||
      (st = dalloc(&p->flatdist, 4 * (size_t)p->N)) || (st = dalloc(&p->label, 4 * (size_t)p->N)) ||
      (st = dalloc(&p->counts, 4 * (size_t)p->N)) ||
      (st = dalloc(&p->fill_ws, fill_workspace_bytes(W, H))) ||
      (st = dalloc(&p->route_ws, route_workspace_bytes(W, H))) ||
      (st = dalloc(&p->trace_ws, trace_workspace_bytes(W, H))) ||
      (st = dalloc(&p->dscal, sizeof(uint32_t) * (3 + 4096))))
    return fail(st);
  p->fw = fill_carve(p->fill_ws, W, H);
  p->rw = route_carve(p->route_ws, W, H);
  p->tw = trace_carve(p->trace_ws, W, H);
  cudaStream_t s = p->stream;
#define PCUDA(call)                                          \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return fail(cuda_fail(e_, #call)); \
  } while (0)
  PCUDA(cudaMemcpyAsync(p->filter, hf.data(), sizeof(float) * taps, cudaMemcpyHostToDevice, s));
  PCUDA(cudaMemcpyAsync(p->dem, dem, fb, kind, s));
  PCUDA(cudaMemcpyAsync(p->streams, streams, fb, kind, s));
  PCUDA(cudaMemsetAsync(p->counts, 0, 4 * (size_t)p->N, s));
  PCUDA(cudaMemsetAsync(p->dscal, 0, sizeof(uint32_t) * 3, s));
  {
    // dscal[4..5] holds the digest until the first realization.
    unsigned long long* dig = (unsigned long long*)(p->dscal + 4);
    PCUDA(cudaMemsetAsync(dig, 0, 8, s));
    grid_digest_kernel<<<1024, 256, 0, s>>>(p->dem, p->N, 0x44454dull, dig);
    grid_digest_kernel<<<1024, 256, 0, s>>>(p->streams, p->N, 0x535452ull << 20, dig);
    PCUDA(cudaGetLastError());
    PCUDA(cudaMemcpyAsync(&p->input_digest, dig, 8, cudaMemcpyDeviceToHost, s));
  }
  if ((st = launch_burn_code(p->streams, p->code, W, H, cfg->nodata_stream, cfg->bevel_radius,
                             p->fp.factor, s)))
    return fail(st);
  p->fp.dem = p->dem;
  p->fp.code = p->code;
  p->fp.q = p->q;
  p->fp.min_ord = fill_min_slot(p->fw);
  p->fp.anomaly = (int*)p->dscal + 1;
  p->fp.nodata_dem = cfg->nodata_dem;
  p->fp.quantize = cfg->fill_mode == CAGEO_FILL_EXACT ? 0 : 1;
  // The CPU-compatible fill's set-up runs in the front's epilogue.
  if (p->fp.quantize) {
    p->fp.flags = p->fw.flags;
    p->fp.start = p->filled;
    p->fp.tseed = p->fw.tseed;
    p->fp.tiles_x = p->fw.tiles_x;
    p->fp.row0 = 0;
    p->fp.W = W;
    p->fp.H = H;
    p->fw.front_init = true;
  }
  PCUDA(cudaStreamSynchronize(s));
#undef PCUDA
  *out = p;
  return CAGEO_OK;
}

}  // namespace

extern "C" cageo_status cageo_pipeline_create(cageo_pipeline** out,
                                              const cageo_pipeline_config* cfg,
                                              const float* h_dem, const float* h_streams) {
  return guarded("cageo_pipeline_create", [&] {
    return create_common(out, cfg, h_dem, h_streams, cudaMemcpyHostToDevice);
  });
}

extern "C" cageo_status cageo_pipeline_create_device(cageo_pipeline** out,
                                                     const cageo_pipeline_config* cfg,
                                                     const float* d_dem,
                                                     const float* d_streams) {
  return guarded("cageo_pipeline_create_device", [&] {
    return create_common(out, cfg, d_dem, d_streams, cudaMemcpyDeviceToDevice);
  });
}

static cageo_status pipeline_run(cageo_pipeline* p, uint32_t first, int count) {
  CAGEO_CHECK_ARG(p && count >= 0, "pipeline and count");
  cudaStream_t s = p->stream;
  cageo_status st;
  CAGEO_CUDA(cudaMemcpyAsync(p->dscal, &first, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  CAGEO_CUDA(cudaMemsetAsync(p->dscal + 1, 0, 2 * sizeof(uint32_t), s));
  const bool stage_only = p->cfg.nodata_dem == 0.0f;
  // Learned warm starts run on the fast path too (never batched).
  const bool learned = p->ws_params != nullptr && !stage_only;
  int done = 0;
  // Whole batched steps first (cageo_pipeline_set_batch), then single
  // realizations for the rest.  Both advance the same device counter.
  const int K = p->batch;
  const bool batched = !stage_only && !learned && K > 1 && count >= K;
  const int in_batches = batched ? count / K * K : 0;
  if (batched) {
    const int nb = count / K;
    int b = 0;
    if (p->cfg.use_graphs && !p->exec_b && !p->graph_b) {
      // Warm-up outside capture, then capture one batched step.
      if ((st = enqueue_batch(p))) return st;
      b = 1;
      CAGEO_CUDA(cudaStreamSynchronize(s));
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        cageo_status cst = enqueue_batch(p);
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (cst != CAGEO_OK || e != cudaSuccess ||
            cudaGraphInstantiate(&p->exec_b, g, 0) != cudaSuccess) {
          p->exec_b = nullptr;
        }
        cudaGetLastError();
      }
      // Kept even when the capture failed: it marks the capture as tried
      // (batched steps then run as direct launches).
      p->graph_b = g;
    }
    for (; b < nb; b++) {
      if (p->exec_b) CAGEO_CUDA(cudaGraphLaunch(p->exec_b, s));
      else if ((st = enqueue_batch(p))) return st;
    }
    done = nb * K;
  }
  if (!stage_only && count > done && p->cfg.use_graphs && !p->graph_ok && !p->exec) {
    // Warm-up outside capture (kernel attributes, occupancy caches), then
    // capture one realization.
    if ((st = enqueue_fast(p))) return st;
    done += 1;
    CAGEO_CUDA(cudaStreamSynchronize(s));
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      cageo_status cst = enqueue_fast(p);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(s, &g);
      if (cst == CAGEO_OK && e == cudaSuccess &&
          cudaGraphInstantiate(&p->exec, g, 0) == cudaSuccess) {
        p->graph = g;
        p->graph_ok = true;
      } else {
        if (g) cudaGraphDestroy(g);
        p->exec = nullptr;
      }
      cudaGetLastError();
    }
    // A failed capture leaves the flag off: the launches run directly.
    if (!p->graph_ok) p->cfg.use_graphs = 0;
  }
  for (int i = done; i < count; i++) {
    if (stage_only) {
      if ((st = run_stage_path(p, first + (uint32_t)i))) return st;
    } else if (p->graph_ok) {
      CAGEO_CUDA(cudaGraphLaunch(p->exec, s));
    } else {
      if ((st = enqueue_fast(p))) return st;
    }
  }
  CAGEO_CUDA(cudaStreamSynchronize(s));
  int64_t fs[kFillStats] = {}, rs[7] = {}, jumps = 0;
  p->last_batched = batched && in_batches == count;
  if (batched && (st = fill_check_status(p->fwb, p->last_batched ? fs : nullptr))) return st;
  if (batched && (st = route_check_status(p->rwb, p->last_batched ? rs : nullptr))) return st;
  if ((st = fill_check_status(p->fw, p->last_batched ? nullptr : fs))) return st;
  if ((st = route_check_status(p->rw, p->last_batched ? nullptr : rs))) return st;
  if ((st = trace_check_status(p->tw, &jumps))) return st;
  uint32_t nredo = 0;
  CAGEO_CUDA(cudaMemcpy(&nredo, p->dscal + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (nredo) {
    if (nredo > 4096) {
      set_error("more than 4096 realizations need the exact burning path in one run");
      return CAGEO_ERR_NO_CONVERGENCE;
    }
    std::vector<uint32_t> redo(nredo);
    CAGEO_CUDA(cudaMemcpy(redo.data(), p->dscal + 3, sizeof(uint32_t) * nredo,
                          cudaMemcpyDeviceToHost));
    for (uint32_t r : redo)
      if ((st = run_stage_path(p, r))) return st;
    CAGEO_CUDA(cudaStreamSynchronize(s));
    if ((st = fill_check_status(p->fw, fs))) return st;
  }
  p->stats[0] = fs[0];
  p->stats[1] = fs[1];
  p->stats[2] = rs[0];
  p->stats[3] = jumps;
  p->stats[4] = nredo;
  for (int k = 0; k < 9; k++) p->stats[5 + k] = fs[2 + k];
  p->stats[14] = rs[1];
  p->stats[15] = rs[2];
  for (int k = 0; k < 3; k++) p->stats[16 + k] = fs[11 + k];
  for (int k = 0; k < 4; k++) p->stats[19 + k] = rs[3 + k];
  p->stats[23] = fs[14];
  p->stats[24] = fs[15];
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_run(cageo_pipeline* p, uint32_t first, int count) {
  return guarded("cageo_pipeline_run", [&] { return pipeline_run(p, first, count); });
}

// One fast-path realization with CUDA events between the stages on the
// pipeline's stream (no graph).  It is a real realization: its border mask
// is accumulated like any other.  h_ms receives up to 6 stage times:
// noise, front (convolution+realistic+burn+quantize), fill, routing,
// tracing, border.
extern "C" cageo_status cageo_pipeline_profile(cageo_pipeline* p, uint32_t realization,
                                               float* h_ms, int n) {
  CAGEO_CHECK_ARG(p && h_ms, "null argument");
  CAGEO_CHECK_ARG(p->cfg.nodata_dem != 0.0f, "profiling needs the fused path (NODATA != 0)");
  cudaStream_t s = p->stream;
  const cageo_pipeline_config& c = p->cfg;
  cudaEvent_t ev[7], fm[4];
  for (auto& e : ev) CAGEO_CUDA(cudaEventCreate(&e));
  for (auto& e : fm) CAGEO_CUDA(cudaEventCreate(&e));
  cageo_status st = CAGEO_OK;
  do {
    if (cudaMemcpyAsync(p->dscal, &realization, 4, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      st = cuda_fail(cudaGetLastError(), "cudaMemcpyAsync");
      break;
    }
    if ((st = fill_reset_scalars(p->fw, s))) break;
    if (p->fw.front_init && (st = fill_clear_seeds(p->fw, s))) break;
    cudaEventRecord(ev[0], s);
    if ((st = launch_noise(p->noise, p->N, c.seed, 0, p->dscal, c.error_mean, c.error_stddev, s)))
      break;
    cudaEventRecord(ev[1], s);
    if ((st = launch_front(p->noise, p->W, p->H, c.filter_model, p->filter, p->radius, p->fp, s,
                           p->conv_tile)))
      break;
    cudaEventRecord(ev[2], s);
    if (!exact_mode(p)) p->fw.marks = fm;
    st = enqueue_fill(p);
    p->fw.marks = nullptr;
    if (st) break;
    cudaEventRecord(ev[3], s);
    if ((st = enqueue_route(p))) break;
    cudaEventRecord(ev[4], s);
    if ((st = trace_run(p->dir, p->streams, p->label, p->tw, s, trace_mode(p), false))) break;
    cudaEventRecord(ev[5], s);  // the border stage decodes the labels
    if ((st = border_u32_from_state(p->tw, p->label, p->counts,
                                    (const int*)p->dscal + 1, trace_mode(p), s)))
      break;
    realization_end_kernel<<<1, 32, 0, s>>>(p->dscal, (int*)p->dscal + 1, p->dscal + 3,
                                            p->dscal + 2, 1u);
    cudaEventRecord(ev[6], s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      st = cuda_fail(cudaGetLastError(), "cudaStreamSynchronize");
      break;
    }
    for (int i = 0; i < 6 && i < n; i++) cudaEventElapsedTime(&h_ms[i], ev[i], ev[i + 1]);
    // The fill's parts (CPU-compatible mode): set-up, flood A, flood B with
    // the undecided-cell kernels, confirmation phases, final pass.
    const cudaEvent_t fill_marks[6] = {ev[2], fm[0], fm[1], fm[2], fm[3], ev[3]};
    for (int i = 0; i < 5 && 6 + i < n; i++) {
      if (exact_mode(p)) h_ms[6 + i] = 0.0f;
      else cudaEventElapsedTime(&h_ms[6 + i], fill_marks[i], fill_marks[i + 1]);
    }
    int64_t fs[kFillStats], rs[7];
    if ((st = fill_check_status(p->fw, fs))) break;
    p->stats[0] = fs[0];
    p->stats[1] = fs[1];
    for (int k = 0; k < 9; k++) p->stats[5 + k] = fs[2 + k];
    if ((st = route_check_status(p->rw, rs))) break;
    p->stats[2] = rs[0];
    p->stats[14] = rs[1];
    p->stats[15] = rs[2];
    for (int k = 0; k < 3; k++) p->stats[16 + k] = fs[11 + k];
    for (int k = 0; k < 4; k++) p->stats[19 + k] = rs[3 + k];
    p->stats[23] = fs[14];
    p->stats[24] = fs[15];
    st = trace_check_status(p->tw, &p->stats[3]);
  } while (0);
  for (auto& e : ev) cudaEventDestroy(e);
  for (auto& e : fm) cudaEventDestroy(e);
  return st;
}

static cageo_status pipeline_run_filter(cageo_pipeline* p, uint32_t first, int count, int model,
                                        float practical_range, float error_mean,
                                        float error_stddev) {
  CAGEO_CHECK_ARG(p && count >= 0, "pipeline and count");
  CAGEO_CHECK_ARG(model == CAGEO_FILTER_GAUSSIAN || model == CAGEO_FILTER_EXPONENTIAL,
                  "filter model");
  CAGEO_CHECK_ARG(practical_range > 0, "practical range");
  const int r = cageo_filter_radius(practical_range, p->cfg.cell_size);
  CAGEO_CHECK_ARG(r >= 0 && r < p->W && r < p->H && r <= kMaxRunRadius,
                  "filter radius must be below the grid size and 64");
  const int L = 2 * r + 1, taps = model == CAGEO_FILTER_GAUSSIAN ? L : L * L;
  std::vector<float> hf(taps);
  cageo_status st = cageo_filter_build(model, practical_range, p->cfg.cell_size, r, hf.data());
  if (st) return st;
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  CAGEO_CUDA(cudaMemcpy(p->filter, hf.data(), sizeof(float) * taps, cudaMemcpyHostToDevice));
  p->cfg.filter_model = model;
  p->cfg.practical_range = practical_range;
  p->cfg.error_mean = error_mean;
  p->cfg.error_stddev = error_stddev;
  p->radius = r;
  // The captured graphs hold the old filter's launch shapes: drop them.
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->exec_b) cudaGraphExecDestroy(p->exec_b);
  if (p->graph_b) cudaGraphDestroy(p->graph_b);
  p->exec = nullptr;
  p->graph = nullptr;
  p->exec_b = nullptr;
  p->graph_b = nullptr;
  p->graph_ok = false;
  p->cfg.use_graphs = 0;
  return pipeline_run(p, first, count);
}

extern "C" cageo_status cageo_pipeline_run_filter(cageo_pipeline* p, uint32_t first, int count,
                                                  int model, float practical_range,
                                                  float error_mean, float error_stddev) {
  return guarded("cageo_pipeline_run_filter", [&] {
    return pipeline_run_filter(p, first, count, model, practical_range, error_mean,
                               error_stddev);
  });
}

// Checkpoint file (native byte order): the 8-byte magic "CAGEOCK2", a
// fixed header recording everything the counts depend on -- the grid size,
// the seed, the next realization number, the pipeline's filter and error
// model, bevel radius, fill mode, NODATA values and cell size, and a digest
// of the DEM and stream grids -- then W*H uint32 counts.  Loading refuses a
// checkpoint whose header differs from the pipeline in any of them, so a
// resume can only continue the same Monte Carlo run.
struct CheckpointHeader {
  char magic[8];
  int32_t width, height;
  uint64_t seed;
  uint32_t next_realization;
  int32_t filter_model;
  float practical_range, cell_size, error_mean, error_stddev;
  int32_t bevel_radius, fill_mode;
  float nodata_dem, nodata_stream;
  uint64_t input_digest;
};

static CheckpointHeader checkpoint_header(const cageo_pipeline* p, uint32_t next) {
  CheckpointHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, "CAGEOCK2", 8);
  h.width = p->W;
  h.height = p->H;
  h.seed = p->cfg.seed;
  h.next_realization = next;
  h.filter_model = p->cfg.filter_model;
  h.practical_range = p->cfg.practical_range;
  h.cell_size = p->cfg.cell_size;
  h.error_mean = p->cfg.error_mean;
  h.error_stddev = p->cfg.error_stddev;
  h.bevel_radius = p->cfg.bevel_radius;
  h.fill_mode = p->cfg.fill_mode;
  h.nodata_dem = p->cfg.nodata_dem;
  h.nodata_stream = p->cfg.nodata_stream;
  h.input_digest = p->input_digest;
  return h;
}

// The first header field that differs, or nullptr.  Floats compare by bits.
static const char* checkpoint_mismatch(const CheckpointHeader& a, const CheckpointHeader& b) {
  auto same = [](const void* x, const void* y, size_t n) { return std::memcmp(x, y, n) == 0; };
  if (a.width != b.width || a.height != b.height) return "grid size";
  if (a.seed != b.seed) return "seed";
  if (a.filter_model != b.filter_model) return "filter model";
  if (!same(&a.practical_range, &b.practical_range, 4)) return "practical range";
  if (!same(&a.cell_size, &b.cell_size, 4)) return "cell size";
  if (!same(&a.error_mean, &b.error_mean, 4)) return "error mean";
  if (!same(&a.error_stddev, &b.error_stddev, 4)) return "error standard deviation";
  if (a.bevel_radius != b.bevel_radius) return "bevel radius";
  if (a.fill_mode != b.fill_mode) return "fill mode";
  if (!same(&a.nodata_dem, &b.nodata_dem, 4) || !same(&a.nodata_stream, &b.nodata_stream, 4))
    return "NODATA values";
  if (a.input_digest != b.input_digest) return "DEM or stream grid";
  return nullptr;
}

// The file is written beside the target as "<path>.tmp", flushed to disk and
// renamed over the target, so a crash or kill during the write leaves the
// previous checkpoint intact.
static cageo_status pipeline_save(cageo_pipeline* p, const char* path,
                                  uint32_t next_realization) {
  CAGEO_CHECK_ARG(p && path, "null argument");
  std::vector<uint32_t> h((size_t)p->N);
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  CAGEO_CUDA(cudaMemcpy(h.data(), p->counts, 4 * (size_t)p->N, cudaMemcpyDeviceToHost));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) {
    set_error("unable to open \"%s\" for writing", tmp.c_str());
    return CAGEO_ERR_IO;
  }
  const CheckpointHeader hd = checkpoint_header(p, next_realization);
  bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
            std::fwrite(h.data(), 4, h.size(), f) == h.size();
  ok = ok && std::fflush(f) == 0 && fsync(fileno(f)) == 0;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    std::remove(tmp.c_str());
    set_error("short write to \"%s\"", tmp.c_str());
    return CAGEO_ERR_IO;
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    set_error("unable to replace \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_save(cageo_pipeline* p, const char* path,
                                            uint32_t next_realization) {
  return guarded("cageo_pipeline_save", [&] { return pipeline_save(p, path, next_realization); });
}

static cageo_status pipeline_load(cageo_pipeline* p, const char* path,
                                  uint32_t* next_realization) {
  CAGEO_CHECK_ARG(p && path && next_realization, "null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_error("unable to open checkpoint \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  CheckpointHeader hd;
  std::vector<uint32_t> h((size_t)p->N);
  bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, "CAGEOCK2", 8) == 0;
  if (ok) {
    const CheckpointHeader mine = checkpoint_header(p, hd.next_realization);
    if (const char* what = checkpoint_mismatch(hd, mine)) {
      std::fclose(f);
      set_error("checkpoint \"%s\" belongs to another run (its %s differs)", path, what);
      return CAGEO_ERR_FORMAT;
    }
  }
  ok = ok && std::fread(h.data(), 4, h.size(), f) == h.size() && std::fgetc(f) == EOF;
  std::fclose(f);
  if (!ok) {
    set_error("\"%s\" is not a complete checkpoint", path);
    return CAGEO_ERR_FORMAT;
  }
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  CAGEO_CUDA(cudaMemcpy(p->counts, h.data(), 4 * (size_t)p->N, cudaMemcpyHostToDevice));
  *next_realization = hd.next_realization;
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_load(cageo_pipeline* p, const char* path,
                                            uint32_t* next_realization) {
  return guarded("cageo_pipeline_load", [&] { return pipeline_load(p, path, next_realization); });
}

extern "C" cageo_status cageo_pipeline_counts_device(cageo_pipeline* p, float* d_out) {
  CAGEO_CHECK_ARG(p && d_out, "null argument");
  counts_to_float_kernel<<<(unsigned)((p->N + 255) / 256), 256, 0, p->stream>>>(p->counts, d_out,
                                                                                 p->N);
  CAGEO_CUDA(cudaGetLastError());
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_counts(cageo_pipeline* p, float* h_out) {
  CAGEO_CHECK_ARG(p && h_out, "null argument");
  counts_to_float_kernel<<<(unsigned)((p->N + 255) / 256), 256, 0, p->stream>>>(p->counts, p->tmp,
                                                                                 p->N);
  CAGEO_CUDA(cudaGetLastError());
  CAGEO_CUDA(cudaMemcpyAsync(h_out, p->tmp, sizeof(float) * p->N, cudaMemcpyDeviceToHost,
                             p->stream));
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_counts_bytes(cageo_pipeline* p, uint8_t* h_out) {
  CAGEO_CHECK_ARG(p && h_out, "null argument");
  cudaStream_t s = p->stream;
  counts_to_float_kernel<<<(unsigned)((p->N + 255) / 256), 256, 0, s>>>(p->counts, p->tmp, p->N);
  CAGEO_CUDA(cudaGetLastError());
  // The byte image is staged in the noise buffer and the min/max pair in the
  // flat-distance grid; both are rewritten by the next realization.
  uint8_t* bytes = (uint8_t*)p->noise;
  unsigned int* mm = (unsigned int*)p->flatdist;
  cageo_status st = launch_to_bytes(p->tmp, bytes, p->N, mm, s);
  if (st) return st;
  CAGEO_CUDA(cudaMemcpyAsync(h_out, bytes, (size_t)p->N, cudaMemcpyDeviceToHost, s));
  CAGEO_CUDA(cudaStreamSynchronize(s));
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_last_stages(cageo_pipeline* p, float* h_filled,
                                                   int8_t* h_dir, int* h_label) {
  CAGEO_CHECK_ARG(p, "null pipeline");
  cudaStream_t s = p->stream;
  // After a batched step the last realization's filled grid is its top slab.
  const float* filled = p->last_batched ? p->filledb + (size_t)(p->batch - 1) * p->N : p->filled;
  if (h_filled)
    CAGEO_CUDA(cudaMemcpyAsync(h_filled, filled, 4 * p->N, cudaMemcpyDeviceToHost, s));
  const int8_t* dir = p->last_batched ? p->dirb + 2 * (size_t)(p->batch - 1) * p->N : p->dir;
  if (h_dir) CAGEO_CUDA(cudaMemcpyAsync(h_dir, dir, 2 * p->N, cudaMemcpyDeviceToHost, s));
  if (h_label) CAGEO_CUDA(cudaMemcpyAsync(h_label, p->label, 4 * p->N, cudaMemcpyDeviceToHost, s));
  CAGEO_CUDA(cudaStreamSynchronize(s));
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_reset_counts(cageo_pipeline* p) {
  CAGEO_CHECK_ARG(p, "null pipeline");
  CAGEO_CUDA(cudaMemsetAsync(p->counts, 0, 4 * (size_t)p->N, p->stream));
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  return CAGEO_OK;
}

// Candidate settings of the autotuner: sweep rounds per fill tile visit x
// warps per SM of the fill's lower-bound flood (with the first convolution
// tile), then the other convolution tiles with the fill setting chosen
// among those (fill fields 0).  The front and the fill are separate stages,
// so tuning them one after the other finds the best of the product.
static const int kTuneRounds[3] = {16, 32, 64};
static const int kTuneWarps[3] = {16, 20, 22};
constexpr int kTuneFill = 9;
constexpr int kTuneCandidates = kTuneFill + kConvTiles - 1;

extern "C" int cageo_autotune_candidates(cageo_tuning* h_out, int n) {
  for (int k = 0; h_out && k < n && k < kTuneCandidates; k++) {
    if (k < kTuneFill) {
      h_out[k] = cageo_tuning{kTuneRounds[k % 3], kTuneWarps[k / 3], 0};
    } else {
      h_out[k] = cageo_tuning{0, 0, k - kTuneFill + 1};
    }
  }
  return kTuneCandidates;
}

static void drop_graph(cageo_pipeline* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->exec_b) cudaGraphExecDestroy(p->exec_b);
  if (p->graph_b) cudaGraphDestroy(p->graph_b);
  p->exec = nullptr;
  p->graph = nullptr;
  p->exec_b = nullptr;
  p->graph_b = nullptr;
  p->graph_ok = false;
}

// The batched fill runs with the single fill's tuning.
static void sync_batch_tuning(cageo_pipeline* p) {
  p->fwb.max_rounds = p->fw.max_rounds;
  p->fwb.flood_warps = p->fw.flood_warps;
}

extern "C" cageo_status cageo_pipeline_set_tuning(cageo_pipeline* p, const cageo_tuning* t) {
  CAGEO_CHECK_ARG(p && t, "null argument");
  CAGEO_CHECK_ARG(t->fill_rounds >= 1 && t->fill_rounds <= 1024, "fill rounds must be 1..1024");
  CAGEO_CHECK_ARG(fill_flood_warps_valid(t->fill_warps), "fill warps must be 16, 20 or 22");
  CAGEO_CHECK_ARG(t->conv_tile >= 0 && t->conv_tile < kConvTiles,
                  "convolution tile must be 0..3");
  CAGEO_CHECK_ARG(conv_tile_applies(p->cfg.filter_model, p->radius, t->conv_tile),
                  "the convolution tile does not fit this filter radius in shared memory");
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  p->fw.max_rounds = t->fill_rounds;
  p->fw.flood_warps = t->fill_warps;
  p->conv_tile = t->conv_tile;
  sync_batch_tuning(p);
  drop_graph(p);  // captured with the old launch shapes
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_get_tuning(cageo_pipeline* p, cageo_tuning* t) {
  CAGEO_CHECK_ARG(p && t, "null argument");
  t->fill_rounds = p->fw.max_rounds;
  t->fill_warps = p->fw.flood_warps;
  t->conv_tile = p->conv_tile;
  return CAGEO_OK;
}

// Autotuning: each candidate runs one warm-up and `trials` realizations on
// the fast path (direct launches, timed with events on the pipeline's
// stream); the fastest is kept and the CUDA graph is captured again on the
// next run.  The counts are reset to zero afterwards.
extern "C" cageo_status cageo_pipeline_autotune(cageo_pipeline* p, uint32_t first, int trials,
                                                cageo_tuning* h_best, float* h_ms, int n_ms) {
  CAGEO_CHECK_ARG(p && trials >= 1, "pipeline and trials");
  CAGEO_CHECK_ARG(p->cfg.nodata_dem != 0.0f && !p->ws_params,
                  "autotuning times the fused path (NODATA != 0, no warm start)");
  cudaStream_t s = p->stream;
  cudaEvent_t e0, e1;
  CAGEO_CUDA(cudaEventCreate(&e0));
  CAGEO_CUDA(cudaEventCreate(&e1));
  cageo_status st = CAGEO_OK;
  float best_ms = 0.0f;
  cageo_tuning best{p->fw.max_rounds, p->fw.flood_warps, p->conv_tile};
  cageo_tuning cand[kTuneCandidates];
  cageo_autotune_candidates(cand, kTuneCandidates);
  for (int c = 0; c < kTuneCandidates && st == CAGEO_OK; c++) {
    if (c < kTuneFill) {
      p->fw.max_rounds = cand[c].fill_rounds;
      p->fw.flood_warps = cand[c].fill_warps;
    } else {
      // Another convolution tile with the fill setting chosen above; a tile
      // that does not apply (exponential filters use the 2D kernel) or does
      // not fit the radius is skipped (0 ms).
      cand[c].fill_rounds = best.fill_rounds;
      cand[c].fill_warps = best.fill_warps;
      if (!conv_tile_applies(p->cfg.filter_model, p->radius, cand[c].conv_tile)) {
        if (h_ms && c < n_ms) h_ms[c] = 0.0f;
        continue;
      }
      p->fw.max_rounds = best.fill_rounds;
      p->fw.flood_warps = best.fill_warps;
    }
    p->conv_tile = cand[c].conv_tile;
    uint32_t r0 = first + (uint32_t)(c * (trials + 1));
    if (cudaMemcpyAsync(p->dscal, &r0, sizeof(r0), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      st = cuda_fail(cudaGetLastError(), "cudaMemcpyAsync");
      break;
    }
    if ((st = enqueue_fast(p))) break;  // warm-up
    cudaEventRecord(e0, s);
    for (int k = 0; k < trials && st == CAGEO_OK; k++) st = enqueue_fast(p);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      st = cuda_fail(cudaGetLastError(), "cudaEventSynchronize");
      break;
    }
    if (st == CAGEO_OK) st = fill_check_status(p->fw, nullptr);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)trials;
    if (h_ms && c < n_ms) h_ms[c] = ms;
    if (c == 0 || ms < best_ms) {
      best_ms = ms;
      best = cand[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  p->fw.max_rounds = best.fill_rounds;
  p->fw.flood_warps = best.fill_warps;
  p->conv_tile = best.conv_tile;
  sync_batch_tuning(p);
  drop_graph(p);
  if (h_best) *h_best = best;
  CAGEO_CUDA(cudaMemsetAsync(p->counts, 0, 4 * (size_t)p->N, s));
  CAGEO_CUDA(cudaMemsetAsync(p->dscal + 1, 0, 2 * sizeof(uint32_t), s));
  CAGEO_CUDA(cudaStreamSynchronize(s));
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_set_batch(cageo_pipeline* p, int batch) {
  CAGEO_CHECK_ARG(p, "null pipeline");
  CAGEO_CHECK_ARG(batch >= 1 && batch <= 64, "batch must be 1..64 realizations");
  if (batch > 1) {
    CAGEO_CHECK_ARG(p->cfg.fill_mode == CAGEO_FILL_CPU_COMPAT,
                    "batched steps need the CPU-compatible fill mode");
    CAGEO_CHECK_ARG((int64_t)batch * p->N < kMaxCells, "batch * grid cells must stay below 2^31");
  }
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  free_batch(p);
  p->last_batched = false;
  if (batch == 1) return CAGEO_OK;
  const size_t nb = (size_t)batch * p->N;
  cageo_status st;
  if ((st = dalloc(&p->qb, sizeof(float) * nb)) || (st = dalloc(&p->filledb, sizeof(float) * nb)) ||
      (st = dalloc(&p->fill_ws_b, fill_workspace_bytes(p->W, batch * p->H))) ||
      (st = dalloc(&p->slab_min, sizeof(unsigned int) * 64)) ||
      (st = dalloc(&p->dirb, 2 * nb)) || (st = dalloc(&p->flatdistb, sizeof(int) * nb)) ||
      (st = dalloc(&p->route_ws_b, route_workspace_bytes(p->W, batch * p->H)))) {
    free_batch(p);
    return st;
  }
  p->rwb = route_carve(p->route_ws_b, p->W, batch * p->H);
  p->rwb.slab_h = p->H;
  p->fwb = fill_carve(p->fill_ws_b, p->W, batch * p->H);
  p->fwb.slab_h = p->H;
  p->fwb.slab_min = p->slab_min;
  p->fwb.front_init = true;
  sync_batch_tuning(p);
  p->batch = batch;
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_set_warmstart(cageo_pipeline* p, const float* h_params,
                                                     int n, float threshold) {
  CAGEO_CHECK_ARG(p, "null pipeline");
  CAGEO_CUDA(cudaStreamSynchronize(p->stream));
  drop_graph(p);  // the captured step holds the old fill
  if (!h_params) {
    if (p->ws_params) cudaFree(p->ws_params);
    p->ws_params = nullptr;
    return CAGEO_OK;
  }
  CAGEO_CHECK_ARG(p->cfg.fill_mode == CAGEO_FILL_EXACT,
                  "the learned warm start needs the exact fill mode");
  CAGEO_CHECK_ARG(n == cageo_ws_param_count(), "parameter count");
  if (!p->ws_params) CAGEO_CUDA(cudaMalloc((void**)&p->ws_params, sizeof(float) * n));
  if (!p->warm) CAGEO_CUDA(cudaMalloc((void**)&p->warm, sizeof(float) * p->N));
  if (!p->ws_acc) CAGEO_CUDA(cudaMalloc((void**)&p->ws_acc, sizeof(unsigned long long) * 9));
  CAGEO_CUDA(cudaMemcpy(p->ws_params, h_params, sizeof(float) * n, cudaMemcpyHostToDevice));
  CAGEO_CUDA(cudaMemset(p->ws_acc, 0, sizeof(unsigned long long) * 9));
  p->ws_threshold = threshold;
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_warmstart_stats(cageo_pipeline* p, int64_t* h_stats,
                                                       int n) {
  CAGEO_CHECK_ARG(p && h_stats, "null argument");
  unsigned long long acc[9] = {};
  if (p->ws_acc) {
    CAGEO_CUDA(cudaStreamSynchronize(p->stream));
    CAGEO_CUDA(cudaMemcpy(acc, p->ws_acc, sizeof(acc), cudaMemcpyDeviceToHost));
  }
  for (int i = 0; i < n && i < 9; i++) h_stats[i] = (int64_t)acc[i];
  return CAGEO_OK;
}

extern "C" cageo_status cageo_pipeline_graph_kernels(cageo_pipeline* p, int64_t* h_count) {
  CAGEO_CHECK_ARG(p && h_count, "null argument");
  // The batched step's graph when batching is on and it was captured.
  cudaGraph_t g = (p->batch > 1 && p->exec_b) ? p->graph_b : (p->graph_ok ? p->graph : nullptr);
  CAGEO_CHECK_ARG(g, "no step has been captured in a CUDA graph");
  size_t n = 0;
  CAGEO_CUDA(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  CAGEO_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
  int64_t kernels = 0;
  for (size_t i = 0; i < n; i++) {
    cudaGraphNodeType t;
    CAGEO_CUDA(cudaGraphNodeGetType(nodes[i], &t));
    kernels += t == cudaGraphNodeTypeKernel;
  }
  *h_count = kernels;
  return CAGEO_OK;
}

extern "C" cudaStream_t cageo_pipeline_stream(cageo_pipeline* p) { return p ? p->stream : nullptr; }

extern "C" cageo_status cageo_pipeline_stats(cageo_pipeline* p, int64_t* h_stats, int n) {
  CAGEO_CHECK_ARG(p && h_stats, "null argument");
  for (int i = 0; i < n && i < 25; i++) h_stats[i] = p->stats[i];
  return CAGEO_OK;
}

extern "C" void cageo_pipeline_destroy(cageo_pipeline* p) {
  if (!p) return;
  cudaStreamSynchronize(p->stream);
  free_all(p);
  delete p;
}
