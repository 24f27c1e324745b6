// routing.cuh -- A7 flow routing and A8/A9 tracing and border internals,
// shared with pipeline.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "cageo.h"

namespace cageo {

struct RouteWork {
  int W = 0, H = 0;
  int tiles_x = 0, tiles_y = 0;
  uint8_t* tflat = nullptr;      // per 32x32 tile: holds a flat cell
  int* queued = nullptr;         // per tile: last pass it was queued for
  int* lists = nullptr;          // 2 * ntiles: tile worklists
  unsigned int* scal = nullptr;  // counters, barrier, error
  // Stacked realizations: H / slab_h grids of slab_h rows each, one above
  // the other; each slab's first and last rows are its border (0: one grid).
  // Only the steepest-descent pass needs it: flat cells are interior, so
  // their neighbours lie in their own slab.
  int slab_h = 0;
};
size_t route_workspace_bytes(int W, int H);
RouteWork route_carve(void* base, int W, int H);
// mode: CAGEO_ROUTE_CPU_COMPAT or CAGEO_ROUTE_GPU_ORDER (nodata is used by
// the latter only).
cageo_status route_run(const float* filled, int8_t* dir, int* flatdist,
                       const RouteWork& w, cudaStream_t s, int mode, float nodata);
// stats (7 entries, may be null): flat relaxation passes, flat cells,
// microseconds of the flat relaxation, flat tile visits, and kilo-cycles
// summed over visits spent staging, searching, storing.
cageo_status route_check_status(const RouteWork& w, int64_t* stats);

struct TraceWork {
  int W = 0, H = 0, tiles_x = 0, tiles_y = 0;
  int* state = nullptr;          // W*H: label, or the tile-border cell the path leaves by
  int* bstate = nullptr;         // 124 per 32x32 tile: the same for the tiles' border cells
  unsigned int* scal = nullptr;
};
size_t trace_workspace_bytes(int W, int H);
TraceWork trace_carve(void* base, int W, int H);
// is_stream(c) = streams[c] >= 0; the label of a stream terminal is
// (int)(-streams[c]).
// mode CAGEO_TRACE_DEAD_END_ERROR: cells whose path ends without an
// outlet are ERROR instead of taking cell 0's label.
// write_labels = false leaves the labels to border_u32_from_state.
cageo_status trace_run(const int8_t* dir, const float* streams, int* label,
                       const TraceWork& w, cudaStream_t s, int mode, bool write_labels);
cageo_status trace_check_status(const TraceWork& w, int64_t* jumps);

// count[i] += border(label) for float (stage API) or uint32 (pipeline) counts.
cageo_status border_float(const int* label, float* count, int W, int H,
                          cudaStream_t s);
cageo_status border_u32(const int* label, uint32_t* count, int W, int H,
                        cudaStream_t s);
// From the trace states of a trace_run without labels: writes the labels
// (mode as for tracing) and adds the border mask unless *gate is set.
cageo_status border_u32_from_state(const TraceWork& w, int* label, uint32_t* count,
                                   const int* gate, int mode, cudaStream_t s);
// The same, skipped entirely when *gate (device) is non-zero.
cageo_status border_u32_gated(const int* label, uint32_t* count, int W, int H,
                              const int* gate, cudaStream_t s);

}  // namespace cageo
