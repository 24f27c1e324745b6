// pitfill.cuh -- CPU-path-compatible pit filling on the GPU (shared with
// pipeline.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "cageo.h"

namespace cageo {

// Workspace of one fill: per-cell flags, per-tile worklists, counters and
// the candidate list of the confirmation phases.
struct FillWork {
  int W = 0, H = 0;
  int tiles_x = 0, tiles_y = 0;
  uint8_t* flags = nullptr;      // W*H
  int* queued = nullptr;         // ntiles: tile state in the work queue (idle, queued, processing, re-queued, done)
  int* lists = nullptr;          // 2 * ntiles: tile worklists (double buffer)
  uint8_t* tseed = nullptr;      // ntiles: tile holds a relaying outlet
  uint8_t* tconv = nullptr;      // ntiles: tile converged on its last visit
  uint32_t* cand = nullptr;      // W*H: list of undecided cells of the phases
  uint32_t* aux = nullptr;       // W*H: flood A's result, then component labels
  uint32_t* cmin = nullptr;      // W*H: per-component phase minima (at roots)
  unsigned int* scal = nullptr;  // scalar block (see pitfill.cu)
  int max_rounds = 64;           // sweep rounds per tile visit before the tile re-queues itself
  int flood_warps = 20;          // warps per block (per SM) of flood A: 16, 20 or 22
  // Stacked realizations (CPU-compatible fill only): the grid holds
  // H / slab_h realizations of slab_h rows each, one above the other.
  // Every slab's first and last rows are its border (outlets), so no flood
  // value crosses from one slab to another: a cell that is not on a border
  // has all 8 neighbours in its own slab, and border cells never change.
  // slab_min holds each slab's ordered minimum of q (the passability test's
  // minE).  slab_h = 0: one realization, minimum in the scalar block.
  int slab_h = 0;
  const unsigned int* slab_min = nullptr;
  // The fused front has set up the flags, the start values and the tile
  // seeds (with minE = 0; fill_clear_seeds must run before it): fill_run
  // only redoes the set-up of the slabs whose minimum of q is not 0.
  bool front_init = false;
  // Profiling only: when set, fill_run records marks[0] after the set-up,
  // [1] after flood A, [2] after flood B's main drain and the undecided-cell
  // kernels, [3] after the confirmation phases.
  const cudaEvent_t* marks = nullptr;
};

// Whether `warps` is a block size flood A is built for.
bool fill_flood_warps_valid(int warps);

size_t fill_workspace_bytes(int W, int H);
FillWork fill_carve(void* base, int W, int H);

// Fill q (already quantized, min already in scal) into `filled`.  Runs on
// `s`; does not synchronize.  Errors found on the device are reported by
// fill_check_status after the stream has drained.
cageo_status fill_run(const float* q, float* filled, const FillWork& w,
                      float nodata, cudaStream_t s);
// Exact float fill of v (the reference's GPU path): no quantization, no
// minimum needed.  `warm` (may be null): per-cell start values.  The fill
// verifies a warm start itself: after the warm flood, cells whose level no
// chain of relays from an outlet supports restart from +inf and a repair
// flood visits their tiles, so the result is the exact fill for any start.
cageo_status fill_run_exact(const float* v, float* filled, const FillWork& w, float nodata,
                            const float* warm, cudaStream_t s);
// Quantize d in place (the reference's step (i)) and reduce its minimum
// into the scalar block.
cageo_status fill_quantize_min(float* d, const FillWork& w, float nodata,
                               cudaStream_t s);
// Clears the tile seeds before a fused front sets them (FillWork::front_init).
cageo_status fill_clear_seeds(const FillWork& w, cudaStream_t s);
// Launch-time setup of the scalar block and the ordered minimum of q.
cageo_status fill_reset_scalars(const FillWork& w, cudaStream_t s);
unsigned int* fill_min_slot(const FillWork& w);
// Copies the device status (0 ok) and stats into host memory; the stream
// must have been synchronized.  stats (kFillStats entries): last pass
// number, phases, passes of flood A, passes of flood B before the first
// phase, microseconds of flood A, of flood B to convergence, of the phase
// loop, tiles and sweep rounds of flood A, tiles and rounds of flood B,
// kilo-cycles summed over tile visits spent staging, sweeping, storing, and
// kilo-cycles warps of flood A and of flood B spent waiting for a tile,
// and the cells a warm-started exact fill restarted from +inf.
constexpr int kFillStats = 17;
cageo_status fill_check_status(const FillWork& w, int64_t* stats);
// Adds the last warm-started exact fill's counters to acc (9 device
// uint64: fills, fills that restarted cells, cells restarted, warm-flood
// tile visits and sweep rounds, repair sweep rounds, warm and repair
// microseconds, repair tile visits).  Stream-ordered, no synchronization.
cageo_status fill_accumulate_warm_stats(const FillWork& w, unsigned long long* acc,
                                        cudaStream_t s);

}  // namespace cageo
