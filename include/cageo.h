/* cageo.h -- C ABI of the GB300 (sm_103a) Monte Carlo drainage-basin pipeline.
 *
 * Drop-in for the per-realization stage algorithms of the drainage program
 * (jsoksane/cageo).  Each stage entry point replaces one reference
 * interface, cited beside it.  The semantics are those of the reference's
 * CPU path (`drainage --cpu`), which these kernels reproduce bit-for-bit on
 * the same inputs.
 *
 * Conventions
 *  - Grids are row-major, index y*W + x, no padding (the reference's
 *    CellGrid layout, src/framework/CellGrid.h:491-500).
 *  - Every grid pointer named d_* is a caller-owned DEVICE pointer on the
 *    current CUDA device; h_* pointers are host memory.
 *  - Every call is asynchronous on `stream` (0 = the legacy default stream)
 *    unless it says otherwise.  Calls return a cageo_status; on failure
 *    cageo_last_error_string() describes the error.  Nothing calls exit().
 *  - Flow directions are 2 signed bytes per cell (dx, dy), the reference's
 *    char2 FlowDirDataType (src/flowrouting/FlowDirClass.h:44).
 *  - Basin labels are int32: -(int)streams[terminal stream cell],
 *    CAGEO_OUTSIDE or CAGEO_LAKE (src/flowtracing/FlowTracingCommon.h:18-21).
 *  - Stages that need scratch memory take (d_workspace, workspace_bytes);
 *    query the size with the matching *_workspace_size().  A workspace must
 *    start on a 256-byte boundary (CAGEO_ERR_ARGUMENT otherwise).  Passing
 *    NULL lets the call allocate and free it stream-ordered (cudaMallocAsync).
 *  - Threads: stage calls keep no state between calls (launch set-up is
 *    cached per device, safely), so host threads may call them at once on
 *    different buffers and streams.  A pipeline object is used by one host
 *    thread at a time; separate pipelines may run on separate threads, as
 *    the batched workload does.  cageo_pitfill_static shares one scratch
 *    array among all callers and must be serialized by them.
 */
#ifndef CAGEO_H_
#define CAGEO_H_

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int cageo_status;
#define CAGEO_OK 0
#define CAGEO_ERR_ARGUMENT 1   /* a size, pointer or option is invalid */
#define CAGEO_ERR_CUDA 2       /* a CUDA runtime call failed */
#define CAGEO_ERR_NO_CONVERGENCE 3 /* an iterative stage hit its iteration or wait limit */
#define CAGEO_ERR_IO 4         /* a raster or header file could not be read or written */
#define CAGEO_ERR_FORMAT 5     /* a header tag or value is not understood */
#define CAGEO_ERR_HOST 6       /* host memory could not be allocated (no C++ exception
                                  leaves the library) */

/* Filter models, src/convolution/ConvolutionCommon.h:21-24. */
#define CAGEO_FILTER_EXPONENTIAL 0
#define CAGEO_FILTER_GAUSSIAN 1

/* Basin label codes, src/flowtracing/FlowTracingCommon.h:18-21. */
#define CAGEO_OUTSIDE (-9999)
#define CAGEO_LAKE (-9998)
#define CAGEO_ERROR (-9996)

/* Pit-filling modes.  CPU_COMPAT reproduces the reference CPU path
 * (src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:68-242).  EXACT is the
 * reference GPU path's exact float fill
 * (src/pitfilling/PitFillingAlgorithmGPUCUDA.cu:201-381): no quantization;
 * border cells and cells equal to 0 are outlets; every other cell ends at
 * the least, over paths from an outlet through non-NODATA cells, of the
 * largest elevation on the path; cells no path reaches end at 99990000. */
#define CAGEO_FILL_CPU_COMPAT 0
#define CAGEO_FILL_EXACT 1

/* Routing modes: the CPU path's flat rules, or the GPU path's
 * (src/flowrouting/FlowRoutingAlgorithmGPUCUDAOriginal.cu:200-271,391-437:
 * NODATA skipped, streams are first-layer outlets, first match in
 * N, W, E, S, NW, NE, SW, SE order). */
#define CAGEO_ROUTE_CPU_COMPAT 0
#define CAGEO_ROUTE_GPU_ORDER 1

/* Tracing modes: cells whose path ends without an outlet take cell 0's
 * label (CPU path), or are CAGEO_ERROR (used with the GPU semantics). */
#define CAGEO_TRACE_CPU_COMPAT 0
#define CAGEO_TRACE_DEAD_END_ERROR 1

const char* cageo_version(void);
/* Text of the last error raised on the calling host thread. */
const char* cageo_last_error_string(void);

/* ---- A1 random field ----------------------------------------------------
 * Replaces RandomFieldAlgorithm<T>::execute(field, seed)
 * (src/randomfield/RandomFieldAlgorithm.h:82-93; CPU
 * src/randomfield/RandomFieldAlgorithmCPUOpenMP.h:47-76).
 * d_field[i] = mean + stddev * N(0,1), where the normal deviates come from
 * Philox4x32-10 (key = seed, counter = (cell/4, realization)) and the
 * Box-Muller transform.  Deterministic for a given (seed, realization). */
cageo_status cageo_noise_philox(float* d_field, int W, int H, uint64_t seed,
                                uint32_t realization, float mean, float stddev,
                                cudaStream_t stream);

/* The generator behind cageo_noise_philox, exposed so that it can be
 * checked against the published Philox4x32-10 known-answer vectors (Salmon
 * et al., SC'11; the Random123 distribution).  No counterpart in the
 * reference (whose CPU path draws from thrust's default engine and its GPU
 * path from cuRAND, src/randomfield/RandomFieldAlgorithmCPUOpenMP.h:56-74).
 * d_out receives n blocks of 4 words; block i is Philox4x32-10 of the
 * counter (h_ctr[0] + i mod 2^32, h_ctr[1], h_ctr[2], h_ctr[3]) under the key
 * (h_key[0], h_key[1]).  0 < n < 2^31. */
cageo_status cageo_philox4x32_10(uint32_t* d_out, int64_t n, const uint32_t* h_ctr,
                                 const uint32_t* h_key, cudaStream_t stream);

/* ---- A2 filter ----------------------------------------------------------
 * Radius used by the driver: ceil(range/cell*2.5) (src/main.cpp:110). */
int cageo_filter_radius(float practical_range, float cell_size);
/* Replaces ConvolutionAlgorithm::createFilter(range, cell)
 * (src/convolution/ConvolutionAlgorithm.cpp:18-172), host FP64:
 * correlogram -> 2D DFT -> sqrt|F| -> inverse DFT / n^2 -> fftshift; the
 * Gaussian model keeps the rank-1 factor u0*sqrt(s0).  h_filter receives
 * 2r+1 taps (Gaussian) or (2r+1)^2 row-major taps (exponential).
 * Synchronous, host only. */
cageo_status cageo_filter_build(int model, float practical_range,
                                float cell_size, int radius, float* h_filter);

/* ---- A3 convolution -----------------------------------------------------
 * Replaces ConvolutionAlgorithm::execute -> performConvolution
 * (src/convolution/ConvolutionAlgorithm.h:124-140; CPU
 * src/convolution/ConvolutionAlgorithmCPUOpenMP.h:70-248).  Periodic wrap;
 * Gaussian = column pass then row pass; ascending tap order, unfused
 * multiply and add, so results equal the CPU path bit-for-bit.
 * d_filter holds the taps on the device.  d_in != d_out.  Needs r < W, r < H. */
cageo_status cageo_convolve(const float* d_in, float* d_out, int W, int H,
                            int model, const float* d_filter, int radius,
                            cudaStream_t stream);

/* ---- A4 realistic DEM ---------------------------------------------------
 * Replaces RealisticDemAlgorithm::execute(dem, rand, rDem) with rDem
 * aliasing rand (src/realisticdem/RealisticDemAlgorithm.h:49-70,
 * src/main.cpp:200-204): d_field = dem + field where dem != nodata_dem, then
 * values <= 0 that are not nodata_dem become 1.0.  In place on d_field. */
cageo_status cageo_realistic_dem(const float* d_dem, float* d_field, int W,
                                 int H, float nodata_dem, cudaStream_t stream);

/* ---- A5 stream burning --------------------------------------------------
 * Replaces StreamBurningAlgorithm::execute(rDem, streams)
 * (src/streamburning/StreamBurningAlgorithm.h:116-134; CPU
 * src/streamburning/StreamBurningAlgorithmCPUOpenMP.h:32-82).  In place on
 * d_dem; bevel radius 1..5 (MAX_BEVEL_RADIUS). */
cageo_status cageo_stream_burn(float* d_dem, const float* d_streams, int W,
                               int H, int bevel_radius, float nodata_dem,
                               float nodata_stream, cudaStream_t stream);

/* ---- A6 pit filling -----------------------------------------------------
 * Replaces PitFillingAlgorithm::execute(filled, rDem)
 * (src/pitfilling/PitFillingAlgorithm.h:88-98; CPU
 * src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:68-242; GPU
 * src/pitfilling/PitFillingAlgorithmGPUCUDA.cu:201-381).  In CPU_COMPAT
 * mode, like the reference, d_dem is quantized to 1/1000 m in place; in
 * EXACT mode it is left unchanged.  d_filled receives the filled surface.
 * W, H <= 65535 (the reference's Cell coordinates). */
size_t cageo_pitfill_workspace_size(int W, int H);
cageo_status cageo_pitfill(float* d_dem, float* d_filled, int W, int H,
                           float nodata_dem, int mode, void* d_workspace,
                           size_t workspace_bytes, cudaStream_t stream);

/* Exact fill (CAGEO_FILL_EXACT semantics) relaxed down from per-cell start
 * values d_warm (NULL: +inf, the plain fill) instead of +inf.  No
 * counterpart in the reference: it is the building block of the learned
 * warm start.  The fill verifies the start itself: after the warm-started
 * flood, a cell's level counts only if a chain of relaying cells from an
 * outlet supports it (no step above the level); every other cell (started
 * too low, pulled down by one that was, or unreached) restarts from +inf and
 * a repair flood visits the tiles holding them.  The result is the exact
 * fill for any start.  h_stats (may be NULL) receives the fill's 17
 * statistics (passes, tiles, sweep rounds ..., [16] cells restarted). */
cageo_status cageo_pitfill_exact_warm(const float* d_dem, const float* d_warm,
                                      float* d_filled, int W, int H,
                                      float nodata_dem, void* d_workspace,
                                      size_t workspace_bytes, int64_t* h_stats,
                                      cudaStream_t stream);

/* Pit filling that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that cannot allocate -- e.g. a host
 * application that has reserved the GPU's memory for its own allocator and
 * forbids plug-ins from calling cudaMalloc, or a loop that must not pay an
 * allocation's latency or implicit synchronization.  Same semantics and
 * result as cageo_pitfill; its scratch is a fixed array inside the library
 * (cageo_pitfill_static_max_bytes(), 64 MiB, held on every GPU that loads
 * the library until the process exits), enough for grids up to 2048 x 2048
 * cells; larger grids are refused with CAGEO_ERR_ARGUMENT.  The first call
 * on a device looks up the array's device address (make that first call
 * before any stream capture).  All calls share the array: each call clears
 * what must start at zero, and calls that overlap on the GPU race, so the
 * caller must serialize them.  Synchronizes `stream` before returning. */
size_t cageo_pitfill_static_max_bytes(void);
cageo_status cageo_pitfill_static(float* d_dem, float* d_filled, int W, int H,
                                  float nodata_dem, int mode, cudaStream_t stream);

/* ---- A7 flow routing ----------------------------------------------------
 * Replaces FlowRoutingAlgorithm::execute(flowDir, filled)
 * (src/flowrouting/FlowRoutingAlgorithm.h:69-94; CPU
 * src/flowrouting/FlowRoutingAlgorithmCPUOpenMP.h:53-249): D8 steepest
 * descent, border cells point outward, flat cells by layered BFS.
 * d_dir: 2*W*H int8 (dx,dy).  d_flatdist (optional, may be NULL): the
 * reference's flat-distance grid (-1 has a direction, -2 stream, k >= 1
 * flat layer, 0 unresolved). */
size_t cageo_route_workspace_size(int W, int H);
cageo_status cageo_route_d8(const float* d_filled, int8_t* d_dir,
                            int* d_flatdist, int W, int H, void* d_workspace,
                            size_t workspace_bytes, cudaStream_t stream);
/* Same with a routing mode (CAGEO_ROUTE_*); CAGEO_ROUTE_GPU_ORDER replaces
 * the reference's FlowRoutingAlgorithm_GPU_CUDA_Original::performFlowRouting
 * + performFlowRoutingOnFlatSurfaces and also writes flatDist -3 on NODATA
 * cells.  nodata_dem is used by the GPU order only. */
cageo_status cageo_route_d8_mode(const float* d_filled, int8_t* d_dir,
                                 int* d_flatdist, int W, int H, float nodata_dem,
                                 int mode, void* d_workspace,
                                 size_t workspace_bytes, cudaStream_t stream);

/* ---- A8 flow tracing ----------------------------------------------------
 * Replaces FlowTracingAlgorithm::execute(trace, flowDir, streams)
 * (src/flowtracing/FlowTracingAlgorithm.h:52-69; CPU
 * src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:34-134), by pointer
 * jumping.  d_label: W*H int32. */
size_t cageo_trace_workspace_size(int W, int H);
cageo_status cageo_trace(const int8_t* d_dir, const float* d_streams,
                         int* d_label, int W, int H, void* d_workspace,
                         size_t workspace_bytes, cudaStream_t stream);
/* Same with a tracing mode (CAGEO_TRACE_*). */
cageo_status cageo_trace_mode(const int8_t* d_dir, const float* d_streams,
                              int* d_label, int W, int H, int mode,
                              void* d_workspace, size_t workspace_bytes,
                              cudaStream_t stream);

/* ---- A9 catchment border ------------------------------------------------
 * Replaces CatchmentBorderAlgorithm::execute(mc, trace)
 * (src/catchmentborder/CatchmentBorderAlgorithm.h:53-74; CPU
 * src/catchmentborder/CatchmentBorderAlgorithmCPUOpenMP.h:30-82):
 * d_count += border mask (float counts, like the reference's grid). */
cageo_status cageo_border_accumulate(const int* d_label, float* d_count, int W,
                                     int H, cudaStream_t stream);

/* ---- Learned warm start of the exact fill ------------------------------------
 * No counterpart in the reference.  A convolutional network (features of 4
 * channels -> 3x3 conv, 32 channels, ReLU -> 3x3 conv, 32 channels, ReLU ->
 * 3x3 conv, 1 channel) predicts the depth the exact fill gives each cell;
 * cells predicted dry start cageo_pitfill_exact_warm at their elevation.
 * Weights are rounded to bf16 where they are used, sums accumulate in fp32.
 * Parameters: cageo_ws_param_count() floats, laid out W1[32][4][9], b1[32],
 * W2[32][32][9], b2[32], W3[1][32][9], b3[1] (tap t = (dy+1)*3 + dx+1).
 * Grids of a batch are stored one after another, channels planar:
 * [batch][channel][H][W]. */
int cageo_ws_param_count(void);
/* Features of B grids d_v [B][H][W] into d_feat [B][4][H][W]: v minus the
 * 3x3 minimum, v minus the 7x7 minimum, the 7x7 maximum minus v, v minus the
 * 7x7 mean (over in-grid, non-NODATA cells; NODATA cells get zeros). */
cageo_status cageo_ws_features(const float* d_v, float* d_feat, int W, int H, int B,
                               float nodata_dem, cudaStream_t stream);
/* Training forward pass (fp32 activations): d_a1, d_a2 [B][32][H][W] keep
 * the hidden layers for the backward pass, d_out [B][H][W]. */
cageo_status cageo_ws_forward(const float* d_params, const float* d_feat, int W, int H,
                              int B, float* d_a1, float* d_a2, float* d_out,
                              cudaStream_t stream);
/* Backward pass: adds the gradient of the loss (given d_dout = dL/d out)
 * with respect to every parameter into d_grad.  d_tmp1, d_tmp2:
 * [B][32][H][W] scratch; d_wflip: 9216 floats of scratch. */
cageo_status cageo_ws_backward(const float* d_params, const float* d_feat, const float* d_a1,
                               const float* d_a2, const float* d_dout, int W, int H, int B,
                               float* d_grad, float* d_tmp1, float* d_tmp2, float* d_wflip,
                               cudaStream_t stream);
/* Mean squared error over the cells at least `margin` cells inside each
 * grid: writes dL/dy into d_dy and adds the loss into *d_loss. */
cageo_status cageo_ws_mse(const float* d_y, const float* d_target, float* d_dy, float* d_loss,
                          int W, int H, int B, int margin, cudaStream_t stream);
/* One Adam step (bias-corrected, `step` counts from 1). */
cageo_status cageo_ws_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, int n,
                           float lr, float beta1, float beta2, float eps, int step,
                           cudaStream_t stream);
/* Inference on one grid d_v [H][W] (burned realistic elevations, not
 * quantized): d_depth (may be NULL) receives the predicted depths, d_warm
 * (may be NULL) the warm start: v where the depth is below `threshold`,
 * +inf elsewhere.  Hidden activations are bf16 here (fp32 in training). */
cageo_status cageo_ws_infer(const float* d_params, const float* d_v, float* d_warm,
                            float* d_depth, int W, int H, float nodata_dem, float threshold,
                            cudaStream_t stream);

/* ---- Pipeline: the whole Monte Carlo loop of src/main.cpp:180-283 -------
 * Owns its device buffers; runs realizations [first, first+count) with
 * noise Philox(seed, realization) and accumulates the border counts
 * internally (uint32).  The per-realization stage sequence runs as fused
 * kernels; outputs are bit-identical to calling the stage functions above
 * in the reference order. */
typedef struct cageo_pipeline cageo_pipeline;
typedef struct {
  int width, height;
  float cell_size;
  int filter_model;        /* CAGEO_FILTER_* */
  float practical_range;
  float error_mean, error_stddev;
  int bevel_radius;        /* reference default 2 */
  float nodata_dem, nodata_stream;
  uint64_t seed;
  int use_graphs;          /* capture the per-realization launches in a CUDA graph */
  int fill_mode;           /* CAGEO_FILL_CPU_COMPAT: the CPU path throughout;
                              CAGEO_FILL_EXACT: the GPU path's semantics (exact
                              fill, GPU routing order, dead ends ERROR) */
} cageo_pipeline_config;

/* h_dem, h_streams: host grids (W*H floats).  The filter is built with
 * cageo_filter_build().  Synchronous. */
cageo_status cageo_pipeline_create(cageo_pipeline** out,
                                   const cageo_pipeline_config* cfg,
                                   const float* h_dem, const float* h_streams);
/* Same, from device grids (copied). */
cageo_status cageo_pipeline_create_device(cageo_pipeline** out,
                                          const cageo_pipeline_config* cfg,
                                          const float* d_dem,
                                          const float* d_streams);
cageo_status cageo_pipeline_run(cageo_pipeline* p, uint32_t first_realization,
                                int count);
/* Same with another filter and error model from now on (rebuilt on the
 * host; radius <= 64): for batches whose realizations draw their practical
 * range and error standard deviation.  Runs without a CUDA graph. */
cageo_status cageo_pipeline_run_filter(cageo_pipeline* p, uint32_t first_realization,
                                       int count, int model, float practical_range,
                                       float error_mean, float error_stddev);
/* Batched steps (no counterpart in the reference, whose Monte Carlo loop
 * runs one realization after another, src/main.cpp:180-283): with batch > 1
 * cageo_pipeline_run processes realizations `batch` at a time.  Their noise
 * and fused front run one after another into the slabs of a stacked grid,
 * one pit fill covers the whole stack (the slabs' borders are outlets, so no
 * value crosses between them), so does the routing (flat cells are interior
 * to their slab), and tracing and the border counts run per realization; a
 * batched step is captured in a CUDA graph of its own.
 * The counts and every stage output equal single realizations bit for bit;
 * batching only shares the persistent launches of the fill and the flat
 * BFS (their grid barriers and idle tails) among the realizations of a step.  A run
 * of `count` realizations takes count / batch batched steps and the rest
 * singly.  1 <= batch <= 64, batch * cells < 2^31, CPU-compatible fill
 * mode only.  Allocates the stacked grids and the fill and routing
 * workspaces for them (about 27 bytes per cell per realization); batch = 1
 * frees them. */
cageo_status cageo_pipeline_set_batch(cageo_pipeline* p, int batch);
/* Border counts so far as float (the reference's CatchmentBorderType). */
cageo_status cageo_pipeline_counts(cageo_pipeline* p, float* h_out);
cageo_status cageo_pipeline_counts_device(cageo_pipeline* p, float* d_out);
/* Border counts as the reference's JPEG byte image (cageo_to_bytes), host. */
cageo_status cageo_pipeline_counts_bytes(cageo_pipeline* p, uint8_t* h_out);
/* Stage outputs of the most recent realization (any pointer may be NULL):
 * filled surface (float), dir (2 int8 per cell), labels (int32).  Host. */
cageo_status cageo_pipeline_last_stages(cageo_pipeline* p, float* h_filled,
                                        int8_t* h_dir, int* h_label);
cageo_status cageo_pipeline_reset_counts(cageo_pipeline* p);
/* Checkpoint / resume of a long Monte Carlo run (no counterpart in the
 * reference, whose only persistence is the per-frame output,
 * src/main.cpp:250-256): the count grid, the next realization number and
 * every setting the counts depend on (grid size, seed, filter model,
 * practical range, cell size, error mean and standard deviation, bevel
 * radius, fill mode, NODATA values) plus a digest of the DEM and stream
 * grids.  Loading refuses (CAGEO_ERR_FORMAT) a checkpoint that differs in
 * any of them, or that is truncated.  Saving writes "<path>.tmp" and
 * renames it over `path`, so an interrupted save leaves the previous
 * checkpoint intact. */
cageo_status cageo_pipeline_save(cageo_pipeline* p, const char* path,
                                 uint32_t next_realization);
cageo_status cageo_pipeline_load(cageo_pipeline* p, const char* path,
                                 uint32_t* next_realization);
cudaStream_t cageo_pipeline_stream(cageo_pipeline* p);
/* Kernel launches in the CUDA graph that one step replays (the graph's
 * kernel nodes; memset nodes are not counted): the batched step's graph when
 * batching is on and captured, else the single realization's.
 * CAGEO_ERR_ARGUMENT until a run has captured one.  No counterpart in the
 * reference. */
cageo_status cageo_pipeline_graph_kernels(cageo_pipeline* p, int64_t* h_count);
/* One realization with CUDA events between stages (fused path, no graph);
 * it is accumulated like any other.  h_ms[0..5]: noise, front
 * (convolution + realistic DEM + burning + quantization), pit fill,
 * routing, tracing, border (milliseconds); with n >= 11, h_ms[6..10]: the
 * pit fill's parts -- set-up, lower-bound flood, walled flood with the
 * undecided-cell kernels, confirmation phases, final pass (0 in exact
 * mode). */
cageo_status cageo_pipeline_profile(cageo_pipeline* p, uint32_t realization,
                                    float* h_ms, int n);
/* Counters of the last run: [0] fill work-queue drains, [1] confirmation
 * phases, [2] flat-BFS passes, [3] trace jumps, [4] burn re-runs, [5] drains
 * of the lower-bound flood, [6] drains of the walled flood before the first
 * phase, [7..9] microseconds of the lower-bound flood, of the walled flood
 * to convergence and of the phase loop, [10..13] tiles and sweep rounds of
 * the two floods, [14] flat cells, [15] microseconds of the flat BFS,
 * [16..18] kilo-cycles summed over the fill's tile visits spent staging,
 * sweeping and storing, [19] tile visits of the flat BFS, [20..22]
 * kilo-cycles summed over them spent staging, searching and storing,
 * [23..24] kilo-cycles the warps of the fill's lower-bound flood and of its
 * walled flood spent waiting for a tile, end of the queue included (last
 * realization). */
cageo_status cageo_pipeline_stats(cageo_pipeline* p, int64_t* h_stats, int n);
/* Tuning of the pipeline's kernels (no counterpart in the reference).  The
 * results never depend on it.  fill_rounds: sweep rounds a fill tile visit
 * may run before the tile queues itself again (1..1024; default 64).
 * fill_warps: warps per SM of the fill's lower-bound flood (16, 20 or 22;
 * more warps hide more latency, fewer leave more registers to each; default
 * 20).  The fill's tile shape is fixed at 32 x 32 cells, the warp width: a
 * warp owns a tile and holds its rows as 32-bit lane masks.  conv_tile:
 * output tile of the fused front's separable (Gaussian) convolution per
 * block, 0 = 64 x 32 (default), 1 = 128 x 32, 2 = 64 x 64, 3 = 96 x 32
 * (columns x rows); only 0 applies to exponential filters, and a tile whose
 * staged block does not fit shared memory for the radius is refused. */
typedef struct {
  int fill_rounds;
  int fill_warps;
  int conv_tile;
} cageo_tuning;
/* The autotuner's candidates: writes up to n of them to h_out (may be NULL)
 * and returns how many there are: the fill settings (with conv_tile 0),
 * then the other convolution tiles, whose fill fields are 0 (they run with
 * the fill setting chosen among the first ones). */
int cageo_autotune_candidates(cageo_tuning* h_out, int n);
cageo_status cageo_pipeline_set_tuning(cageo_pipeline* p, const cageo_tuning* t);
cageo_status cageo_pipeline_get_tuning(cageo_pipeline* p, cageo_tuning* t);
/* Autotuner: runs each candidate setting for one warm-up and `trials`
 * realizations from `first_realization` on, timed with CUDA events on the
 * pipeline's stream, and keeps the fastest.  h_best (may be NULL) receives
 * the choice, h_ms (may be NULL) up to n_ms milliseconds per realization,
 * one per candidate in cageo_autotune_candidates() order (0 for a
 * convolution tile that does not apply).  Resets the counts to zero. */
cageo_status cageo_pipeline_autotune(cageo_pipeline* p, uint32_t first_realization,
                                     int trials, cageo_tuning* h_best, float* h_ms,
                                     int n_ms);
/* Learned warm start for an exact-mode pipeline (no counterpart in the
 * reference): each realization infers a warm surface from its burned
 * realistic DEM (cells predicted shallower than `threshold` metres start at
 * their elevation, the rest at +inf) and fills from it with
 * cageo_pitfill_exact_warm's verification and repair, all on the device (the
 * step is captured in a CUDA graph like a plain one); the counts equal the
 * plain exact fill's.  h_params: cageo_ws_param_count() floats, or NULL to
 * switch the warm start off. */
cageo_status cageo_pipeline_set_warmstart(cageo_pipeline* p, const float* h_params, int n,
                                          float threshold);
/* Counters since set_warmstart: [0] warm-started realizations, [1] of them
 * with cells restarted from +inf, [2] cells restarted, [3] tile visits and
 * [4] sweep rounds of the warm-started floods, [5] sweep rounds of the
 * repair floods, [6] microseconds of the warm floods, [7] of the repairs,
 * [8] tile visits of the repairs.  Synchronizes the pipeline's stream. */
cageo_status cageo_pipeline_warmstart_stats(cageo_pipeline* p, int64_t* h_stats, int n);
void cageo_pipeline_destroy(cageo_pipeline* p);

/* ---- A10 raster I/O -----------------------------------------------------
 * Header: ESRI-style tags ncols nrows xllcorner yllcorner cellsize
 * NODATA_value byteorder (src/utils/utils.cpp:58-112); an unknown tag is an
 * error.  Rasters: raw native-endian float32 (src/utils/SystemUtils.h:53-86);
 * the read fails unless the file holds exactly `count` floats. */
typedef struct {
  int ncols, nrows;
  double xllcorner, yllcorner;
  float cellsize;
  float nodata_value;
  int byteorder_msb;  /* 1 for MSBFIRST; the reference parses but ignores it */
} cageo_raster_info;
/* Byte image for the JPEG output: (uint8)rintf(255*((v-min)/max)) with the
 * grid's min and max, replacing ToByteArrayAlgorithm::execute
 * (src/utils/tobytearray/ToByteArrayAlgorithmCPUOpenMP.h:33-52).  A grid
 * whose max is 0 gives 0 everywhere. */
cageo_status cageo_to_bytes(const float* d_in, uint8_t* d_out, int W, int H,
                            cudaStream_t stream);
/* JPEG file of a byte image, byte-identical to what the reference's jpge
 * encoder writes for it with its default parameters and the given quality
 * (src/main.cpp:265-270 passes jpge::params(): quality 85, YCbCr H2V2 with
 * neutral chroma, standard tables).  Quality 1..100.  Host only. */
cageo_status cageo_write_jpeg(const char* path, const uint8_t* h_gray, int W, int H,
                              int quality);
cageo_status cageo_read_header(const char* path, cageo_raster_info* info);
cageo_status cageo_write_header(const char* path, const cageo_raster_info* info);
cageo_status cageo_read_raster(const char* path, float* h_out, size_t count);
cageo_status cageo_write_raster(const char* path, const float* h_data,
                                size_t count);

#ifdef __cplusplus
}
#endif
#endif /* CAGEO_H_ */
