// front.cuh -- the "front" of a realization: convolved noise -> realistic
// DEM -> stream burning -> pit-fill quantization, fused into the epilogue of
// the convolution kernels.  Shared by noise_conv.cu (kernels) and
// pipeline.cu (launch).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "fillflags.cuh"
#include "stage_math.cuh"

namespace cageo {

// Per-cell static code computed once per pipeline from the stream raster:
//   bits 0-4: index (1..) into the burn-factor table of the nearest stream
//             within the bevel radius, 0 = none;
//   bit 6   : tracing stream   (streams >= 0, FlowTracingAlgorithmCPUOpenMP.h:58)
//   bit 7   : burning stream   (streams != NODATA, StreamBurningAlgorithmCPUOpenMP.h:51)
constexpr uint8_t kCodeTraceStream = 0x40;
constexpr uint8_t kCodeBurnStream = 0x80;
constexpr int kMaxBurnClasses = 31;

// Tile shapes of the fused front's separable convolution (output columns x
// rows per block), chosen per pipeline by its autotuner; the outputs never
// depend on the shape.
constexpr int kConvTiles = 4;

struct FrontParams {
  const float* dem;        // W*H
  const uint8_t* code;     // W*H static codes
  float* q;                // W*H output: quantized burned realistic DEM
  unsigned int* min_ord;   // ordered-uint min of q (pit-fill minE)
  int* anomaly;            // set when the precomputed burn factor may not apply
  float nodata_dem;
  int quantize;            // 1: the CPU fill's 1 mm quantization; 0: raw (exact fill)
  // The pit fill's set-up, fused (CPU-compatible mode; flags null: not
  // fused): each cell's flags and start value, and the seed mark of a tile
  // holding a relaying outlet, computed with minE = 0.  That is the minimum
  // whenever a stream cell is burned to 0; the fill checks the real minimum
  // of each realization and redoes the set-up where it differs.
  uint8_t* flags;          // W*H fill flags
  float* start;            // W*H fill start values (the filled grid)
  uint8_t* tseed;          // fill tile seeds (of the whole, possibly stacked, grid)
  int tiles_x;             // fill tiles per row
  int row0;                // this grid's first row in the stacked grid
  int W, H;                // this grid's size (its border)
  float factor[kMaxBurnClasses + 1];  // factor[0] unused
};

// Writes one output of the fused front (cell i at column x, row y) from the
// convolved value and the cell's DEM value and static code; returns q for
// the min reduction.
__device__ inline float front_epilogue(const FrontParams& p, int64_t i, int x, int y, float conv,
                                       float dem, uint8_t c) {
  float v = realistic_value(dem, conv, p.nodata_dem);
  if (c & kCodeBurnStream) {
    // The reference tests a stream neighbour's elevation against NODATA;
    // the precomputed factors assume that test passes.
    if (v == p.nodata_dem) atomicExch(p.anomaly, 1);
    v = 0.0f;
  }
  int k = c & 0x1f;
  if (k) v = __fmul_rn(v, p.factor[k]);
  float q = p.quantize ? fill_quantize(v, p.nodata_dem) : v;
  p.q[i] = q;
  if (p.flags) {
    const uint8_t f =
        fill_init_flags(q, p.nodata_dem, 0.0f, x == 0 || y == 0 || x == p.W - 1 || y == p.H - 1);
    p.flags[i] = f;
    p.start[i] = (f & (FNODATA | FOUTLET)) ? q : __builtin_huge_valf();
    if ((f & (FOUTLET | FNONPASS)) == FOUTLET) p.tseed[((p.row0 + y) >> 5) * p.tiles_x + (x >> 5)] = 1;
  }
  return q;
}

}  // namespace cageo
