// front.cuh -- the "front" of a realization: convolved noise -> realistic
// DEM -> stream burning -> pit-fill quantization, fused into the epilogue of
// the convolution kernels.  Shared by noise_conv.cu (kernels) and
// pipeline.cu (launch).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
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

struct FrontParams {
  const float* dem;        // W*H
  const uint8_t* code;     // W*H static codes
  float* q;                // W*H output: quantized burned realistic DEM
  unsigned int* min_ord;   // ordered-uint min of q (pit-fill minE)
  int* anomaly;            // set when the precomputed burn factor may not apply
  float nodata_dem;
  int quantize;            // 1: the CPU fill's 1 mm quantization; 0: raw (exact fill)
  float factor[kMaxBurnClasses + 1];  // factor[0] unused
};

// Writes one output of the fused front from the convolved value and the
// cell's DEM value and static code; returns q for the min reduction.
__device__ inline float front_epilogue(const FrontParams& p, int64_t i, float conv, float dem,
                                       uint8_t c) {
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
  return q;
}

}  // namespace cageo
