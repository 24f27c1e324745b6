// stage_math.cuh -- per-cell arithmetic shared by the kernels (and by host
// code where noted).  Every float operation that the reference's CPU path
// performs is written with an explicit round-to-nearest intrinsic so nvcc
// never fuses a multiply and an add: results equal the reference's
// (unfused, x86-64) float arithmetic bit for bit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cageo {

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
// as easy as 1, 2, 3", SC'11).  Ten rounds of two 32x32->64 multiplies with
// the published multipliers and Weyl key increments.
struct U4 { uint32_t x, y, z, w; };

__host__ __device__ inline void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi,
                                          uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

__host__ __device__ inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, c.x, &hi0, &lo0);
    mulhilo32(M1, c.z, &hi1, &lo1);
    U4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// 24-bit uniform in (0, 1): never 0, so the logarithm below stays finite
// (the reference redraws -inf deviates, RandomFieldAlgorithmCPUOpenMP.h:66-71).
__device__ inline float u01_open(uint32_t x) {
  return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Counter tag distinguishing the noise stream from any other Philox use.
constexpr uint32_t kNoiseTag = 0x63616765u;

// ---- pit-filling quantization, src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:56-66
// toIndex(v, minE) = (size_t)(1000 * (v - minE)), float arithmetic; a
// non-positive product gives 0 (the reference's conversion of a negative
// float is undefined; 0 is what aarch64 produces).
__host__ __device__ inline uint32_t fill_to_index(float v, float minE) {
#ifdef __CUDA_ARCH__
  float p = __fmul_rn(1000.0f, __fsub_rn(v, minE));
  if (!(p > 0.0f)) return 0u;
  if (p >= 4294967040.0f) return 0xffffffffu;
  return __float2uint_rz(p);
#else
  volatile float d = v - minE;
  volatile float p = 1000.0f * d;
  if (!(p > 0.0f)) return 0u;
  if (p >= 4294967040.0f) return 0xffffffffu;
  return (uint32_t)p;
#endif
}

// toElev(z, minE) = ((float)z)/1000 + minE.
__host__ __device__ inline float fill_to_elev(uint32_t z, float minE) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(__fdiv_rn(__uint2float_rn(z), 1000.0f), minE);
#else
  volatile float a = (float)z / 1000.0f;
  return a + minE;
#endif
}

// A popped cell expands its neighbours only when its value survives the
// index round trip (PitFillingAlgorithmCPUOpenMP.h:178).
__host__ __device__ inline bool fill_passable(float v, float minE) {
  return fill_to_elev(fill_to_index(v, minE), minE) == v;
}

// Step (i) of the CPU fill: 1 mm truncation that never maps a nonzero
// elevation to 0 (PitFillingAlgorithmCPUOpenMP.h:84-106).
__host__ __device__ inline float fill_quantize(float e, float nodata) {
  if (e == nodata) return e;
  uint32_t qi = fill_to_index(e, 0.0f);
  if (e != 0.0f && qi == 0u) qi = 1u;
  return fill_to_elev(qi, 0.0f);
}

// ---- realistic DEM, src/utils/addsurfaces/AddSurfacesAlgorithmCPUOpenMP.h:50-55
// and RemoveNegativeElevationsAlgorithmCPUOpenMP.h:42-46.
__device__ inline float realistic_value(float dem, float field, float nodata) {
  float v = (dem != nodata) ? __fadd_rn(dem, field) : field;
  if (v <= 0.0f && v != nodata) v = 1.0f;
  return v;
}

// ---- D8 neighbour order N, NE, E, SE, S, SW, W, NW
// (src/flowrouting/FlowRoutingAlgorithmCPUOpenMP.h:105-114).
__host__ __device__ constexpr int d8_dx(int n) {
  return n == 1 || n == 2 || n == 3 ? 1 : (n == 5 || n == 6 || n == 7 ? -1 : 0);
}
__host__ __device__ constexpr int d8_dy(int n) {
  return n == 0 || n == 1 || n == 7 ? -1 : (n == 3 || n == 4 || n == 5 ? 1 : 0);
}

// Basin labels and flat-distance codes.
constexpr int kOutside = -9999;
constexpr int kLake = -9998;
constexpr int kError = -9996;

}  // namespace cageo
