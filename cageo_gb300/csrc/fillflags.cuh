// fillflags.cuh -- the pit fill's per-cell flags and their set-up, shared by
// the fill (pitfill.cu) and the fused front, which sets them up as it writes
// the quantized grid.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "stage_math.cuh"

namespace cageo {

// Per-cell flag bits.  FCLEAN (flood A with clean marks): the cell's level
// is reached by a path of passable relays from an outlet, so flood B, whose
// walls are non-passable cells only, gives it the same value.
constexpr uint8_t FNODATA = 0x01, FOUTLET = 0x02, FNONPASS = 0x04, FCONF = 0x08,
                  FBELOW = 0x10, FBELOWA = 0x20, FCLEAN = 0x40, FUNSURE = 0x80;

// fill_passable() of a quantized value q = RN(k / 1000) (k an integer, as
// fill_quantize makes every value the fill sees).  With minE = 0 and
// 0 <= q < 4096, p = RN(1000 q) lies within 0.25 of k: |q - k/1000| is at
// most half an ulp of q (<= 2^-13), so |1000 q - k| <= 0.123, and rounding
// 1000 q (< 2^22) moves it by at most 0.125.  Then toIndex(q) = trunc(p)
// equals k exactly when p >= k = rint(p), and toElev(k) = RN(k / 1000) = q,
// while toElev of any other index differs from q (values 0.001 apart are
// distinct floats below 8192): passable <=> p >= rint(p), no division.
// Other values take the general test.
__device__ __forceinline__ bool passable_quantized(float q, float minE) {
  if (minE == 0.0f && q >= 0.0f && q < 4096.0f) {
    const float p = __fmul_rn(1000.0f, q);
    return p >= rintf(p);
  }
  return fill_passable(q, minE);
}

// Flags of a cell before the floods: NODATA; otherwise non-passable when
// its quantized value q fails the round trip at minE, and an outlet (clean
// from the start: outlets keep q in both floods) on the border or at 0.
__device__ __forceinline__ uint8_t fill_init_flags(float q, float nodata, float minE,
                                                   bool border) {
  if (q == nodata) return FNODATA;
  uint8_t f = passable_quantized(q, minE) ? 0 : FNONPASS;
  if (border || q == 0.0f) f |= FOUTLET | FCLEAN;
  return f;
}

}  // namespace cageo
