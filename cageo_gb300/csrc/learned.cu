// learned.cu -- the learned warm start of the exact fill (no counterpart in
// the reference).
//
// A small convolutional network predicts, per cell, how deep the exact fill
// will flood it.  Cells predicted dry start the fill at their own elevation,
// the others at +inf; the fill then relaxes down from that start
// (fill_run_exact with a warm surface).  A start below the answer anywhere
// leaves a wrong, lower surface, so the pipeline verifies every warm-started
// realization by its tracing (every cell must drain to an outlet) and
// repairs the cells that do not drain (see pipeline.cu): the counts stay
// bit-identical to the plain exact fill.
//
// Network: features (4 channels) -> conv 3x3, 32 channels, ReLU -> conv 3x3,
// 32 channels, ReLU -> conv 3x3, 1 channel (predicted depth, metres).  Zero
// padding at the grid's edges.  Weights are rounded to bf16 wherever they
// are used; every sum accumulates in fp32.
//
// Parameter vector (fp32 master copy, CAGEO_WS_PARAMS floats):
//   W1[32][4][9], b1[32], W2[32][32][9], b2[32], W3[1][32][9], b3[1]
// with taps t = (dy+1)*3 + (dx+1), a cell's output reading input (y+dy, x+dx).
//
// Training kernels (plain fp32 CUDA cores, planar [batch][channel][H][W]
// activations): forward convolution, input gradients as the forward
// convolution with flipped, transposed weights, weight gradients as per
// (output, input) channel reductions, mean-squared-error loss, Adam.
// Inference: one fused kernel per 32x16 tile of cells that computes the
// features and the three layers in shared memory with bf16 mma.sync tensor
// instructions (fp32 accumulation) and writes the warm surface.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cuda_bf16.h>
#include "common.cuh"

namespace cageo {

constexpr int kWsCin = 4, kWsCh = 32;
constexpr int kOffW1 = 0, kOffB1 = 1152, kOffW2 = 1184, kOffB2 = 10400, kOffW3 = 10432,
              kOffB3 = 10720, kWsParams = 10721;
static_assert(kOffB1 == kWsCh * kWsCin * 9 && kOffW2 == kOffB1 + kWsCh &&
                  kOffB2 == kOffW2 + kWsCh * kWsCh * 9 && kOffW3 == kOffB2 + kWsCh &&
                  kOffB3 == kOffW3 + kWsCh * 9 && kWsParams == kOffB3 + 1,
              "parameter layout");

__host__ __device__ inline float bf16_round(float x) {
  return __bfloat162float(__float2bfloat16_rn(x));
}

// ---- features ----------------------------------------------------------------
// Per cell, from the burned realistic elevations v over the valid (in-grid,
// non-NODATA) cells of its neighbourhood:
//   f0 = v - min over 3x3, f1 = v - min over 7x7, f2 = max over 7x7 - v,
//   f3 = v - mean over 7x7 (sum in row order, then divided by the count).
// NODATA cells have all-zero features.  `at(dy, dx)` returns the value at
// the offset or NAN outside the grid.
template <class At>
__device__ __forceinline__ void ws_features(float c, float nodata, At at, float f[4]) {
  if (c == nodata) {
    f[0] = f[1] = f[2] = f[3] = 0.0f;
    return;
  }
  float mn3 = c, mn7 = c, mx7 = c, sum = 0.0f;
  int cnt = 0;
  for (int dy = -3; dy <= 3; dy++)
    for (int dx = -3; dx <= 3; dx++) {
      const float e = at(dy, dx);
      if (e != e || e == nodata) continue;  // outside the grid or NODATA
      mn7 = fminf(mn7, e);
      mx7 = fmaxf(mx7, e);
      sum = __fadd_rn(sum, e);
      cnt++;
      if (dy >= -1 && dy <= 1 && dx >= -1 && dx <= 1) mn3 = fminf(mn3, e);
    }
  f[0] = __fsub_rn(c, mn3);
  f[1] = __fsub_rn(c, mn7);
  f[2] = __fsub_rn(mx7, c);
  f[3] = __fsub_rn(c, __fdiv_rn(sum, (float)cnt));
}

// Planar features [b][4][H][W] of a batch of B grids [b][H][W].
__global__ void ws_features_kernel(const float* __restrict__ v, float* __restrict__ feat, int W,
                                   int H, int B, float nodata) {
  const int64_t n = (int64_t)W * H;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * B) return;
  const int b = (int)(i / n);
  const int64_t c = i - (int64_t)b * n;
  const int x = (int)(c % W), y = (int)(c / W);
  const float* g = v + (int64_t)b * n;
  auto at = [&](int dy, int dx) {
    const int xx = x + dx, yy = y + dy;
    return (xx < 0 || yy < 0 || xx >= W || yy >= H) ? NAN : g[(int64_t)yy * W + xx];
  };
  float f[4];
  ws_features(g[c], nodata, at, f);
  for (int k = 0; k < 4; k++) feat[((int64_t)b * 4 + k) * n + c] = f[k];
}

// ---- training: convolution forward (also used for input gradients) ----------
// out[b][co](y,x) = bias[co] + sum_ci sum_t w[co][ci][t] * in[b][ci](y+dy, x+dx),
// zero outside; optional ReLU.  Weights (bf16-rounded) staged in shared
// memory; one thread per output cell, all output channels in registers.
template <int COUT>
__global__ void __launch_bounds__(128) ws_conv_fwd_kernel(const float* __restrict__ in,
                                                          int cin, const float* __restrict__ w,
                                                          const float* __restrict__ bias,
                                                          float* __restrict__ out, int W, int H,
                                                          int B, int relu) {
  extern __shared__ float sw[];  // [COUT][cin][9]
  for (int k = threadIdx.x; k < COUT * cin * 9; k += blockDim.x) sw[k] = bf16_round(w[k]);
  __syncthreads();
  const int64_t n = (int64_t)W * H;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * B) return;
  const int b = (int)(i / n);
  const int64_t c = i - (int64_t)b * n;
  const int x = (int)(c % W), y = (int)(c / W);
  float acc[COUT];
#pragma unroll
  for (int co = 0; co < COUT; co++) acc[co] = bias ? bf16_round(bias[co]) : 0.0f;
  for (int ci = 0; ci < cin; ci++) {
    const float* plane = in + ((int64_t)b * cin + ci) * n;
#pragma unroll
    for (int t = 0; t < 9; t++) {
      const int xx = x + t % 3 - 1, yy = y + t / 3 - 1;
      if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
      const float a = plane[(int64_t)yy * W + xx];
#pragma unroll
      for (int co = 0; co < COUT; co++) acc[co] = fmaf(sw[(co * cin + ci) * 9 + t], a, acc[co]);
    }
  }
  float* o = out + (int64_t)b * COUT * n + c;
#pragma unroll
  for (int co = 0; co < COUT; co++) o[(int64_t)co * n] = relu ? fmaxf(acc[co], 0.0f) : acc[co];
}

// wt[ci][co][t] = w[co][ci][8 - t]: the weights of the input-gradient pass.
__global__ void ws_flip_kernel(const float* __restrict__ w, float* __restrict__ wt, int cout,
                               int cin) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cout * cin * 9) return;
  const int t = k % 9, ci = (k / 9) % cin, co = k / (9 * cin);
  wt[(ci * cout + co) * 9 + (8 - t)] = w[k];
}

// g *= (a > 0): the ReLU's gradient mask.
__global__ void ws_relu_mask_kernel(float* __restrict__ g, const float* __restrict__ a,
                                    int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(a[i] > 0.0f)) g[i] = 0.0f;
}

// Weight gradients of one (output, input) channel pair per block:
// gw[co][ci][t] += sum_b sum_cell dz[b][co](y,x) * a[b][ci](y+dy, x+dx);
// the blocks with ci == 0 also add gb[co] += sum dz[b][co].
__global__ void __launch_bounds__(256) ws_wgrad_kernel(const float* __restrict__ dz, int cout,
                                                       const float* __restrict__ a, int cin,
                                                       float* __restrict__ gw,
                                                       float* __restrict__ gb, int W, int H,
                                                       int B) {
  const int co = blockIdx.x / cin, ci = blockIdx.x % cin;
  const int64_t n = (int64_t)W * H;
  float s[10] = {};
  for (int b = 0; b < B; b++) {
    const float* d = dz + ((int64_t)b * cout + co) * n;
    const float* p = a + ((int64_t)b * cin + ci) * n;
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
      const float g = d[c];
      if (g == 0.0f) continue;
      const int x = (int)(c % W), y = (int)(c / W);
#pragma unroll
      for (int t = 0; t < 9; t++) {
        const int xx = x + t % 3 - 1, yy = y + t / 3 - 1;
        if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
        s[t] = fmaf(g, p[(int64_t)yy * W + xx], s[t]);
      }
      s[9] += g;
    }
  }
  __shared__ float red[8][10];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 10; t++) {
    float v = s[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][t] = v;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    float v = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) v += red[k][threadIdx.x];
    if (threadIdx.x < 9) gw[(co * cin + ci) * 9 + threadIdx.x] += v;
    else if (ci == 0 && gb) gb[co] += v;
  }
}

// Mean squared error over the cells at least `margin` cells inside each
// grid: dy = 2 (y - t) / count there, 0 elsewhere; loss (sum) accumulated.
__global__ void ws_mse_kernel(const float* __restrict__ y, const float* __restrict__ t,
                              float* __restrict__ dy, float* __restrict__ loss, int W, int H,
                              int B, int margin, float inv_count) {
  const int64_t n = (int64_t)W * H;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (i < n * B) {
    const int64_t c = i % n;
    const int x = (int)(c % W), yy = (int)(c / W);
    const bool in = x >= margin && yy >= margin && x < W - margin && yy < H - margin;
    const float d = y[i] - t[i];
    dy[i] = in ? 2.0f * d * inv_count : 0.0f;
    l = in ? d * d * inv_count : 0.0f;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.0f) atomicAdd(loss, l);
}

__global__ void ws_adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                               float* __restrict__ m, float* __restrict__ v, int n, float lr,
                               float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace cageo

namespace cageo {

// ---- inference: fused features + 3 layers on bf16 tensor instructions --------
// A block owns a 32x16 tile of outputs; the layers need one more cell of
// context each: layer-2 outputs over 34x18, layer-1 outputs over 36x20,
// features over 38x22, elevations over 44x28 (the 7x7 feature window).
// Everything outside the grid is zero for the convolutions (their padding).
constexpr int kTX = 32, kTY = 16;
constexpr int kVX = kTX + 12, kVY = kTY + 12;    // elevations
constexpr int kFX = kTX + 6, kFY = kTY + 6;      // features
constexpr int kA1X = kTX + 4, kA1Y = kTY + 4;    // layer-1 outputs
constexpr int kA2X = kTX + 2, kA2Y = kTY + 2;    // layer-2 outputs
constexpr int kAS = 40;                          // activation row stride (bf16), 80 B
constexpr int kW1S = 56, kW2S = 296;             // weight row strides (bf16)
constexpr int kInferWarps = 16;

struct InferSmem {
  float v[kVY * kVX];
  __nv_bfloat16 f[kFY * kFX * 4];
  __nv_bfloat16 a1[kA1Y * kA1X * kAS];
  __nv_bfloat16 a2[kA2Y * kA2X * kAS];
  __nv_bfloat16 w1[kWsCh * kW1S];     // [n][k], k = tap*4 + ci (36 used, 48 in the k-steps)
  __nv_bfloat16 w2[kWsCh * kW2S];     // [n][k], k = tap*32 + ci
  __nv_bfloat16 w3[8 * kW2S];         // [n][k], only n = 0 non-zero
  float b1[kWsCh], b2[kWsCh], b3;
};

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ void mma_bf16(float c[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ldmatrix: four (two) 8x8 b16 matrices from shared memory; lane i gives
// the address of row i % 8 of matrix i / 8 (16 contiguous bytes, 16-byte
// aligned), and receives the elements (row i / 4, columns 2 (i % 4) and
// 2 (i % 4) + 1) of each matrix in order: the mma.sync fragment layout.
__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3,
                                        const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a)
               : "memory");
}

__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(a)
               : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&h);
}

__global__ void __launch_bounds__(kInferWarps * 32, 1)
ws_infer_kernel(const float* __restrict__ params, const float* __restrict__ vg,
                float* __restrict__ warm, float* __restrict__ depth, int W, int H, float nodata,
                float threshold) {
  extern __shared__ __align__(16) unsigned char smraw[];
  InferSmem& s = *reinterpret_cast<InferSmem*>(smraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, tq = lane & 3;
  // Weights, bf16, in the [n][k] layouts the B fragments read.
  for (int k = tid; k < kWsCh * kW1S; k += blockDim.x) {
    const int n = k / kW1S, kk = k % kW1S;
    float w = 0.0f;
    if (kk < 36) w = params[kOffW1 + (n * kWsCin + kk % 4) * 9 + kk / 4];
    s.w1[k] = __float2bfloat16_rn(w);
  }
  for (int k = tid; k < kWsCh * kW2S; k += blockDim.x) {
    const int n = k / kW2S, kk = k % kW2S;
    float w = 0.0f;
    if (kk < 288) w = params[kOffW2 + (n * kWsCh + kk % 32) * 9 + kk / 32];
    s.w2[k] = __float2bfloat16_rn(w);
  }
  for (int k = tid; k < 8 * kW2S; k += blockDim.x) {
    const int n = k / kW2S, kk = k % kW2S;
    float w = 0.0f;
    if (n == 0 && kk < 288) w = params[kOffW3 + (kk % 32) * 9 + kk / 32];
    s.w3[k] = __float2bfloat16_rn(w);
  }
  if (tid < kWsCh) {
    s.b1[tid] = bf16_round(params[kOffB1 + tid]);
    s.b2[tid] = bf16_round(params[kOffB2 + tid]);
  }
  if (tid == 0) s.b3 = bf16_round(params[kOffB3]);
  __syncthreads();  // weights staged
  // Layer 3's B fragments for its 18 k-steps (only output column 0 is used).
  uint32_t b3[36];
  {
    const int bn = lane & 7, bkoff = ((lane >> 3) & 1) << 3;
#pragma unroll
    for (int ks = 0; ks < 18; ks++)
      ldsm_x2(b3[2 * ks], b3[2 * ks + 1], &s.w3[bn * kW2S + ks * 16 + bkoff]);
  }
  const int tiles_x = (W + kTX - 1) / kTX, tiles_y = (H + kTY - 1) / kTY;
  for (int tile = blockIdx.x; tile < tiles_x * tiles_y; tile += gridDim.x) {
    const int x0 = (tile % tiles_x) * kTX, y0 = (tile / tiles_x) * kTY;
    __syncthreads();  // weights staged / previous tile done
    for (int k = tid; k < kVY * kVX; k += blockDim.x) {
      const int gy = y0 - 6 + k / kVX, gx = x0 - 6 + k % kVX;
      if (gx < 0 || gy < 0 || gx >= W || gy >= H) s.v[k] = NAN;
      else cp_async4(&s.v[k], vg + (int64_t)gy * W + gx);  // all in flight at once
    }
    cp_async_wait();
    __syncthreads();
    // Features (ws_features), separably: first per elevation row and
    // feature column the 7-wide minimum, maximum, sum and count of the
    // valid cells and the 3-wide minimum, then the 7-high (3-high) column
    // of those.  Minima and maxima equal ws_features' exactly; the mean's
    // sum runs in another order (last bits).  The row results use the
    // layer-1 buffer, which is free until layer 1 runs.
    {
      float* rmn7 = reinterpret_cast<float*>(s.a1);
      float* rmx7 = rmn7 + kVY * kFX;
      float* rsum = rmx7 + kVY * kFX;
      float* rcnt = rsum + kVY * kFX;
      float* rmn3 = rcnt + kVY * kFX;
      for (int k = tid; k < kVY * kFX; k += blockDim.x) {
        const int vy = k / kFX, fx = k - vy * kFX;
        const float* r = &s.v[vy * kVX + fx];  // columns fx .. fx + 6 (centre fx + 3)
        float mn = kInf, mx = -kInf, sm = 0.0f, m3 = kInf;
        int cnt = 0;
#pragma unroll
        for (int dx = 0; dx < 7; dx++) {
          const float e = r[dx];
          if (e != e || e == nodata) continue;  // outside the grid or NODATA
          mn = fminf(mn, e);
          mx = fmaxf(mx, e);
          sm = __fadd_rn(sm, e);
          cnt++;
          if (dx >= 2 && dx <= 4) m3 = fminf(m3, e);
        }
        rmn7[k] = mn;
        rmx7[k] = mx;
        rsum[k] = sm;
        rcnt[k] = (float)cnt;
        rmn3[k] = m3;
      }
      __syncthreads();
      for (int k = tid; k < kFY * kFX; k += blockDim.x) {
        const int fy = k / kFX, fx = k - fy * kFX;
        const float c = s.v[(fy + 3) * kVX + fx + 3];
        float f[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (c == c && c != nodata) {  // inside the grid and not NODATA
          float mn = kInf, mx = -kInf, sm = 0.0f, cn = 0.0f, m3 = kInf;
#pragma unroll
          for (int dy = 0; dy < 7; dy++) {
            const int b = (fy + dy) * kFX + fx;
            mn = fminf(mn, rmn7[b]);
            mx = fmaxf(mx, rmx7[b]);
            sm = __fadd_rn(sm, rsum[b]);
            cn += rcnt[b];
            if (dy >= 2 && dy <= 4) m3 = fminf(m3, rmn3[b]);
          }
          f[0] = __fsub_rn(c, m3);
          f[1] = __fsub_rn(c, mn);
          f[2] = __fsub_rn(mx, c);
          f[3] = __fsub_rn(c, __fdiv_rn(sm, cn));
        }
        uint2 pk;
        pk.x = pack_bf16(f[0], f[1]);
        pk.y = pack_bf16(f[2], f[3]);
        *reinterpret_cast<uint2*>(&s.f[k * 4]) = pk;
      }
    }
    __syncthreads();
    // Layer 1: M = 36x20 cells (45 m-tiles), K = 9 taps x 4 features (3 k-steps), N = 32.
    for (int mt = warp; mt < kA1X * kA1Y / 16; mt += kInferWarps) {
      float acc[4][4] = {};
      const int r0 = mt * 16 + g, r1 = r0 + 8;
      const int p0 = (r0 / kA1X) * kFX + r0 % kA1X, p1 = (r1 / kA1X) * kFX + r1 % kA1X;
#pragma unroll
      for (int ks = 0; ks < 3; ks++) {
        uint32_t a[4];
#pragma unroll
        for (int h = 0; h < 2; h++) {  // k = ks*16 + 2tq (+8h)
          const int k = ks * 16 + 2 * tq + 8 * h, tap = k >> 2, ci = k & 3;
          if (tap < 9) {
            const int off = (tap / 3) * kFX + tap % 3;
            a[2 * h] = ld32(&s.f[(p0 + off) * 4 + ci]);
            a[2 * h + 1] = ld32(&s.f[(p1 + off) * 4 + ci]);
          } else {
            a[2 * h] = a[2 * h + 1] = 0u;
          }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const __nv_bfloat16* wb = &s.w1[(j * 8 + g) * kW1S + ks * 16 + 2 * tq];
          mma_bf16(acc[j], a[0], a[1], a[2], a[3], ld32(wb), ld32(wb + 8));
        }
      }
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = h ? r1 : r0;
        const int gy = y0 - 2 + r / kA1X, gx = x0 - 2 + r % kA1X;
        const bool in = gx >= 0 && gy >= 0 && gx < W && gy < H;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int n = j * 8 + 2 * tq;
          const float lo = in ? fmaxf(acc[j][2 * h] + s.b1[n], 0.0f) : 0.0f;
          const float hi = in ? fmaxf(acc[j][2 * h + 1] + s.b1[n + 1], 0.0f) : 0.0f;
          *reinterpret_cast<uint32_t*>(&s.a1[r * kAS + n]) = pack_bf16(lo, hi);
        }
      }
    }
    __syncthreads();
    // Layer 2: M = 34x18 cells (39 m-tiles, the last one partly padding),
    // K = 9 taps x 32 channels (18 k-steps), N = 32.  A and B fragments come
    // from ldmatrix: the A rows are cells (the 16 channels of a k-step are
    // 32 contiguous bytes of a cell), the B rows output channels.  A warp
    // takes two m-tiles at a time so each k-step's B fragments serve both.
    constexpr int kM2 = kA2X * kA2Y, kMT2 = (kM2 + 15) / 16;
    {
      const int arow = lane & 15, akoff = (lane >> 4) << 3;
      const int bn = (lane & 7) + ((lane >> 4) << 3), bkoff = ((lane >> 3) & 1) << 3;
      for (int mt = warp; mt < kMT2; mt += 2 * kInferWarps) {
        const int mtb = mt + kInferWarps;
        const bool two = mtb < kMT2;
        const int ra = min(mt * 16 + arow, kM2 - 1), rb = min(mtb * 16 + arow, kM2 - 1);
        const int pa = (ra / kA2X) * kA1X + ra % kA2X, pb = (rb / kA2X) * kA1X + rb % kA2X;
        float acc[2][4][4] = {};
#pragma unroll 2
        for (int ks = 0; ks < 18; ks++) {
          const int tap = ks >> 1, cb = (ks & 1) * 16;
          const int off = (tap / 3) * kA1X + tap % 3;
          uint32_t b[8];
          ldsm_x4(b[0], b[1], b[2], b[3], &s.w2[bn * kW2S + ks * 16 + bkoff]);
          ldsm_x4(b[4], b[5], b[6], b[7], &s.w2[(bn + 16) * kW2S + ks * 16 + bkoff]);
          uint32_t a[4];
          ldsm_x4(a[0], a[1], a[2], a[3], &s.a1[(pa + off) * kAS + cb + akoff]);
#pragma unroll
          for (int j = 0; j < 4; j++) mma_bf16(acc[0][j], a[0], a[1], a[2], a[3], b[2 * j], b[2 * j + 1]);
          if (two) {
            ldsm_x4(a[0], a[1], a[2], a[3], &s.a1[(pb + off) * kAS + cb + akoff]);
#pragma unroll
            for (int j = 0; j < 4; j++)
              mma_bf16(acc[1][j], a[0], a[1], a[2], a[3], b[2 * j], b[2 * j + 1]);
          }
        }
#pragma unroll
        for (int m = 0; m < 2; m++) {
          if (m == 1 && !two) break;
          const int r0 = (m ? mtb : mt) * 16 + g, r1 = r0 + 8;
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const int r = h ? r1 : r0;
            if (r >= kM2) continue;
            const int gy = y0 - 1 + r / kA2X, gx = x0 - 1 + r % kA2X;
            const bool in = gx >= 0 && gy >= 0 && gx < W && gy < H;
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const int n = j * 8 + 2 * tq;
              const float lo = in ? fmaxf(acc[m][j][2 * h] + s.b2[n], 0.0f) : 0.0f;
              const float hi = in ? fmaxf(acc[m][j][2 * h + 1] + s.b2[n + 1], 0.0f) : 0.0f;
              *reinterpret_cast<uint32_t*>(&s.a2[r * kAS + n]) = pack_bf16(lo, hi);
            }
          }
        }
      }
    }
    __syncthreads();
    // Layer 3: M = 32x16 outputs (32 m-tiles), K = 288, N = 8 (only column 0
    // used).  The B fragments of all 18 k-steps are the same for every
    // m-tile and stay in registers (b3, loaded once per block).
    for (int mt = warp; mt < kTX * kTY / 16; mt += kInferWarps) {
      // Two accumulators (even and odd k-steps) halve the dependent chain.
      float acc[4] = {}, acc2[4] = {};
      const int r0 = mt * 16 + g, r1 = r0 + 8;
      const int ar = mt * 16 + (lane & 15), akoff = (lane >> 4) << 3;
      const int pa = (ar / kTX) * kA2X + ar % kTX;
#pragma unroll
      for (int ks = 0; ks < 18; ks++) {
        const int tap = ks >> 1, cb = (ks & 1) * 16;
        const int off = (tap / 3) * kA2X + tap % 3;
        uint32_t a[4];
        ldsm_x4(a[0], a[1], a[2], a[3], &s.a2[(pa + off) * kAS + cb + akoff]);
        mma_bf16((ks & 1) ? acc2 : acc, a[0], a[1], a[2], a[3], b3[2 * ks], b3[2 * ks + 1]);
      }
#pragma unroll
      for (int q = 0; q < 4; q++) acc[q] += acc2[q];
      if (tq == 0) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int r = h ? r1 : r0;
          const int gy = y0 + r / kTX, gx = x0 + r % kTX;
          if (gx >= W || gy >= H) continue;
          const int64_t i = (int64_t)gy * W + gx;
          const float d = acc[2 * h] + s.b3;
          if (depth) depth[i] = d;
          if (warm) warm[i] = d < threshold ? vg[i] : kInf;
        }
      }
    }
  }
}

cageo_status ws_infer(const float* params, const float* v, float* warm, float* depth, int W,
                      int H, float nodata, float threshold, cudaStream_t s) {
  static PerDevice sm_count;
  const size_t smem = sizeof(InferSmem);
  int blocks = 0;
  cageo_status st = per_device(sm_count, &blocks, [&](int dev, int* v) -> cageo_status {
    CAGEO_CUDA(cudaFuncSetAttribute(ws_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    int sms = 0;
    CAGEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *v = sms > 1 ? sms : 1;
    return CAGEO_OK;
  });
  if (st) return st;
  const int tiles = ((W + kTX - 1) / kTX) * ((H + kTY - 1) / kTY);
  ws_infer_kernel<<<std::min(blocks, tiles), kInferWarps * 32, smem, s>>>(params, v, warm, depth,
                                                                         W, H, nodata, threshold);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

}  // namespace cageo

using namespace cageo;

namespace {
inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }
}  // namespace

extern "C" int cageo_ws_param_count(void) { return kWsParams; }

extern "C" cageo_status cageo_ws_features(const float* d_v, float* d_feat, int W, int H, int B,
                                          float nodata_dem, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_v && d_feat && valid_dims(W, H) && B >= 1, "pointers, size and batch");
  const int64_t n = (int64_t)W * H * B;
  ws_features_kernel<<<nblk(n, 256), 256, 0, stream>>>(d_v, d_feat, W, H, B, nodata_dem);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

extern "C" cageo_status cageo_ws_forward(const float* d_params, const float* d_feat, int W,
                                         int H, int B, float* d_a1, float* d_a2, float* d_out,
                                         cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_params && d_feat && d_a1 && d_a2 && d_out && valid_dims(W, H) && B >= 1,
                  "pointers, size and batch");
  const int64_t n = (int64_t)W * H * B;
  const unsigned g = nblk(n, 128);
  ws_conv_fwd_kernel<32><<<g, 128, 32 * 4 * 9 * 4, stream>>>(
      d_feat, 4, d_params + kOffW1, d_params + kOffB1, d_a1, W, H, B, 1);
  ws_conv_fwd_kernel<32><<<g, 128, 32 * 32 * 9 * 4, stream>>>(
      d_a1, 32, d_params + kOffW2, d_params + kOffB2, d_a2, W, H, B, 1);
  ws_conv_fwd_kernel<1><<<g, 128, 32 * 9 * 4, stream>>>(d_a2, 32, d_params + kOffW3,
                                                         d_params + kOffB3, d_out, W, H, B, 0);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

extern "C" cageo_status cageo_ws_backward(const float* d_params, const float* d_feat,
                                          const float* d_a1, const float* d_a2,
                                          const float* d_dout, int W, int H, int B,
                                          float* d_grad, float* d_tmp1, float* d_tmp2,
                                          float* d_wflip, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_params && d_feat && d_a1 && d_a2 && d_dout && d_grad && d_tmp1 && d_tmp2 &&
                      d_wflip && valid_dims(W, H) && B >= 1,
                  "pointers, size and batch");
  const int64_t n = (int64_t)W * H * B, n32 = 32 * n;
  const unsigned g = nblk(n, 128);
  // Layer 3: weight gradients, then the gradient of its input (ReLU-masked).
  ws_wgrad_kernel<<<32, 256, 0, stream>>>(d_dout, 1, d_a2, 32, d_grad + kOffW3,
                                          d_grad + kOffB3, W, H, B);
  ws_flip_kernel<<<nblk(288, 256), 256, 0, stream>>>(d_params + kOffW3, d_wflip, 1, 32);
  ws_conv_fwd_kernel<32><<<g, 128, 32 * 1 * 9 * 4, stream>>>(d_dout, 1, d_wflip, nullptr, d_tmp1,
                                                             W, H, B, 0);
  ws_relu_mask_kernel<<<nblk(n32, 256), 256, 0, stream>>>(d_tmp1, d_a2, n32);
  // Layer 2.
  ws_wgrad_kernel<<<32 * 32, 256, 0, stream>>>(d_tmp1, 32, d_a1, 32, d_grad + kOffW2,
                                               d_grad + kOffB2, W, H, B);
  ws_flip_kernel<<<nblk(9216, 256), 256, 0, stream>>>(d_params + kOffW2, d_wflip, 32, 32);
  ws_conv_fwd_kernel<32><<<g, 128, 32 * 32 * 9 * 4, stream>>>(d_tmp1, 32, d_wflip, nullptr,
                                                              d_tmp2, W, H, B, 0);
  ws_relu_mask_kernel<<<nblk(n32, 256), 256, 0, stream>>>(d_tmp2, d_a1, n32);
  // Layer 1 (its input, the features, needs no gradient).
  ws_wgrad_kernel<<<32 * 4, 256, 0, stream>>>(d_tmp2, 32, d_feat, 4, d_grad + kOffW1,
                                              d_grad + kOffB1, W, H, B);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

extern "C" cageo_status cageo_ws_mse(const float* d_y, const float* d_target, float* d_dy,
                                     float* d_loss, int W, int H, int B, int margin,
                                     cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_y && d_target && d_dy && d_loss && valid_dims(W, H) && B >= 1,
                  "pointers, size and batch");
  CAGEO_CHECK_ARG(margin >= 0 && 2 * margin < W && 2 * margin < H, "margin");
  const int64_t n = (int64_t)W * H * B;
  const float cnt = (float)(W - 2 * margin) * (float)(H - 2 * margin) * (float)B;
  ws_mse_kernel<<<nblk(n, 256), 256, 0, stream>>>(d_y, d_target, d_dy, d_loss, W, H, B, margin,
                                                  1.0f / cnt);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

extern "C" cageo_status cageo_ws_adam(float* d_params, const float* d_grad, float* d_m,
                                      float* d_v, int n, float lr, float beta1, float beta2,
                                      float eps, int step, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_params && d_grad && d_m && d_v && n > 0 && step >= 1, "arguments");
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  ws_adam_kernel<<<nblk(n, 256), 256, 0, stream>>>(d_params, d_grad, d_m, d_v, n, lr, beta1,
                                                   beta2, eps, c1, c2);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

extern "C" cageo_status cageo_ws_infer(const float* d_params, const float* d_v, float* d_warm,
                                       float* d_depth, int W, int H, float nodata_dem,
                                       float threshold, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_params && d_v && (d_warm || d_depth) && valid_dims(W, H),
                  "pointers and size");
  return ws_infer(d_params, d_v, d_warm, d_depth, W, H, nodata_dem, threshold, stream);
}
