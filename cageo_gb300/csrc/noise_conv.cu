// noise_conv.cu -- A1 Philox Gaussian noise and A3 process convolution.
//
// Convolution kernels stage a (tile + 2r halo) block of the input in shared
// memory with periodic wrap and compute every output with the reference's
// summation order (ascending taps, sum starting at 0, unfused multiply and
// add), so they equal ConvolutionAlgorithm_CPU_OpenMP bit for bit.  The
// same kernels, instantiated with the FrontEpilogue, fuse the realistic-DEM,
// burning and quantization steps of a realization into their store.
#include <type_traits>
#include "common.cuh"
#include "front.cuh"
#include "stage_math.cuh"

namespace cageo {

// ---- A1 ------------------------------------------------------------------
// One thread per group of 4 consecutive cells: one Philox call gives four
// uniforms -> two Box-Muller pairs -> four N(0,1) deviates.
__global__ void noise_kernel(float* __restrict__ out, int64_t n, uint32_t k0,
                             uint32_t k1, uint32_t realization,
                             const uint32_t* __restrict__ dreal, float mean,
                             float sd) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t base = g * 4;
  if (base >= n) return;
  if (dreal) realization += *dreal;  // an offset from the device counter
  U4 ctr = {(uint32_t)g, realization, kNoiseTag, (uint32_t)(g >> 32)};
  U4 r = philox4x32_10(ctr, k0, k1);
  float z[4];
  {
    float rad = sqrtf(-2.0f * logf(u01_open(r.x)));
    float s, c;
    sincospif(2.0f * u01_open(r.y), &s, &c);
    z[0] = rad * c;
    z[1] = rad * s;
  }
  {
    float rad = sqrtf(-2.0f * logf(u01_open(r.z)));
    float s, c;
    sincospif(2.0f * u01_open(r.w), &s, &c);
    z[2] = rad * c;
    z[3] = rad * s;
  }
  float v[4];
#pragma unroll
  for (int j = 0; j < 4; j++) v[j] = __fadd_rn(mean, __fmul_rn(z[j], sd));
  // One float4 store when the field is 16-byte aligned (a caller's buffer
  // may start at any 4-byte boundary: then four scalar stores).
  if (base + 4 <= n && (((uintptr_t)out) & 15u) == 0) {
    *reinterpret_cast<float4*>(out + base) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    for (int j = 0; j < 4 && base + j < n; j++) out[base + j] = v[j];
  }
}

// ---- A3 separable (Gaussian) ----------------------------------------------
// Output tile of a block (columns x rows), 256 threads.  A wider or taller
// tile stages less halo per output but leaves fewer blocks per SM, and the
// column pass (items of 8 rows x 2 columns over the tile's width plus the
// halo) and the row pass (8 outputs per item) fill the 256 threads
// differently for each shape and radius: at radius 15, 64 x 32 gives the
// column pass 188 items, 96 x 32 gives it 252.  The cageo_convolve stage
// uses the first shape; the fused front takes the pipeline's choice.
struct SepTile {
  int tw, th;
};
constexpr SepTile kSepTiles[kConvTiles] = {{64, 32}, {128, 32}, {64, 64}, {96, 32}};
constexpr int kSepThreads = 256;

// Periodic index: one period either way by compare-and-add (every index a
// valid output reads is within one period, since r < W and r < H); the
// modulo only serves padding rows/columns of very small grids.
__device__ __forceinline__ int wrap_idx(int v, int n) {
  if (v < 0) v += n;
  else if (v >= n) v -= n;
  if ((unsigned)v >= (unsigned)n) {
    v %= n;
    if (v < 0) v += n;
  }
  return v;
}

// Epilogues: pre(i) loads what the output at i needs besides the
// convolved value (issued before the convolution so the loads overlap it);
// operator() writes the output.
struct StoreEpilogue {
  float* out;
  struct Pre {};
  __device__ inline Pre pre(int64_t) const { return {}; }
  __device__ inline float operator()(int64_t i, int, int, float v, Pre) const {
    out[i] = v;
    return v;
  }
};

struct FrontEpilogue {
  FrontParams p;
  struct Pre {
    float dem;
    uint8_t code;
  };
  __device__ inline Pre pre(int64_t i) const { return {p.dem[i], p.code[i]}; }
  __device__ inline float operator()(int64_t i, int x, int y, float v, Pre pr) const {
    return front_epilogue(p, i, x, y, v, pr.dem, pr.code);
  }
};

template <class Epi>
__device__ inline void block_min_out(float local_min, const Epi&) {}

__device__ inline void block_min_out(float local_min, const FrontEpilogue& e) {
  // Block-wide min of q, then one ordered atomicMin.
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1)
    local_min = fminf(local_min, __shfl_xor_sync(0xffffffffu, local_min, o));
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = local_min;
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    float m = lane < nw ? red[lane] : kInf;
    for (int o = 16; o > 0; o >>= 1)
      m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m < kInf) atomicMin(e.p.min_ord, float_to_ordered(m));
  }
}

// a0 += w0 * t and a1 += w1 * t, each product and each sum rounded to
// nearest on its own (as __fmul_rn / __fadd_rn, no contraction): the two
// products as one packed single-precision multiply, the sums as scalar
// __fadd_rn.  (A packed multiply feeding a packed add is contracted into a
// fused multiply-add by the assembler, .rn notwithstanding: one rounding
// fewer, different last bits.  A packed multiply feeding scalar adds, or
// scalar multiplies feeding a packed add, keep both roundings; both were
// checked against __fmul_rn + __fadd_rn over 4 M random operand pairs.)
__device__ __forceinline__ void muladd2_rn(float& a0, float& a1, float w0, float w1, float t) {
  float p0, p1;
  asm("{\n\t.reg .b64 wa, tt;\n\t"
      "mov.b64 wa, {%2, %3};\n\t"
      "mov.b64 tt, {%4, %4};\n\t"
      "mul.rn.f32x2 wa, wa, tt;\n\t"
      "mov.b64 {%0, %1}, wa;\n\t}"
      : "=f"(p0), "=f"(p1)
      : "f"(w0), "f"(w1), "f"(t));
  a0 = __fadd_rn(a0, p0);
  a1 = __fadd_rn(a1, p1);
}

// 8 outputs along a line from a sliding window of 8 registers: out[j] =
// sum_t v[j + t] * taps[t], t ascending, each sum starting at 0.  LC > 0:
// the tap count is a compile-time constant and the loop is fully unrolled
// (the window shifts become register renames); LC = 0: runtime count L.
template <int LC>
__device__ __forceinline__ void conv_line8(const float* __restrict__ v, int stride,
                                           const float* __restrict__ taps, int L,
                                           float acc[8]) {
  float win[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    win[j] = v[j * stride];
    acc[j] = 0.0f;
  }
  if (LC > 0) {
#pragma unroll
    for (int t = 0; t < LC; t++) {
      const float tap = taps[t];
#pragma unroll
      for (int j = 0; j < 8; j += 2) muladd2_rn(acc[j], acc[j + 1], win[j], win[j + 1], tap);
#pragma unroll
      for (int j = 0; j < 7; j++) win[j] = win[j + 1];
      if (t + 1 < LC) win[7] = v[(t + 8) * stride];
    }
  } else {
#pragma unroll 8
    for (int t = 0; t < L; t++) {
      const float tap = taps[t];
#pragma unroll
      for (int j = 0; j < 8; j += 2) muladd2_rn(acc[j], acc[j + 1], win[j], win[j + 1], tap);
#pragma unroll
      for (int j = 0; j < 7; j++) win[j] = win[j + 1];
      win[7] = (t + 1 < L) ? v[(t + 8) * stride] : 0.0f;
    }
  }
}

// p0 = w0 * t and p1 = w1 * t, each rounded to nearest, as one packed
// single-precision multiply.
__device__ __forceinline__ void mul2_rn(float& p0, float& p1, float w0, float w1, float t) {
  asm("{\n\t.reg .b64 wa, tt;\n\t"
      "mov.b64 wa, {%2, %3};\n\t"
      "mov.b64 tt, {%4, %4};\n\t"
      "mul.rn.f32x2 wa, wa, tt;\n\t"
      "mov.b64 {%0, %1}, wa;\n\t}"
      : "=f"(p0), "=f"(p1)
      : "f"(w0), "f"(w1), "f"(t));
}

// conv_line8 for two lines at once (v0, v1; same stride and taps): the
// window values of the two lines at one position are multiplied as one
// packed pair, and the two windows shift together, so the pairs stay put
// in registers.  ADJ: the lines are adjacent columns (v1 = v0 + 1, v0
// 8-byte aligned), loaded as one float2.  Each sum runs over t ascending,
// as in conv_line8.
template <int LC, bool ADJ>
__device__ __forceinline__ void conv_line8x2(const float* __restrict__ v0,
                                             const float* __restrict__ v1, int stride,
                                             const float* __restrict__ taps, int L,
                                             float a0[8], float a1[8]) {
  float w0[8], w1[8];
  auto load = [&](int k, float& x0, float& x1) {
    if (ADJ) {
      const float2 p = *reinterpret_cast<const float2*>(v0 + k * stride);
      x0 = p.x;
      x1 = p.y;
    } else {
      x0 = v0[k * stride];
      x1 = v1[k * stride];
    }
  };
#pragma unroll
  for (int j = 0; j < 8; j++) {
    load(j, w0[j], w1[j]);
    a0[j] = 0.0f;
    a1[j] = 0.0f;
  }
  auto tap_step = [&](float tap) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      float p0, p1;
      mul2_rn(p0, p1, w0[j], w1[j], tap);
      a0[j] = __fadd_rn(a0[j], p0);
      a1[j] = __fadd_rn(a1[j], p1);
    }
#pragma unroll
    for (int j = 0; j < 7; j++) {
      w0[j] = w0[j + 1];
      w1[j] = w1[j + 1];
    }
  };
  if (LC > 0) {
#pragma unroll
    for (int t = 0; t < LC; t++) {
      tap_step(taps[t]);
      if (t + 1 < LC) load(t + 8, w0[7], w1[7]);
    }
  } else {
#pragma unroll 4
    for (int t = 0; t < L; t++) {
      tap_step(taps[t]);
      if (t + 1 < L) load(t + 8, w0[7], w1[7]);
    }
  }
}

template <class Epi, int LC, int TW, int TH>
__global__ void __launch_bounds__(kSepThreads)
conv_sep_kernel(const float* __restrict__ in, int W, int H,
                const float* __restrict__ taps, int r, Epi epi) {
  static_assert(TW % 8 == 0 && TH % 8 == 0, "items are 8 outputs wide / 8 rows tall");
  extern __shared__ float sm[];
  const int L = 2 * r + 1;
  const int IW = TW + 2 * r, IH = TH + 2 * r;
  float* s_taps = sm;
  float* s_in = sm + ((L + 3) & ~3);
  float* s_tmp = s_in + IW * IH;
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  for (int t = threadIdx.x; t < L; t += blockDim.x) s_taps[t] = taps[t];
  {
    // Row and column of this thread's element, stepped by blockDim.x.
    int iy = threadIdx.x / IW, ix = threadIdx.x - iy * IW;
    const int dy = blockDim.x / IW, dx = blockDim.x - dy * IW;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < IW * IH; idx += blockDim.x) {
      const int gy = wrap_idx(y0 - r + iy, H), gx = wrap_idx(x0 - r + ix, W);
      cp_async4(&s_in[idx], &in[(int64_t)gy * W + gx]);  // all of them in flight at once
      iy += dy;
      ix += dx;
      if (ix >= IW) {
        ix -= IW;
        iy++;
      }
    }
    cp_async_wait();
  }
  __syncthreads();
  // Column pass: tmp[y][ix] = sum_t in[y+t][ix] * taps[t]; an item is 8
  // rows of two adjacent columns (IW is even).
  const int IW2 = IW / 2;
  for (int item = threadIdx.x; item < IW2 * (TH / 8); item += blockDim.x) {
    const int g = item / IW2, ix = 2 * (item - g * IW2);
    float a0[8], a1[8];
    conv_line8x2<LC, true>(s_in + (8 * g) * IW + ix, nullptr, IW, s_taps, L, a0, a1);
#pragma unroll
    for (int j = 0; j < 8; j++)
      *reinterpret_cast<float2*>(&s_tmp[(8 * g + j) * IW + ix]) = make_float2(a0[j], a1[j]);
  }
  __syncthreads();
  // Row pass (8 consecutive outputs per item) and store.
  float local_min = kInf;
  for (int item = threadIdx.x; item < TH * (TW / 8); item += blockDim.x) {
    const int y = item / (TW / 8), g = item - y * (TW / 8);
    const int gy = y0 + y;
    typename Epi::Pre pre[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int gx = x0 + 8 * g + j;
      if (gy < H && gx < W) pre[j] = epi.pre((int64_t)gy * W + gx);
    }
    float acc[8];
    conv_line8<LC>(s_tmp + y * IW + 8 * g, 1, s_taps, L, acc);
    if (gy >= H) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int gx = x0 + 8 * g + j;
      if (gx < W) local_min = fminf(local_min, epi((int64_t)gy * W + gx, gx, gy, acc[j], pre[j]));
    }
  }
  block_min_out(local_min, epi);
}

// ---- A3 full 2D (exponential) -----------------------------------------------
// A block computes a 64 x 32 tile; a thread 8 consecutive outputs of one row
// from a sliding window of 8 registers, so each tap costs one shared-memory
// load of input (and a broadcast load of the tap) per 8 outputs.  Each
// output's sum runs over the filter rows, and inside a row over its taps,
// in ascending order, as the reference's 2D loop does.
constexpr int kTwoDTW = 64, kTwoDTH = 32, kTwoDThreads = 256;

template <class Epi>
__global__ void __launch_bounds__(kTwoDThreads)
conv_2d_kernel(const float* __restrict__ in, int W, int H,
               const float* __restrict__ filt, int r, Epi epi) {
  extern __shared__ float sm[];
  const int L = 2 * r + 1;
  const int IW = kTwoDTW + 2 * r, IH = kTwoDTH + 2 * r;
  float* s_f = sm;
  float* s_in = sm + ((L * L + 3) & ~3);
  const int x0 = blockIdx.x * kTwoDTW, y0 = blockIdx.y * kTwoDTH;
  for (int t = threadIdx.x; t < L * L; t += blockDim.x) s_f[t] = filt[t];
  {
    int iy = threadIdx.x / IW, ix = threadIdx.x - iy * IW;
    const int dy = blockDim.x / IW, dx = blockDim.x - dy * IW;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < IW * IH; idx += blockDim.x) {
      const int gy = wrap_idx(y0 - r + iy, H), gx = wrap_idx(x0 - r + ix, W);
      cp_async4(&s_in[idx], &in[(int64_t)gy * W + gx]);  // all of them in flight at once
      iy += dy;
      ix += dx;
      if (ix >= IW) {
        ix -= IW;
        iy++;
      }
    }
    cp_async_wait();
  }
  __syncthreads();
  const int ox = 8 * (threadIdx.x & 7), ty = threadIdx.x >> 3;
  const int gy = y0 + ty;
  typename Epi::Pre pre[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int gx = x0 + ox + j;
    if (gy < H && gx < W) pre[j] = epi.pre((int64_t)gy * W + gx);
  }
  float acc[8];
#pragma unroll
  for (int j = 0; j < 8; j++) acc[j] = 0.0f;
  for (int fy = 0; fy < L; fy++) {
    const float* row = s_in + (ty + fy) * IW + ox;
    const float* frow = s_f + fy * L;
    float win[8];
#pragma unroll
    for (int j = 0; j < 8; j++) win[j] = row[j];
#pragma unroll 8
    for (int fx = 0; fx < L; fx++) {
      const float f = frow[fx];
#pragma unroll
      for (int j = 0; j < 8; j += 2) muladd2_rn(acc[j], acc[j + 1], win[j], win[j + 1], f);
#pragma unroll
      for (int j = 0; j < 7; j++) win[j] = win[j + 1];
      win[7] = (fx + 1 < L) ? row[fx + 8] : 0.0f;
    }
  }
  float local_min = kInf;
  if (gy < H) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int gx = x0 + ox + j;
      if (gx < W) local_min = fminf(local_min, epi((int64_t)gy * W + gx, gx, gy, acc[j], pre[j]));
    }
  }
  block_min_out(local_min, epi);
}

size_t conv_smem_bytes(int model, int r, int tile) {
  int L = 2 * r + 1;
  if (model == CAGEO_FILTER_GAUSSIAN) {
    const SepTile t = kSepTiles[tile];
    int IW = t.tw + 2 * r, IH = t.th + 2 * r;
    return sizeof(float) * (((L + 3) & ~3) + (size_t)IW * IH + (size_t)IW * t.th);
  }
  int IW = kTwoDTW + 2 * r, IH = kTwoDTH + 2 * r;
  return sizeof(float) * (((L * L + 3) & ~3) + (size_t)IW * IH);
}

// Whether a tile shape of the fused front applies: Gaussian filters (the
// separable kernel) whose staged block fits the device's shared memory.
bool conv_tile_applies(int model, int r, int tile) {
  if (model != CAGEO_FILTER_GAUSSIAN || tile < 0 || tile >= kConvTiles) return tile == 0;
  int optin = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return tile == 0;
  // The kernels' own static shared memory (the block minimum) is small.
  return conv_smem_bytes(model, r, tile) + 1024 <= (size_t)optin;
}

// The separable kernel for a tile shape and radius: fully unrolled for the
// 60 m and 90 m ranges at 10 m cells (radius 15 and 23).
template <class Epi>
using SepKernel = void (*)(const float*, int, int, const float*, int, Epi);

template <class Epi, int TW, int TH>
SepKernel<Epi> sep_kernel_for(int r) {
  return r == 15 ? conv_sep_kernel<Epi, 31, TW, TH>
                 : r == 23 ? conv_sep_kernel<Epi, 47, TW, TH> : conv_sep_kernel<Epi, 0, TW, TH>;
}

template <class Epi>
SepKernel<Epi> sep_kernel(int r, int tile) {
  if constexpr (std::is_same<Epi, FrontEpilogue>::value) {
    switch (tile) {
      case 1: return sep_kernel_for<Epi, kSepTiles[1].tw, kSepTiles[1].th>(r);
      case 2: return sep_kernel_for<Epi, kSepTiles[2].tw, kSepTiles[2].th>(r);
      case 3: return sep_kernel_for<Epi, kSepTiles[3].tw, kSepTiles[3].th>(r);
      default: break;
    }
  }
  return sep_kernel_for<Epi, kSepTiles[0].tw, kSepTiles[0].th>(r);
}

template <class Epi>
cageo_status launch_conv(const float* in, int W, int H, int model,
                         const float* filt, int r, const Epi& epi,
                         cudaStream_t s, int tile = 0) {
  if (!std::is_same<Epi, FrontEpilogue>::value || tile < 0 || tile >= kConvTiles) tile = 0;
  // The kernels' dynamic shared-memory limit is raised to the most the
  // device allows (its opt-in maximum less the kernel's static shared
  // memory), the same value on every call: pipelines on other host threads
  // launch the same kernels with other radii, and a per-call limit set by
  // one thread could fall below another thread's launch between its set
  // and launch.  (Occupancy follows each launch's own size, not the limit.)
  int optin = 0, dev = 0;
  CAGEO_CUDA(cudaGetDevice(&dev));
  CAGEO_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  auto raise_limit = [&](const void* fn, int* limit) -> cageo_status {
    cudaFuncAttributes fa;
    CAGEO_CUDA(cudaFuncGetAttributes(&fa, fn));
    *limit = optin - (int)fa.sharedSizeBytes;
    CAGEO_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, *limit));
    return CAGEO_OK;
  };
  const size_t smem = conv_smem_bytes(model, r, tile);
  if (model == CAGEO_FILTER_GAUSSIAN) {
    const SepKernel<Epi> fn = sep_kernel<Epi>(r, tile);
    int limit = 0;
    cageo_status st = raise_limit((const void*)fn, &limit);
    if (st) return st;
    if (smem > (size_t)limit) {
      set_error("filter radius %d needs %zu bytes of shared memory (%d available)", r, smem, limit);
      return CAGEO_ERR_ARGUMENT;
    }
    const SepTile t = kSepTiles[tile];
    dim3 grid((W + t.tw - 1) / t.tw, (H + t.th - 1) / t.th);
    fn<<<grid, kSepThreads, smem, s>>>(in, W, H, filt, r, epi);
  } else {
    int limit = 0;
    cageo_status st = raise_limit((const void*)conv_2d_kernel<Epi>, &limit);
    if (st) return st;
    if (smem > (size_t)limit) {
      set_error("filter radius %d needs %zu bytes of shared memory (%d available)", r, smem, limit);
      return CAGEO_ERR_ARGUMENT;
    }
    dim3 grid((W + kTwoDTW - 1) / kTwoDTW, (H + kTwoDTH - 1) / kTwoDTH);
    conv_2d_kernel<Epi><<<grid, kTwoDThreads, smem, s>>>(in, W, H, filt, r, epi);
  }
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status launch_noise(float* d, int64_t n, uint64_t seed, uint32_t realization,
                          const uint32_t* dreal, float mean, float sd, cudaStream_t s) {
  int64_t groups = (n + 3) / 4;
  int threads = 256;
  int64_t blocks = (groups + threads - 1) / threads;
  noise_kernel<<<(unsigned)blocks, threads, 0, s>>>(d, n, (uint32_t)seed,
                                                    (uint32_t)(seed >> 32), realization,
                                                    dreal, mean, sd);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status launch_front(const float* noise, int W, int H, int model,
                          const float* filt, int r, const FrontParams& fp,
                          cudaStream_t s, int tile) {
  FrontEpilogue e{fp};
  return launch_conv(noise, W, H, model, filt, r, e, s, tile);
}

}  // namespace cageo

using namespace cageo;

extern "C" cageo_status cageo_noise_philox(float* d_field, int W, int H,
                                           uint64_t seed, uint32_t realization,
                                           float mean, float stddev,
                                           cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_field && valid_dims(W, H), "field pointer and size");
  return launch_noise(d_field, (int64_t)W * H, seed, realization, nullptr, mean, stddev,
                      stream);
}

// Raw Philox4x32-10 blocks: block i is philox4x32_10((c0 + i, c1, c2, c3),
// (k0, k1)), the generator noise_kernel draws from.
__global__ void philox_bits_kernel(uint32_t* __restrict__ out, int64_t n, U4 c, uint32_t k0,
                                   uint32_t k1) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  U4 ci = c;
  ci.x += (uint32_t)i;
  const U4 r = philox4x32_10(ci, k0, k1);
  out[4 * i] = r.x;
  out[4 * i + 1] = r.y;
  out[4 * i + 2] = r.z;
  out[4 * i + 3] = r.w;
}

extern "C" cageo_status cageo_philox4x32_10(uint32_t* d_out, int64_t n, const uint32_t* h_ctr,
                                            const uint32_t* h_key, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_out && h_ctr && h_key && n > 0 && n < ((int64_t)1 << 31),
                  "pointers and block count");
  const U4 c = {h_ctr[0], h_ctr[1], h_ctr[2], h_ctr[3]};
  philox_bits_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(d_out, n, c, h_key[0],
                                                                      h_key[1]);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

extern "C" cageo_status cageo_convolve(const float* d_in, float* d_out, int W,
                                       int H, int model, const float* d_filter,
                                       int radius, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_in && d_out && d_filter && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(d_in != d_out, "convolution cannot run in place");
  CAGEO_CHECK_ARG(model == CAGEO_FILTER_GAUSSIAN || model == CAGEO_FILTER_EXPONENTIAL,
                  "filter model");
  CAGEO_CHECK_ARG(radius >= 0 && radius < W && radius < H,
                  "filter radius must be below the grid width and height");
  StoreEpilogue e{d_out};
  return launch_conv(d_in, W, H, model, d_filter, radius, e, stream);
}
