// routing.cu -- A7 D8 flow routing with the reference CPU path's rules
// (src/flowrouting/FlowRoutingAlgorithmCPUOpenMP.h:53-249).
//
// First pass, one thread per cell: border cells point outward (corners
// diagonally), cells equal to 0 are streams (flatDist -2, no direction),
// others take the steepest strictly-descending neighbour in N, NE, E, SE, S,
// SW, W, NW order with diagonal drops divided by 1.41421356f, the first
// maximum winning.  Cells with no descending neighbour are flat.
//
// Flats: the reference assigns layer k = 1, 2, ... to flat cells that have a
// neighbour in layer k-1 (layer 0 = cells with a direction, flatDist -1)
// whose elevation is <= theirs, taking the direction of the LAST such
// neighbour in N..NW order.  Layer numbers are breadth-first distances, so
// they are computed here by a frontier BFS (one grid-wide barrier per
// layer, persistent cooperative kernel) and the directions by one final
// pass that applies the last-match rule to the finished distances.
#include <algorithm>
#include "common.cuh"
#include "routing.cuh"
#include "stage_math.cuh"

namespace cageo {

constexpr int kFlatInf = 0x3fffffff;
enum : int { R_NFLAT = 0, R_ERR = 3, R_CNT = 4, R_LAYERS = 7, R_US_BFS = 8, R_BAR_COUNT = kBarCountSlot,
             R_BAR_GEN = kBarGenSlot, R_SIZE = kScalarSlots };
constexpr int kBfsThreads = 512;

size_t route_workspace_bytes(int W, int H) {
  size_t n = (size_t)W * H;
  return 3 * align_up(n * 4, 256) + 512;
}

RouteWork route_carve(void* base, int W, int H) {
  RouteWork w;
  w.W = W;
  w.H = H;
  size_t n = (size_t)W * H;
  char* p = (char*)base;
  w.flats = (uint32_t*)p;
  p += align_up(n * 4, 256);
  w.front = (uint32_t*)p;
  p += 2 * align_up(n * 4, 256);
  w.scal = (unsigned int*)p;
  return w;
}

// Steepest-descent pass.  flatdist: -1 direction, -2 stream, kFlatInf flat.
__global__ void d8_kernel(const float* __restrict__ dem, char2* __restrict__ dir,
                          int* __restrict__ fd, RouteWork w) {
  const int W = w.W, H = w.H;
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  int64_t i = (int64_t)y * W + x;
  int dxi = 0, dyi = 0;
  if (x == 0) dxi = -1; else if (x == W - 1) dxi = 1;
  if (y == 0) dyi = -1; else if (y == H - 1) dyi = 1;
  if (dxi || dyi) {
    dir[i] = make_char2((signed char)dxi, (signed char)dyi);
    fd[i] = -1;
    return;
  }
  const float c = dem[i];
  if (c == 0.0f) {
    dir[i] = make_char2(0, 0);
    fd[i] = -2;
    return;
  }
  float steepest = 0.0f;
  int sdx = 0, sdy = 0;
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int dx = d8_dx(n), dy = d8_dy(n);
    float s = __fsub_rn(c, dem[(int64_t)(y + dy) * W + (x + dx)]);
    if (s > 0.0f) {
      if (n & 1) s = __fdiv_rn(s, 1.41421356237309505f);
      if (s > steepest) { steepest = s; sdx = dx; sdy = dy; }
    }
  }
  if (steepest > 0.0f) {
    dir[i] = make_char2((signed char)sdx, (signed char)sdy);
    fd[i] = -1;
  } else {
    dir[i] = make_char2(0, 0);
    fd[i] = kFlatInf;
    unsigned int pos = atomicAdd(&w.scal[R_NFLAT], 1u);
    w.flats[pos] = (uint32_t)i;
  }
}

// Layer 1: flat cells next to a cell with a direction (flatDist -1) whose
// elevation is <= theirs.
__global__ void flat_seed_kernel(const float* __restrict__ dem, int* __restrict__ fd,
                                 RouteWork w) {
  const unsigned int nf = w.scal[R_NFLAT];
  const int W = w.W, H = w.H;
  for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf;
       j += gridDim.x * blockDim.x) {
    uint32_t c = w.flats[j];
    int x = (int)(c % (uint32_t)W), y = (int)(c / (uint32_t)W);
    const float e = dem[c];
    bool seed = false;
    for (int n = 0; n < 8 && !seed; n++) {
      int nx = x + d8_dx(n), ny = y + d8_dy(n);
      if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
      int64_t ni = (int64_t)ny * W + nx;
      seed = fd[ni] == -1 && dem[ni] <= e;
    }
    if (seed) {
      // Distances are written after the scan of every flat cell (next kernel)
      // so that no cell of this kernel sees another's layer-1 mark.
      unsigned int pos = atomicAdd(&w.scal[R_CNT + 1], 1u);
      w.front[(size_t)1 * W * H + pos] = c;
    }
  }
}

__global__ void flat_mark_kernel(int* __restrict__ fd, RouteWork w) {
  const unsigned int n1 = w.scal[R_CNT + 1];
  const int64_t N = (int64_t)w.W * w.H;
  for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < n1;
       j += gridDim.x * blockDim.x)
    fd[w.front[N + j]] = 1;
}

// Frontier BFS: layer k -> k+1 over flat cells with elevation >= the
// frontier cell's.  Persistent, one bounded grid barrier per layer.
__global__ void __launch_bounds__(kBfsThreads)
flat_bfs_kernel(const float* __restrict__ dem, int* __restrict__ fd, RouteWork w) {
  const int W = w.W, H = w.H;
  const int64_t N = (int64_t)W * H;
  GridSync gs{w.scal + R_BAR_COUNT, w.scal + R_BAR_GEN, (int*)(w.scal + R_ERR)};
  volatile unsigned int* vs = w.scal;
  int k = 1;
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  while (true) {
    if (blockIdx.x == 0 && threadIdx.x == 0) vs[R_CNT + (k + 2) % 3] = 0u;
    const unsigned int n = vs[R_CNT + k % 3];
    const uint32_t* cur = w.front + (size_t)(k & 1) * N;
    uint32_t* nxt = w.front + (size_t)((k + 1) & 1) * N;
    for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += gridDim.x * blockDim.x) {
      uint32_t c = cur[j];
      int x = (int)(c % (uint32_t)W), y = (int)(c / (uint32_t)W);
      const float e = dem[c];
      for (int q = 0; q < 8; q++) {
        int nx = x + d8_dx(q), ny = y + d8_dy(q);
        if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
        int64_t ni = (int64_t)ny * W + nx;
        if (fd[ni] == kFlatInf && e <= dem[ni] &&
            atomicCAS(&fd[ni], kFlatInf, k + 1) == kFlatInf) {
          unsigned int pos = atomicAdd(&w.scal[R_CNT + (k + 1) % 3], 1u);
          nxt[pos] = (uint32_t)ni;
        }
      }
    }
    if (!grid_barrier(gs, gridDim.x)) break;
    if (vs[R_CNT + (k + 1) % 3] == 0u) break;
    if (k > 1 << 28) {
      if (threadIdx.x == 0) atomicCAS((int*)(w.scal + R_ERR), 0, 2);
      break;
    }
    k++;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    vs[R_LAYERS] = (unsigned int)k;
    vs[R_US_BFS] = (unsigned int)((t1 - t0) / 1000);
  }
}

// Directions of flat cells: last neighbour (N..NW) in the previous layer
// (or with flatDist -1 for layer 1) whose elevation is <= the cell's.
__global__ void flat_dir_kernel(const float* __restrict__ dem, char2* __restrict__ dir,
                                int* __restrict__ fd, RouteWork w) {
  const unsigned int nf = w.scal[R_NFLAT];
  const int W = w.W, H = w.H;
  for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf;
       j += gridDim.x * blockDim.x) {
    uint32_t c = w.flats[j];
    int d = fd[c];
    if (d == kFlatInf) continue;
    int x = (int)(c % (uint32_t)W), y = (int)(c / (uint32_t)W);
    const float e = dem[c];
    const int want = d == 1 ? -1 : d - 1;
    int got = -1;
    for (int n = 0; n < 8; n++) {
      int nx = x + d8_dx(n), ny = y + d8_dy(n);
      if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
      int64_t ni = (int64_t)ny * W + nx;
      if (fd[ni] == want && dem[ni] <= e) got = n;
    }
    if (got >= 0) dir[c] = make_char2((signed char)d8_dx(got), (signed char)d8_dy(got));
  }
}

// Unresolved flats end as flatDist 0 with no direction.
__global__ void flat_final_kernel(int* __restrict__ fd, RouteWork w) {
  const unsigned int nf = w.scal[R_NFLAT];
  for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf;
       j += gridDim.x * blockDim.x) {
    uint32_t c = w.flats[j];
    if (fd[c] == kFlatInf) fd[c] = 0;
  }
}

__global__ void route_scalars_kernel(unsigned int* s) {
  for (int i = threadIdx.x; i < R_SIZE; i += blockDim.x) s[i] = 0u;
}

static int coop_blocks_bfs() {
  static int blocks = 0;
  if (!blocks) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, flat_bfs_kernel, kBfsThreads, 0);
    blocks = std::max(1, std::min(per, 2)) * sms;
  }
  return blocks;
}

cageo_status route_run(const float* filled, int8_t* dir, int* fd, const RouteWork& w,
                       cudaStream_t s) {
  route_scalars_kernel<<<1, 128, 0, s>>>(w.scal);
  dim3 b(32, 8), g((w.W + 31) / 32, (w.H + 7) / 8);
  d8_kernel<<<g, b, 0, s>>>(filled, (char2*)dir, fd, w);
  CAGEO_CUDA(cudaGetLastError());
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned lb = (unsigned)sms * 8;
  flat_seed_kernel<<<lb, 256, 0, s>>>(filled, fd, w);
  flat_mark_kernel<<<lb, 256, 0, s>>>(fd, w);
  CAGEO_CUDA(cudaGetLastError());
  const float* f = filled;
  int* fdp = fd;
  RouteWork wc = w;
  void* params[] = {(void*)&f, (void*)&fdp, (void*)&wc};
  CAGEO_CUDA(cudaLaunchCooperativeKernel((const void*)flat_bfs_kernel, dim3(coop_blocks_bfs()),
                                         dim3(kBfsThreads), params, 0, s));
  flat_dir_kernel<<<lb, 256, 0, s>>>(filled, (char2*)dir, fd, w);
  flat_final_kernel<<<lb, 256, 0, s>>>(fd, w);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status route_check_status(const RouteWork& w, int64_t* stats) {
  unsigned int h[R_SIZE];
  CAGEO_CUDA(cudaMemcpy(h, w.scal, sizeof(h), cudaMemcpyDeviceToHost));
  if (stats) {
    stats[0] = h[R_LAYERS];
    stats[1] = h[R_NFLAT];
    stats[2] = h[R_US_BFS];
  }
  if (h[R_ERR]) {
    set_error("flow routing: flat-surface BFS hit a wait or layer limit");
    return CAGEO_ERR_NO_CONVERGENCE;
  }
  return CAGEO_OK;
}

}  // namespace cageo

using namespace cageo;

extern "C" size_t cageo_route_workspace_size(int W, int H) {
  if (!valid_dims(W, H)) return 0;
  return route_workspace_bytes(W, H) + align_up((size_t)W * H * 4, 256);
}

extern "C" cageo_status cageo_route_d8(const float* d_filled, int8_t* d_dir,
                                       int* d_flatdist, int W, int H, void* d_workspace,
                                       size_t workspace_bytes, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_filled && d_dir && valid_dims(W, H), "pointers and size");
  Scratch ws;
  cageo_status st = ws.acquire(d_workspace, workspace_bytes,
                               cageo_route_workspace_size(W, H), stream);
  if (st) return st;
  RouteWork w = route_carve(ws.ptr, W, H);
  int* fd = d_flatdist ? d_flatdist
                       : (int*)((char*)ws.ptr + route_workspace_bytes(W, H));
  if ((st = route_run(d_filled, d_dir, fd, w, stream))) return st;
  CAGEO_CUDA(cudaStreamSynchronize(stream));
  return route_check_status(w, nullptr);
}
