// trace_border.cu -- A8 flow tracing by pointer jumping and A9 catchment
// border extraction + Monte Carlo accumulation.
//
// Tracing (src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:34-134): a stream
// cell (streams >= 0) is LAKE; every other cell follows its direction until
// it leaves the grid (OUTSIDE) or steps onto a stream cell s (label
// (int)(-streams[s])).  The reference walks each path serially with caching;
// the label of a cell depends only on where its path ends, so here every
// cell holds a packed 32-bit state -- "points to cell p" or "resolved to
// label l".  Paths are first followed inside each 32x32 tile; a path that
// leaves its tile then points at the border cell of the next tile it
// enters, and those border cells (124 per tile, kept in a compact array)
// point only at border cells of other tiles.  Pointer doubling
// (p <- state[p]) over the compact array resolves them in O(log path
// length) passes over 12% of the cells; every other cell then needs one
// lookup.  A cell without a direction
// (0,0) is a dead end: the reference's walk never terminates there, leaves
// the path at 0 and its connect pass then copies the label of cell 0; such
// cells and label-0 terminals take the label of cell 0 here too (or, in the
// dead-end-error mode used with the GPU path's semantics, dead ends and the
// cells draining into them are ERROR).  (The
// reference also abandons walks longer than 100000 steps; paths of that
// length do not occur in these grids and are not modelled.)
//
// Border (src/catchmentborder/CatchmentBorderAlgorithmCPUOpenMP.h:30-82):
// border = 1 where the label is not LAKE and some N8 neighbour has a larger
// label that is not LAKE; the count grid adds it
// (src/catchmentborder/CatchmentBorderAlgorithm.h:53-74).
#include <algorithm>
#include "common.cuh"
#include "routing.cuh"
#include "stage_math.cuh"

namespace cageo {

// Packed per-cell state (int32): >= 0 points to a cell; < 0 is resolved,
// holding code(label) = label - 1 (labels are <= 0, so label 0 stays
// negative); kStuckCode marks a dead end.  Stream values whose negation
// does not fit (|streams| >= 2^31 - 1) are outside the supported range.
constexpr int kStuckCode = (int)0x80000000;
constexpr int kJumpThreads = 256;
enum : int { T_ERR = 2, T_ACTIVE = 3, T_JUMPS = 6, T_BAR_COUNT = kBarCountSlot,
             T_BAR_GEN = kBarGenSlot, T_SIZE = kScalarSlots };

__device__ __forceinline__ int label_code(int label) { return label - 1; }

constexpr int kBorderCells = 124;  // cells on the rim of a 32x32 tile

size_t trace_workspace_bytes(int W, int H) {
  const size_t n = (size_t)W * H;
  const size_t nt = (size_t)((W + 31) / 32) * ((H + 31) / 32);
  return align_up(n * 4, 256) + align_up(nt * kBorderCells * 4, 256) + 512;
}

TraceWork trace_carve(void* base, int W, int H) {
  TraceWork w;
  w.W = W;
  w.H = H;
  w.tiles_x = (W + 31) / 32;
  w.tiles_y = (H + 31) / 32;
  const size_t n = (size_t)W * H;
  const size_t nt = (size_t)w.tiles_x * w.tiles_y;
  char* p = (char*)base;
  w.state = (int*)p;
  p += align_up(n * 4, 256);
  w.bstate = (int*)p;
  p += align_up(nt * kBorderCells * 4, 256);
  w.scal = (unsigned int*)p;
  return w;
}

// Compact index of cell (x, y) on the rim of its 32x32 tile (x % 32 or
// y % 32 is 0 or 31): top row 0..31, bottom row 32..63, left column rows
// 1..30 at 64..93, right column rows 1..30 at 94..123.
__device__ __forceinline__ int border_index(int x, int y, int tiles_x) {
  const int lx = x & 31, ly = y & 31;
  const int b = ly == 0 ? lx : ly == 31 ? 32 + lx : lx == 0 ? 63 + ly : 93 + ly;
  return ((y >> 5) * tiles_x + (x >> 5)) * kBorderCells + b;
}

// Initial state of every cell, then pointer jumping inside its 32x32 tile
// in shared memory: each cell ends resolved (a label or a dead end) or
// pointing at the first cell of its path outside the tile, so the global
// jumps hop from tile to tile.  One thread per cell, one block per tile.
__global__ void __launch_bounds__(256) trace_init_kernel(const char2* __restrict__ dir,
                                                        const float* __restrict__ streams,
                                                        int* __restrict__ st,
                                                        int* __restrict__ bst, int W, int H,
                                                        unsigned int* scal) {
  __shared__ int gs[32 * 32];    // state once the path has left the tile (or resolved)
  __shared__ short lt[32 * 32];  // next cell of the path inside the tile, -1 otherwise
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  int s[4], t[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {  // cell li = threadIdx.x + 256 k: row li / 32, column li % 32
    const int li = threadIdx.x + 256 * k, tx = li & 31, ty = li >> 5;
    const int x = x0 + tx, y = y0 + ty;
    s[k] = kStuckCode;
    t[k] = -1;
    if (x < W && y < H) {
      const int64_t i = (int64_t)y * W + x;
      const char2 d = dir[i];
      const int nx = x + d.x, ny = y + d.y;
      if (streams[i] >= 0.0f) s[k] = label_code(kLake);
      else if (nx < 0 || nx >= W || ny < 0 || ny >= H) s[k] = label_code(kOutside);
      else if (d.x == 0 && d.y == 0) s[k] = kStuckCode;
      else {
        const int64_t n = (int64_t)ny * W + nx;
        const float sn = streams[n];
        if (sn >= 0.0f) {
          s[k] = label_code((int)(-sn));
        } else {
          const int lx = tx + d.x, ly = ty + d.y;
          if (lx >= 0 && lx < 32 && ly >= 0 && ly < 32) {
            t[k] = ly * 32 + lx;  // inside the tile: followed below
            s[k] = 0;
          } else {
            s[k] = border_index(nx, ny, gridDim.x);  // on the rim of the next tile
          }
        }
      }
    }
    gs[li] = s[k];
    lt[li] = (short)t[k];
  }
  __syncthreads();
  for (int it = 0; it < 10; it++) {  // 2^10 cells: every path inside a tile
    int ns[4], nt[4];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      ns[k] = s[k];
      nt[k] = t[k];
      if (t[k] >= 0) {
        ns[k] = gs[t[k]];
        nt[k] = lt[t[k]];
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (t[k] >= 0) {
        const int li = threadIdx.x + 256 * k;
        s[k] = ns[k];
        t[k] = nt[k];
        gs[li] = s[k];
        lt[li] = (short)t[k];
      }
      any |= t[k] >= 0;
    }
    if (!__syncthreads_or(any)) break;
  }
  // A path of a 32x32 tile has at most 1024 cells: one still inside after
  // 2^10 hops is on a cycle, which never resolves (reported as an error).
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (t[k] >= 0) {
      s[k] = kStuckCode;
      atomicCAS((int*)(scal + T_ERR), 0, 2);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int li = threadIdx.x + 256 * k, lx = li & 31, ly = li >> 5;
    const int x = x0 + lx, y = y0 + ly;
    if (x < W && y < H) st[(int64_t)y * W + x] = s[k];
    if (lx == 0 || lx == 31 || ly == 0 || ly == 31) bst[border_index(x, y, gridDim.x)] = s[k];
  }
}

// Pointer doubling in place over the tiles' border cells (reading a
// neighbour's newer state only speeds convergence).  Each thread takes 4 cells per iteration so their dependent
// load pairs overlap.  Persistent; one bounded grid barrier per pass.
__global__ void __launch_bounds__(kJumpThreads, 8) trace_jump_kernel(int* st, TraceWork w) {
  const int64_t N = (int64_t)w.tiles_x * w.tiles_y * kBorderCells;
  GridSync gs{w.scal + T_BAR_COUNT, w.scal + T_BAR_GEN, (int*)(w.scal + T_ERR)};
  volatile unsigned int* vs = w.scal;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int pass = 0;
  while (true) {
    // Slot pass%3 is written during this pass and read after its barrier;
    // slot (pass+1)%3 was last read before the previous barrier.
    if (blockIdx.x == 0 && threadIdx.x == 0) vs[T_ACTIVE + (pass + 1) % 3] = 0u;
    bool active = false;
    for (int64_t base = tid; base < N; base += 4 * nthreads) {
      int s[4], t[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int64_t i = base + k * nthreads;
        s[k] = i < N ? st[i] : -1;
      }
#pragma unroll
      for (int k = 0; k < 4; k++) t[k] = s[k] >= 0 ? ((volatile int*)st)[s[k]] : s[k];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (s[k] >= 0) {
          st[base + k * nthreads] = t[k];
          active |= t[k] >= 0;
        }
      }
    }
    // One flag update per block: same-address atomics from every warp would
    // queue up at the memory system.
    if (__syncthreads_or(active) && threadIdx.x == 0) atomicOr(&w.scal[T_ACTIVE + pass % 3], 1u);
    if (!grid_barrier(gs, gridDim.x)) break;
    if (vs[T_ACTIVE + pass % 3] == 0u) break;
    if (++pass > 64) {  // 2^64 exceeds any path length: a cycle
      if (threadIdx.x == 0) atomicCAS((int*)(w.scal + T_ERR), 0, 2);
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) vs[T_JUMPS] = (unsigned int)(pass + 1);
}

// Label of a resolved state c (cell 0's state c0): label-0 terminals take
// cell 0's label, and so do dead ends (stuck = 0) unless they are reported
// as ERROR (stuck = kError).
__device__ __forceinline__ int decode_label(int c, int c0, int stuck) {
  int l = c == kStuckCode ? stuck : c + 1;
  if (l >= 0) {
    const int l0 = c0 == kStuckCode ? stuck : c0 + 1;
    l = l0 >= 0 ? 0 : l0;
  }
  return l;
}

// Resolved state of a cell from its own state: a path that left the cell's
// tile takes the (resolved) state of the border cell it entered next.
__device__ __forceinline__ int resolve(int c, const int* __restrict__ bst) {
  return c >= 0 ? bst[c] : c;
}

__global__ void trace_final_kernel(const int* __restrict__ st, const int* __restrict__ bst,
                                   int* __restrict__ label, int64_t n, int stuck) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  label[i] = decode_label(resolve(st[i], bst), resolve(st[0], bst), stuck);
}

__global__ void trace_scalars_kernel(unsigned int* s) {
  for (int i = threadIdx.x; i < T_SIZE; i += blockDim.x) s[i] = 0u;
}

cageo_status trace_run(const int8_t* dir, const float* streams, int* label,
                       const TraceWork& w, cudaStream_t s, int mode, bool write_labels) {
  const int64_t n = (int64_t)w.W * w.H;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  trace_scalars_kernel<<<1, 128, 0, s>>>(w.scal);
  trace_init_kernel<<<dim3(w.tiles_x, w.tiles_y), 256, 0, s>>>(
      (const char2*)dir, streams, w.state, w.bstate, w.W, w.H, w.scal);
  CAGEO_CUDA(cudaGetLastError());
  static PerDevice resident;
  int coop = 0;
  cageo_status st = per_device(resident, &coop, [&](int dev, int* v) -> cageo_status {
    return resident_blocks((const void*)trace_jump_kernel, kJumpThreads, 0, dev, v);
  });
  if (st) return st;
  int* stp = w.bstate;
  TraceWork wc = w;
  void* params[] = {(void*)&stp, (void*)&wc};
  // Each thread takes 4 border cells per iteration: no more blocks than
  // that covers.
  const int64_t nb = (int64_t)w.tiles_x * w.tiles_y * kBorderCells;
  const int64_t need = (nb + 4 * kJumpThreads - 1) / (4 * kJumpThreads);
  const int jgrid = (int)std::max<int64_t>(1, std::min<int64_t>(coop, need));
  CAGEO_CUDA(cudaLaunchCooperativeKernel((const void*)trace_jump_kernel, dim3(jgrid),
                                         dim3(kJumpThreads), params, 0, s));
  if (write_labels)
    trace_final_kernel<<<blocks, 256, 0, s>>>(w.state, w.bstate, label, n,
                                              mode == CAGEO_TRACE_DEAD_END_ERROR ? kError : 0);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status trace_check_status(const TraceWork& w, int64_t* jumps) {
  unsigned int h[T_SIZE];
  CAGEO_CUDA(cudaMemcpy(h, w.scal, sizeof(h), cudaMemcpyDeviceToHost));
  if (jumps) *jumps = h[T_JUMPS];
  if (h[T_ERR]) {
    set_error("flow tracing: pointer jumping hit a wait or pass limit");
    return CAGEO_ERR_NO_CONVERGENCE;
  }
  return CAGEO_OK;
}

// ---- A9 -------------------------------------------------------------------
// One 32x32 tile per block: the labels of the tile and a one-cell halo are
// staged in shared memory (cells outside the grid read as LAKE, which never
// makes a border), then each thread tests 4 cells.  `gate` (may be null):
// a flag that, when set, skips the accumulation for this realization.
template <typename T>
__global__ void __launch_bounds__(256) border_kernel(const int* __restrict__ label,
                                                     T* __restrict__ count, int W, int H,
                                                     const int* __restrict__ gate) {
  if (gate && *gate) return;
  __shared__ int L[34 * 35];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  for (int k = threadIdx.y * 32 + threadIdx.x; k < 34 * 34; k += 256) {
    const int hy = k / 34, hx = k - hy * 34;
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
    L[hy * 35 + hx] =
        (gx >= 0 && gx < W && gy >= 0 && gy < H) ? label[(int64_t)gy * W + gx] : kLake;
  }
  __syncthreads();
  const int tx = threadIdx.x, x = x0 + tx;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int ty = threadIdx.y + 8 * k, y = y0 + ty;
    if (x >= W || y >= H) continue;
    const int* c = &L[(ty + 1) * 35 + tx + 1];
    if (*c == kLake) continue;
    bool border = false;
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int v = c[d8_dy(n) * 35 + d8_dx(n)];
      border |= *c < v && v != kLake;
    }
    if (border) {
      const int64_t i = (int64_t)y * W + x;
      count[i] = count[i] + (T)1;
    }
  }
}

// The same from the resolved trace states: decodes the labels of the tile
// and halo (writing the tile's own into `label`), so the labels need no
// pass of their own.  The labels are written even when `gate` skips the
// accumulation.
__global__ void __launch_bounds__(256) border_state_kernel(const int* __restrict__ st,
                                                           const int* __restrict__ bst,
                                                           int* __restrict__ label,
                                                           uint32_t* __restrict__ count, int W,
                                                           int H, const int* __restrict__ gate,
                                                           int stuck) {
  __shared__ int L[34 * 35];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  const int c0 = resolve(st[0], bst);
  for (int k = threadIdx.y * 32 + threadIdx.x; k < 34 * 34; k += 256) {
    const int hy = k / 34, hx = k - hy * 34;
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
    L[hy * 35 + hx] = (gx >= 0 && gx < W && gy >= 0 && gy < H)
                          ? decode_label(resolve(st[(int64_t)gy * W + gx], bst), c0, stuck)
                          : kLake;
  }
  __syncthreads();
  const bool skip = gate && *gate;
  const int tx = threadIdx.x, x = x0 + tx;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int ty = threadIdx.y + 8 * k, y = y0 + ty;
    if (x >= W || y >= H) continue;
    const int64_t i = (int64_t)y * W + x;
    const int* c = &L[(ty + 1) * 35 + tx + 1];
    label[i] = *c;
    if (skip || *c == kLake) continue;
    bool border = false;
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int v = c[d8_dy(n) * 35 + d8_dx(n)];
      border |= *c < v && v != kLake;
    }
    if (border) count[i] += 1u;
  }
}

cageo_status border_u32_from_state(const TraceWork& w, int* label, uint32_t* count,
                                   const int* gate, int mode, cudaStream_t s) {
  dim3 b(32, 8), g(w.tiles_x, w.tiles_y);
  border_state_kernel<<<g, b, 0, s>>>(w.state, w.bstate, label, count, w.W, w.H, gate,
                                      mode == CAGEO_TRACE_DEAD_END_ERROR ? kError : 0);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

template <typename T>
static cageo_status launch_border(const int* label, T* count, int W, int H, const int* gate,
                                  cudaStream_t s) {
  dim3 b(32, 8), g((W + 31) / 32, (H + 31) / 32);
  border_kernel<T><<<g, b, 0, s>>>(label, count, W, H, gate);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status border_float(const int* label, float* count, int W, int H, cudaStream_t s) {
  return launch_border(label, count, W, H, nullptr, s);
}
cageo_status border_u32(const int* label, uint32_t* count, int W, int H, cudaStream_t s) {
  return launch_border(label, count, W, H, nullptr, s);
}
cageo_status border_u32_gated(const int* label, uint32_t* count, int W, int H, const int* gate,
                              cudaStream_t s) {
  return launch_border(label, count, W, H, gate, s);
}

}  // namespace cageo

using namespace cageo;

extern "C" size_t cageo_trace_workspace_size(int W, int H) {
  if (!valid_dims(W, H)) return 0;
  return trace_workspace_bytes(W, H);
}

extern "C" cageo_status cageo_trace_mode(const int8_t* d_dir, const float* d_streams,
                                         int* d_label, int W, int H, int mode,
                                         void* d_workspace, size_t workspace_bytes,
                                         cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_dir && d_streams && d_label && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(mode == CAGEO_TRACE_CPU_COMPAT || mode == CAGEO_TRACE_DEAD_END_ERROR,
                  "tracing mode");
  Scratch ws;
  cageo_status st = ws.acquire(d_workspace, workspace_bytes, trace_workspace_bytes(W, H), stream);
  if (st) return st;
  TraceWork w = trace_carve(ws.ptr, W, H);
  if ((st = trace_run(d_dir, d_streams, d_label, w, stream, mode, true))) return st;
  CAGEO_CUDA(cudaStreamSynchronize(stream));
  return trace_check_status(w, nullptr);
}

extern "C" cageo_status cageo_trace(const int8_t* d_dir, const float* d_streams,
                                    int* d_label, int W, int H, void* d_workspace,
                                    size_t workspace_bytes, cudaStream_t stream) {
  return cageo_trace_mode(d_dir, d_streams, d_label, W, H, CAGEO_TRACE_CPU_COMPAT, d_workspace,
                          workspace_bytes, stream);
}

extern "C" cageo_status cageo_border_accumulate(const int* d_label, float* d_count, int W,
                                                int H, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_label && d_count && valid_dims(W, H), "pointers and size");
  return border_float(d_label, d_count, W, H, stream);
}
