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
// they are computed here as shortest-path distances by tile relaxation (a
// persistent cooperative kernel on an asynchronous tile queue: one warp runs
// a bit-parallel breadth-first search over a 32x32 tile of the tiles that
// hold flat cells, seeded from its halo, and queues the neighbouring tiles
// when its border changed), and
// the directions by one final pass that applies the last-match rule to the
// finished distances.
//
// The GPU-order mode follows the reference's GPU routing instead
// (src/flowrouting/FlowRoutingAlgorithmGPUCUDAOriginal.cu:200-271 and
// :391-437): NODATA cells get flatDist -3 and are skipped as neighbours;
// layer 1 may drain into any cell with a negative flatDist (streams too)
// whose non-NODATA elevation is <= the flat cell's; a later layer k drains
// into a cell of an earlier layer; the FIRST match in the order N, W, E,
// S, NW, NE, SW, SE wins.  The layer numbers are again BFS distances.
#include <algorithm>
#include "common.cuh"
#include "routing.cuh"
#include "stage_math.cuh"
#include "tilequeue.cuh"

namespace cageo {

constexpr int kFlatInf = 0x3fffffff;
constexpr int kOffGrid = (int)0x80000000;  // staged code of a cell outside the grid
enum : int { R_NFLAT = 0, R_ERR = 3, R_US_BFS = 8, R_PASSES = 9,
             R_TILES = 10, R_KCYC_LOAD = 11, R_KCYC_BFS = 12, R_KCYC_STORE = 13,
             R_BAR_COUNT = kBarCountSlot, R_BAR_GEN = kBarGenSlot,
             R_HEAD = 128,     // work-queue tickets handed out (own 128-byte line)
             R_TAIL = 160,     // work-queue entries pushed (own line)
             R_PENDING = 192,  // tiles queued or being searched (own line)
             R_SIZE = 224 };
constexpr int kFT = 32;          // flat tile size
constexpr int kFWarps = 20;      // warps per block of the flat kernel (20 x 9.5 KB smem)
constexpr int kFRS = 35;         // staged row stride

size_t route_workspace_bytes(int W, int H) {
  const size_t nt = (size_t)((W + kFT - 1) / kFT) * ((H + kFT - 1) / kFT);
  return align_up(nt, 256) + align_up(nt * 4, 256) + align_up((2 * nt + kRingSlack) * 4, 256) +
         align_up(R_SIZE * 4, 256);
}

RouteWork route_carve(void* base, int W, int H) {
  RouteWork w;
  w.W = W;
  w.H = H;
  w.tiles_x = (W + kFT - 1) / kFT;
  w.tiles_y = (H + kFT - 1) / kFT;
  const size_t n = (size_t)W * H, nt = (size_t)w.tiles_x * w.tiles_y;
  char* p = (char*)base;
  (void)n;
  w.tflat = (uint8_t*)p;
  p += align_up(nt, 256);
  w.queued = (int*)p;
  p += align_up(nt * 4, 256);
  w.lists = (int*)p;
  p += align_up((2 * nt + kRingSlack) * 4, 256);
  w.scal = (unsigned int*)p;
  return w;
}

// Steepest-descent pass.  flatdist: -1 direction, -2 stream, -3 NODATA
// (GPU order only), kFlatInf flat.  A 32x8 block covers one 32x32 flat
// tile (4 rows per thread), so the tile's "holds a flat cell" flag and the
// flat-cell count take one store and one atomic per block.
template <bool GPU>
__global__ void __launch_bounds__(256) d8_kernel(const float* __restrict__ dem,
                                                 char2* __restrict__ dir,
                                                 int* __restrict__ fd, RouteWork w, float nodata) {
  const int W = w.W, H = w.H;
  const int slab_h = w.slab_h ? w.slab_h : H;
  const int x = blockIdx.x * kFT + threadIdx.x;
  // The tile's elevations and a one-cell halo in shared memory.
  __shared__ float E[34 * 35];
  {
    const int x0 = blockIdx.x * kFT - 1, y0 = blockIdx.y * kFT - 1;
#pragma unroll
    for (int k = threadIdx.y * 32 + threadIdx.x; k < 34 * 34; k += 256) {
      const int hy = k / 34, hx = k - hy * 34;
      const int gx = x0 + hx, gy = y0 + hy;
      if (gx >= 0 && gx < W && gy >= 0 && gy < H)
        cp_async4(&E[hy * 35 + hx], dem + (int64_t)gy * W + gx);  // all in flight at once
      else
        E[hy * 35 + hx] = 0.0f;
    }
    cp_async_wait();
  }
  __syncthreads();
  int nflat = 0;
#pragma unroll
  for (int k = 0; k < kFT / 8; k++) {
    const int y = blockIdx.y * kFT + threadIdx.y + 8 * k;
    if (x >= W || y >= H) continue;
    const int64_t i = (int64_t)y * W + x;
    int dxi = 0, dyi = 0;
    const int ys = y % slab_h;  // row within its realization's slab
    if (x == 0) dxi = -1; else if (x == W - 1) dxi = 1;
    if (ys == 0) dyi = -1; else if (ys == slab_h - 1) dyi = 1;
    if (dxi || dyi) {
      dir[i] = make_char2((signed char)dxi, (signed char)dyi);
      fd[i] = -1;
      continue;
    }
    const float* ec = &E[(threadIdx.y + 8 * k + 1) * 35 + threadIdx.x + 1];
    const float c = *ec;
    if (c == 0.0f) {
      dir[i] = make_char2(0, 0);
      fd[i] = -2;
      continue;
    }
    if (GPU && c == nodata) {
      dir[i] = make_char2(0, 0);
      fd[i] = -3;
      continue;
    }
    float steepest = 0.0f;
    int sdx = 0, sdy = 0;
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int dx = d8_dx(n), dy = d8_dy(n);
      const float e = ec[dy * 35 + dx];
      if (GPU && e == nodata) continue;
      float sl = __fsub_rn(c, e);
      // A diagonal drop only shrinks when divided by sqrt(2), so the
      // (slow, correctly rounded) division is needed only when the
      // undivided drop already beats the steepest so far.
      if (sl > 0.0f && sl > steepest) {
        if (n & 1) sl = __fdiv_rn(sl, 1.41421356237309505f);
        if (sl > steepest) { steepest = sl; sdx = dx; sdy = dy; }
      }
    }
    if (steepest > 0.0f) {
      dir[i] = make_char2((signed char)sdx, (signed char)sdy);
      fd[i] = -1;
    } else {
      dir[i] = make_char2(0, 0);
      fd[i] = kFlatInf;
      nflat++;
    }
  }
  __shared__ int block_flat;
  if (threadIdx.x == 0 && threadIdx.y == 0) block_flat = 0;
  __syncthreads();
  nflat = __reduce_add_sync(0xffffffffu, nflat);
  if (threadIdx.x == 0 && nflat) atomicAdd(&block_flat, nflat);
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0 && block_flat) {
    w.tflat[blockIdx.y * w.tiles_x + blockIdx.x] = 1;
    atomicAdd(&w.scal[R_NFLAT], (unsigned int)block_flat);  // statistics only
  }
}

// ---- flat distances by tile relaxation ----------------------------------
// Staged value of a cell for its neighbours: 0 for a cell a first-layer flat
// cell may drain into (CPU: a direction; GPU order: a direction or a stream,
// with an elevation that is not NODATA), the current distance of a flat
// cell, "infinite" otherwise.
__device__ __forceinline__ int flat_relay(int code, float e, bool gpu, float nodata) {
  if (code >= 0) return code;
  if (gpu) return ((code == -1 || code == -2) && e != nodata) ? 0 : kFlatInf;
  return code == -1 ? 0 : kFlatInf;
}

struct FlatSmem {
  int R[34 * kFRS];      // staged relay values (tile + halo)
  float E[34 * kFRS];    // staged elevations
};

// The flat BFS's queue (tilequeue.cuh): tile states in w.queued, the ring
// in w.lists.
__device__ __forceinline__ TileQueue route_queue(const RouteWork& w) {
  return TileQueue{w.queued,
                   w.lists,
                   2u * (unsigned int)(w.tiles_x * w.tiles_y) + kRingSlack,
                   w.scal + R_HEAD,
                   w.scal + R_TAIL,
                   w.scal + R_PENDING,
                   (int*)(w.scal + R_ERR)};
}

__device__ __forceinline__ void flat_enqueue(const RouteWork& w, int t) {
  if (!((volatile uint8_t*)w.tflat)[t]) return;  // no flat cell: nothing to do
  tq_enqueue(route_queue(w), t);
}

// Per-warp visit statistics (lane 0), flushed every 64 visits and at the end.
struct FlatStats {
  unsigned int tiles = 0, kload = 0, kbfs = 0, kstore = 0;
};

__device__ __forceinline__ void flush_flat_stats(const RouteWork& w, FlatStats& st) {
  if (!st.tiles) return;
  atomicAdd(&w.scal[R_TILES], st.tiles);
  atomicAdd(&w.scal[R_KCYC_LOAD], st.kload);
  atomicAdd(&w.scal[R_KCYC_BFS], st.kbfs);
  atomicAdd(&w.scal[R_KCYC_STORE], st.kstore);
  st = FlatStats{};
}

__device__ void flat_tile(FlatSmem& s, const float* __restrict__ dem, int* fd, const RouteWork& w,
                          int t, int lane, bool gpu, float nodata, FlatStats& st) {
  const int W = w.W, H = w.H;
  const int tx = t % w.tiles_x, ty = t / w.tiles_x;
  const int x0 = tx * kFT, y0 = ty * kFT;
  const long long c0 = clock64();
  // Stage the raw codes and elevations.  The elevations never change: they
  // come by asynchronous copies (all in flight at once).  The codes hold
  // distances other warps write meanwhile: they are read from L2 (an L1
  // line could hold an older value), in a loop
  // of their own so that the copies' memory clobber does not keep each load
  // from being issued before the previous iteration's copy.
  for (int idx = lane; idx < 34 * 34; idx += 32) {
    const int hy = idx / 34, hx = idx - hy * 34;
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
    float* de = &s.E[hy * kFRS + hx];
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) cp_async4(de, dem + (int64_t)gy * W + gx);
    else *de = 0.0f;
  }
#pragma unroll 12
  for (int idx = lane; idx < 34 * 34; idx += 32) {
    const int hy = idx / 34, hx = idx - hy * 34;
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
    int code = kOffGrid;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) code = __ldcg(fd + (int64_t)gy * W + gx);
    s.R[hy * kFRS + hx] = code;
  }
  cp_async_wait();
  __syncwarp();
  // Lane y: the flat cells of row y, and its exits (cells with a direction
  // that a first-layer flat cell may drain into: relay 0).  The staged codes
  // stay raw; the seeds below turn the few they read into relay values.
  const int y = lane;
  unsigned int flat = 0, exitm = 0;
#pragma unroll
  for (int x = 0; x < kFT; x++) {
    const int b = (y + 1) * kFRS + (x + 1);
    const int code = s.R[b];
    if (code == kFlatInf || code >= 1) flat |= 1u << x;
    // flat_relay(code) == 0 for a non-flat cell; the elevation matters in
    // GPU order only.
    const bool ex = gpu ? ((code == -1 || code == -2) && s.E[b] != nodata) : code == -1;
    if (ex) exitm |= 1u << x;
  }
  __syncwarp();
  const long long c1 = clock64();
  // Distances inside the tile by a bit-parallel breadth-first search: lane y
  // holds row y as a bit mask.  A flat cell is a seed at level 1 + the least
  // relay among its neighbours that are not flat cells of this tile (halo
  // cells, or exits inside the tile) and whose elevation is <= its own;
  // flat cells pass levels on to their flat neighbours (which have the same
  // elevation, so the elevation test always holds between them).  Levels are
  // visited in increasing order, so the first level that reaches a cell is
  // its distance; old values inside the tile came from halo values that can
  // only have dropped since, so they are never below the new ones.
  //
  // Only cells on the tile's rim or next to an exit of the tile (a non-flat
  // cell with relay 0) can be seeds.  Inside the rim a seed's non-flat
  // neighbours are all inside the tile, where the least relay is 0 (an exit)
  // or none, so inner seeds are all at level 1.  Rim seeds are held one per lane: the top and bottom rows by
  // column (lane = x), the left and right columns by row (lane = y, rows
  // 1..30); each level's seed masks then come from two ballots.
  unsigned int fup = __shfl_up_sync(0xffffffffu, flat, 1);
  unsigned int fdn = __shfl_down_sync(0xffffffffu, flat, 1);
  if (lane == 0) fup = 0;
  if (lane == kFT - 1) fdn = 0;
  // Seed level of cell (cx, cy) (kFlatInf: none); fr = the flat masks of
  // rows cy-1, cy, cy+1 (bit set = flat cell of this tile).
  auto seed_of = [&](int cx, int cy, unsigned int fu, unsigned int fm, unsigned int fb) {
    const int b = (cy + 1) * kFRS + (cx + 1);
    const float e = s.E[b];
    int best = kFlatInf;
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int nx = cx + d8_dx(n), ny = cy + d8_dy(n);
      const unsigned int row = d8_dy(n) < 0 ? fu : (d8_dy(n) > 0 ? fb : fm);
      const bool inner = nx >= 0 && nx < kFT && ny >= 0 && ny < kFT && ((row >> nx) & 1u);
      const int o = b + d8_dy(n) * kFRS + d8_dx(n);
      const float eo = s.E[o];
      const int v = flat_relay(s.R[o], eo, gpu, nodata);  // the staged codes are raw
      if (!inner && v < best && eo <= e) best = v;
    }
    return best < kFlatInf ? best + 1 : kFlatInf;
  };
  const unsigned int f0 = __shfl_sync(0xffffffffu, flat, 0);
  const unsigned int f1 = __shfl_sync(0xffffffffu, flat, 1);
  const unsigned int f30 = __shfl_sync(0xffffffffu, flat, kFT - 2);
  const unsigned int f31 = __shfl_sync(0xffffffffu, flat, kFT - 1);
  // Top row (0, x = lane) and bottom row (31, x = lane).
  const int tseed = ((f0 >> lane) & 1u) ? seed_of(lane, 0, 0u, f0, f1) : kFlatInf;
  const int bseed = ((f31 >> lane) & 1u) ? seed_of(lane, kFT - 1, f30, f31, 0u) : kFlatInf;
  // Left (y, 0) and right (y, 31) columns, rows 1..30 (y = lane).
  const bool mid = lane >= 1 && lane <= kFT - 2;
  const int lseed = (mid && (flat & 1u)) ? seed_of(0, y, fup, flat, fdn) : kFlatInf;
  const int rseed = (mid && (flat >> 31)) ? seed_of(kFT - 1, y, fup, flat, fdn) : kFlatInf;
  // Inner candidates next to an exit of the tile: level 1 or none (an inner
  // cell's other non-flat neighbours relay nothing).
  unsigned int exu = __shfl_up_sync(0xffffffffu, exitm, 1);
  unsigned int exd = __shfl_down_sync(0xffffffffu, exitm, 1);
  const unsigned int ex3 = exitm | exu | exd;
  const unsigned int near_exit = ex3 | (ex3 << 1) | (ex3 >> 1);
  unsigned int inner1 = 0;
  if (mid) {
    for (unsigned int m = flat & near_exit & 0x7ffffffeu; m; m &= m - 1) {
      const int x = __ffs(m) - 1;
      if (seed_of(x, y, fup, flat, fdn) == 1) inner1 |= 1u << x;
    }
  }
  auto next_level = [&](int after) {  // least seed level above `after`
    int m = kFlatInf;
    if (tseed > after) m = min(m, tseed);
    if (bseed > after) m = min(m, bseed);
    if (lseed > after) m = min(m, lseed);
    if (rseed > after) m = min(m, rseed);
    if (inner1 && after < 1) m = min(m, 1);
    return __reduce_min_sync(0xffffffffu, m);
  };
  int L = next_level(0);
  unsigned int visited = 0, front = 0, changed = 0;
  // The level of each reached cell is kept as an offset from Lb in 6 bit
  // planes (lane = row, bit = column) and written to the staged tile in one
  // pass per segment of at most 64 consecutive levels (when the front dies
  // out, or after 64 levels), so the level loop itself does no shared-memory
  // traffic.
  int Lb = L;
  unsigned int seg = 0, pl0 = 0, pl1 = 0, pl2 = 0, pl3 = 0, pl4 = 0, pl5 = 0;
  auto flush = [&]() {
    for (unsigned int r = seg; r; r &= r - 1) {
      const int x = __ffs(r) - 1;
      const int off = ((pl0 >> x) & 1) | (((pl1 >> x) & 1) << 1) | (((pl2 >> x) & 1) << 2) |
                      (((pl3 >> x) & 1) << 3) | (((pl4 >> x) & 1) << 4) |
                      (((pl5 >> x) & 1) << 5);
      int* cell = &s.R[(y + 1) * kFRS + (x + 1)];
      if (Lb + off < *cell) {
        *cell = Lb + off;
        changed |= 1u << x;
      }
    }
    seg = pl0 = pl1 = pl2 = pl3 = pl4 = pl5 = 0;
  };
  for (int guard = 0; guard < 4 * kFT * kFT && L < kFlatInf; guard++) {
    const unsigned int tb = __ballot_sync(0xffffffffu, tseed == L);
    const unsigned int bb = __ballot_sync(0xffffffffu, bseed == L);
    unsigned int seeds = (L == 1 ? inner1 : 0u) | (lseed == L ? 1u : 0u) |
                         (rseed == L ? 0x80000000u : 0u);
    if (lane == 0) seeds |= tb;
    if (lane == kFT - 1) seeds |= bb;
    unsigned int up = __shfl_up_sync(0xffffffffu, front, 1);
    unsigned int dn = __shfl_down_sync(0xffffffffu, front, 1);
    if (lane == 0) up = 0;
    if (lane == kFT - 1) dn = 0;
    const unsigned int v = front | up | dn;
    const unsigned int reach = ((v | (v << 1) | (v >> 1)) | seeds) & flat & ~visited;
    visited |= reach;
    front = reach;
    const int off = L - Lb;  // 0..63
    seg |= reach;
    if (off & 1) pl0 |= reach;
    if (off & 2) pl1 |= reach;
    if (off & 4) pl2 |= reach;
    if (off & 8) pl3 |= reach;
    if (off & 16) pl4 |= reach;
    if (off & 32) pl5 |= reach;
    // Next level, or jump to the next seed level when the front died out.
    if (__any_sync(0xffffffffu, front != 0)) {
      if (++L - Lb == 64) {
        flush();
        Lb = L;
      }
    } else {
      flush();
      L = next_level(L);
      Lb = L;
    }
  }
  flush();
  __syncwarp();
  const long long c2 = clock64();
  const bool capped = false;
  // Write back the changed distances (lane = column now); note the sides.
  for (int yy = 0; yy < kFT; yy++) {
    const unsigned int row = __shfl_sync(0xffffffffu, changed, yy);
    if ((row >> lane) & 1u)
      fd[(int64_t)(y0 + yy) * W + (x0 + lane)] = s.R[(yy + 1) * kFRS + (lane + 1)];
  }
  // The write-back is visible before any neighbour is queued or the tile's
  // state changes.  A visit that changed nothing wrote nothing.
  if (__any_sync(0xffffffffu, changed != 0)) __threadfence();
  __syncwarp();
  const unsigned int top = __shfl_sync(0xffffffffu, changed, 0);
  const unsigned int bot = __shfl_sync(0xffffffffu, changed, kFT - 1);
  const unsigned int lcol = __ballot_sync(0xffffffffu, changed & 1u);
  const unsigned int rcol = __ballot_sync(0xffffffffu, changed >> 31);
  unsigned int sides = (lcol ? 1u : 0u) | (rcol ? 2u : 0u) | (top ? 4u : 0u) | (bot ? 8u : 0u) |
                       ((top & 1u) ? 16u : 0u) | ((top >> 31) ? 32u : 0u) |
                       ((bot & 1u) ? 64u : 0u) | ((bot >> 31) ? 128u : 0u);
  if (lane < 9) {
    int dx = 0, dy = 0;
    bool want = false;
    switch (lane) {
      case 0: want = capped; break;
      case 1: dx = -1; want = sides & 1; break;
      case 2: dx = 1; want = sides & 2; break;
      case 3: dy = -1; want = sides & 4; break;
      case 4: dy = 1; want = sides & 8; break;
      case 5: dx = -1; dy = -1; want = sides & 16; break;
      case 6: dx = 1; dy = -1; want = sides & 32; break;
      case 7: dx = -1; dy = 1; want = sides & 64; break;
      case 8: dx = 1; dy = 1; want = sides & 128; break;
    }
    const int nx = tx + dx, ny = ty + dy;
    if (want && nx >= 0 && ny >= 0 && nx < w.tiles_x && ny < w.tiles_y)
      flat_enqueue(w, ny * w.tiles_x + nx);
  }
  __syncwarp();
  if (lane == 0) {
    const long long c3 = clock64();
    st.tiles++;
    st.kload += (unsigned int)((c1 - c0) >> 10);
    st.kbfs += (unsigned int)((c2 - c1) >> 10);
    st.kstore += (unsigned int)((c3 - c2) >> 10);
  }
}

// The flat BFS: every tile holding a flat cell is queued, one 2x2 parity
// class of tiles after another (grid barrier between), so tiles searched at
// the same time are rarely neighbours and each class starts from the
// finished borders of the classes before it; then the warps drain the
// asynchronous queue (tilequeue.cuh), a tile whose border distances changed
// queueing its neighbours.  No pass barriers: a free warp takes the next
// queued tile at once.  A CPU simulation of the queue needed no more tile
// visits than pass-synchronous worklists (2.70 against 2.71 per tile at
// 2048^2); on the GPU it took 149 k visits against 186 k at 8192^2.  Waits
// are bounded; a limit sets the error flag.
__global__ void __launch_bounds__(kFWarps * 32, 1)
flat_relax_kernel(const float* __restrict__ dem, int* fd, RouteWork w, int gpu, float nodata) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  FlatSmem& s = reinterpret_cast<FlatSmem*>(smraw)[warp];
  const int ntiles = w.tiles_x * w.tiles_y;
  GridSync gs{w.scal + R_BAR_COUNT, w.scal + R_BAR_GEN, (int*)(w.scal + R_ERR)};
  volatile unsigned int* vs = w.scal;
  const TileQueue q = route_queue(w);
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  const int gwarp = blockIdx.x * kFWarps + warp, nwarps = gridDim.x * kFWarps;
  bool go = true;
  for (int c = 0; c < 4 && go; c++) {
    for (int i = gwarp; i < ntiles; i += nwarps) {
      const int tx = i % w.tiles_x, ty = i / w.tiles_x;
      if (lane == 0 && ((tx & 1) | ((ty & 1) << 1)) == c && w.tflat[i]) tq_enqueue(q, i);
    }
    go = grid_barrier(gs, gridDim.x);
  }
  FlatStats st;
  if (go) {
    const unsigned int visit_cap = 1000u * (unsigned int)min(ntiles, 4000000);
    long long ticket = -1;
    unsigned int ns = 32;
    for (long long idle = 0;;) {
      int t = -1;
      if (lane == 0) t = tq_try_dequeue(q, &ticket);
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t >= 0) {
        flat_tile(s, dem, fd, w, t, lane, gpu != 0, nodata, st);
        if (lane == 0) {
          tq_finish(q, t, false);
          if (st.tiles >= 64) flush_flat_stats(w, st);
        }
        __syncwarp();
        idle = 0;
        ns = 32;
        continue;
      }
      if (vs[R_ERR]) break;
      if (vs[R_PENDING] == 0u) break;
      if (++idle > (1LL << 24) || vs[R_TILES] > visit_cap) {
        if (lane == 0) atomicCAS((int*)(w.scal + R_ERR), 0, 2);
        break;
      }
      __nanosleep(ns);
      if (ns < 1024) ns <<= 1;
    }
  }
  if (lane == 0) flush_flat_stats(w, st);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    vs[R_PASSES] = 1u;  // one drain of the queue
    vs[R_US_BFS] = (unsigned int)((t1 - t0) / 1000);
  }
}

// Directions of flat cells, and flatDist 0 for the flats left unresolved,
// over the tiles that hold flat cells only (a 32x8 block per 32x32 tile, 4
// rows per thread).  CPU rules: the LAST neighbour in N..NW order in the
// previous layer (flatDist -1 for layer 1) whose elevation is <= the
// cell's.  GPU order: the FIRST neighbour in N, W, E, S, NW, NE, SW, SE
// order that is (layer 1) a non-NODATA cell with a negative flatDist and an
// elevation <= the cell's, or (layer d > 1) a cell of layers 1..d-1.  A
// neighbour reset from "unresolved" to 0 meanwhile matches neither rule
// before or after, so the reset can share the pass.
template <bool GPU>
__global__ void __launch_bounds__(256) flat_dir_kernel(const float* __restrict__ dem,
                                                       char2* __restrict__ dir,
                                                       int* __restrict__ fd, RouteWork w,
                                                       float nodata) {
  if (!w.tflat[blockIdx.y * w.tiles_x + blockIdx.x]) return;
  const int W = w.W, H = w.H;
  const int x = blockIdx.x * kFT + threadIdx.x;
  constexpr int order[8] = {0, 6, 2, 4, 7, 1, 5, 3};  // N W E S NW NE SW SE as D8 indices
  // Codes and elevations of the tile and a one-cell halo (outside: kOffGrid).
  __shared__ int F[34 * 35];
  __shared__ float E[34 * 35];
  {
    const int x0 = blockIdx.x * kFT - 1, y0 = blockIdx.y * kFT - 1;
#pragma unroll
    for (int k = threadIdx.y * 32 + threadIdx.x; k < 34 * 34; k += 256) {
      const int hy = k / 34, hx = k - hy * 34;
      const int gx = x0 + hx, gy = y0 + hy;
      if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
        const int64_t i = (int64_t)gy * W + gx;
        cp_async4(&F[hy * 35 + hx], fd + i);  // all in flight at once
        cp_async4(&E[hy * 35 + hx], dem + i);
      } else {
        F[hy * 35 + hx] = kOffGrid;
        E[hy * 35 + hx] = 0.0f;
      }
    }
    cp_async_wait();
  }
  __syncthreads();
#pragma unroll 1
  for (int k = 0; k < kFT / 8; k++) {
    const int y = blockIdx.y * kFT + threadIdx.y + 8 * k;
    if (x >= W || y >= H) continue;
    const int64_t c = (int64_t)y * W + x;
    const int b = (threadIdx.y + 8 * k + 1) * 35 + threadIdx.x + 1;
    const int d = F[b];
    if (d == kFlatInf) {
      fd[c] = 0;
      continue;
    }
    if (d < 1) continue;  // not a flat cell with a layer
    const float e = E[b];
    int nf[8];
    float ne[8];
#pragma unroll
    for (int n = 0; n < 8; n++) {
      nf[n] = F[b + d8_dy(n) * 35 + d8_dx(n)];
      ne[n] = E[b + d8_dy(n) * 35 + d8_dx(n)];
    }
    int got = -1;
    if (GPU) {
#pragma unroll
      for (int q = 7; q >= 0; q--) {
        const int n = order[q];
        const bool ok = d == 1 ? (nf[n] < 0 && nf[n] != kOffGrid && ne[n] != nodata && ne[n] <= e)
                               : (nf[n] >= 1 && nf[n] <= d - 1);
        if (ok) got = n;
      }
    } else {
      const int want = d == 1 ? -1 : d - 1;
#pragma unroll
      for (int n = 0; n < 8; n++)
        if (nf[n] == want && ne[n] <= e) got = n;
    }
    if (got >= 0) dir[c] = make_char2((signed char)d8_dx(got), (signed char)d8_dy(got));
  }
}

__global__ void route_scalars_kernel(unsigned int* s) {
  for (int i = threadIdx.x; i < R_SIZE; i += blockDim.x) s[i] = 0u;
}

cageo_status route_run(const float* filled, int8_t* dir, int* fd, const RouteWork& w,
                       cudaStream_t s, int mode, float nodata) {
  const bool gpu = mode == CAGEO_ROUTE_GPU_ORDER;
  const size_t nt = (size_t)w.tiles_x * w.tiles_y;
  route_scalars_kernel<<<1, 128, 0, s>>>(w.scal);
  CAGEO_CUDA(cudaMemsetAsync(w.tflat, 0, nt, s));
  CAGEO_CUDA(cudaMemsetAsync(w.queued, 0, nt * 4, s));  // all idle
  CAGEO_CUDA(cudaMemsetAsync(w.lists, 0xff, (2 * nt + kRingSlack) * 4, s));  // empty ring
  dim3 b(32, 8), g(w.tiles_x, w.tiles_y);
  if (gpu) d8_kernel<true><<<g, b, 0, s>>>(filled, (char2*)dir, fd, w, nodata);
  else d8_kernel<false><<<g, b, 0, s>>>(filled, (char2*)dir, fd, w, nodata);
  CAGEO_CUDA(cudaGetLastError());
  static PerDevice resident;
  const size_t smem = sizeof(FlatSmem) * kFWarps;
  int coop = 0;
  cageo_status st = per_device(resident, &coop, [&](int dev, int* v) -> cageo_status {
    CAGEO_CUDA(cudaFuncSetAttribute(flat_relax_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return resident_blocks((const void*)flat_relax_kernel, kFWarps * 32, smem, dev, v);
  });
  if (st) return st;
  const float* f = filled;
  int* fdp = fd;
  RouteWork wc = w;
  int gflag = gpu ? 1 : 0;
  float nd = nodata;
  void* params[] = {(void*)&f, (void*)&fdp, (void*)&wc, (void*)&gflag, (void*)&nd};
  const int fgrid = std::max(1, std::min(coop, (int)((nt + kFWarps - 1) / kFWarps)));
  CAGEO_CUDA(cudaLaunchCooperativeKernel((const void*)flat_relax_kernel, dim3(fgrid),
                                         dim3(kFWarps * 32), params, smem, s));
  if (gpu) flat_dir_kernel<true><<<g, b, 0, s>>>(filled, (char2*)dir, fd, w, nodata);
  else flat_dir_kernel<false><<<g, b, 0, s>>>(filled, (char2*)dir, fd, w, nodata);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status route_check_status(const RouteWork& w, int64_t* stats) {
  unsigned int h[R_SIZE];
  CAGEO_CUDA(cudaMemcpy(h, w.scal, sizeof(h), cudaMemcpyDeviceToHost));
  if (stats) {
    stats[0] = h[R_PASSES];
    stats[1] = h[R_NFLAT];
    stats[2] = h[R_US_BFS];
    stats[3] = h[R_TILES];
    stats[4] = h[R_KCYC_LOAD];
    stats[5] = h[R_KCYC_BFS];
    stats[6] = h[R_KCYC_STORE];
  }
  if (h[R_ERR]) {
    set_error("flow routing: flat-surface relaxation hit a wait or pass limit");
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

extern "C" cageo_status cageo_route_d8_mode(const float* d_filled, int8_t* d_dir,
                                            int* d_flatdist, int W, int H, float nodata_dem,
                                            int mode, void* d_workspace, size_t workspace_bytes,
                                            cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_filled && d_dir && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(mode == CAGEO_ROUTE_CPU_COMPAT || mode == CAGEO_ROUTE_GPU_ORDER, "routing mode");
  Scratch ws;
  cageo_status st = ws.acquire(d_workspace, workspace_bytes,
                               cageo_route_workspace_size(W, H), stream);
  if (st) return st;
  RouteWork w = route_carve(ws.ptr, W, H);
  int* fd = d_flatdist ? d_flatdist
                       : (int*)((char*)ws.ptr + route_workspace_bytes(W, H));
  if ((st = route_run(d_filled, d_dir, fd, w, stream, mode, nodata_dem))) return st;
  CAGEO_CUDA(cudaStreamSynchronize(stream));
  return route_check_status(w, nullptr);
}

extern "C" cageo_status cageo_route_d8(const float* d_filled, int8_t* d_dir,
                                       int* d_flatdist, int W, int H, void* d_workspace,
                                       size_t workspace_bytes, cudaStream_t stream) {
  return cageo_route_d8_mode(d_filled, d_dir, d_flatdist, W, H, -9999.0f,
                             CAGEO_ROUTE_CPU_COMPAT, d_workspace, workspace_bytes, stream);
}
