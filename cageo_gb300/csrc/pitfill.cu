// pitfill.cu -- A6 pit filling with the semantics of the reference's CPU
// path (src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:68-242), and the exact
// float fill of its GPU path (src/pitfilling/PitFillingAlgorithmGPUCUDA.cu:
// 201-381) as a second mode: flood A alone on the unquantized grid, every
// outlet relaying, unreached cells ending at the GPU path's 99990000.
//
// The CPU fill is a bucket priority-flood over 1 mm levels in which a
// popped cell expands its neighbours only if its value v survives
// toElev(toIndex(v)) == v ("passable").  The result is: outlets (border
// cells and cells equal to 0) keep q; every other reached cell gets
// W = max(q, L) where L is the lowest value among neighbours that expand;
// a non-passable cell expands only when it was reached at a level L >= q;
// unreached cells keep q.  Whether a non-passable cell expands depends only
// on cells with a strictly lower q, so the solution is unique, and it is
// computed here by monotone relaxations:
//
//   1. flood A: every reached cell relays (non-passable outlets do not):
//      gives L_A <= L everywhere (a lower bound);
//   2. non-passable cells with L_A >= q are certainly expanding ("confirmed");
//      the other non-passable cells are walls for now;
//   3. flood B from +inf with walls: an upper bound L_B >= L;
//   4. phases: M = min L_B over unconfirmed non-passable cells with
//      L_B >= q; every such cell with q <= M is confirmed (no later change
//      can take its level below M >= q); relax again; repeat until none.
//
// Each flood is a persistent cooperative kernel.  One warp owns a 32x32
// tile at a time, stages W, q, flags and the relay values of a one-cell
// halo in shared memory and sweeps it down, up, right and left (Gauss-Seidel)
// until it stops changing; a tile whose border changed queues the
// neighbouring tiles on an asynchronous work queue (no pass barriers; see
// the queue below).  A flood ends when no tile is queued or in process.
// Every wait and every loop is bounded; exceeding a bound sets an error
// flag that the host turns into CAGEO_ERR_NO_CONVERGENCE.
#include <algorithm>
#include <type_traits>
#include "common.cuh"
#include "fillflags.cuh"
#include "pitfill.cuh"
#include "stage_math.cuh"
#include "tilequeue.cuh"

namespace cageo {

// Scalar block layout (unsigned ints).
enum : int {
  S_MIN = 0,       // ordered min of q (minE)
  S_ERR = 3,       // 0 ok; 1 barrier wait; 2 idle wait; 3 queue state; 4 visits; 5 phases; 6 union
  S_M = 7,         // 3 slots: ordered phase minima
  S_CAND = 10,     // number of undecided cells
  S_PASS = 11,     // drains run so far in this fill (a drain empties the work queue)
  S_PHASES = 12,
  S_PASSES_A = 13, // drains of flood A (1)
  S_PASSES_B = 14, // drains of flood B before the first phase (1)
  S_US_A = 15,     // microseconds of flood A
  S_US_B = 16,     // microseconds of flood B up to its first convergence
  S_US_P = 17,     // microseconds of the phase loop
  S_PEND = 18,     // 3 slots: pending cells seen by a phase
  S_RESET = 21,    // warm-started exact fill: cells restarted from +inf (unsupported)
  S_DBG = 24,      // 8 slots: the phase loop's state when it passed its limit (see below)
  // Per-visit statistics, updated by every tile visit: a line of their own
  // (96..127), away from the error flag that idle warps poll.
  S_TILES_A = 96,   // tiles processed by flood A
  S_ROUNDS_A = 97,  // sweep rounds run by flood A
  S_TILES_B = 98,   // tiles processed by flood B (phases included)
  S_ROUNDS_B = 99,  // sweep rounds run by flood B
  S_KCYC_LOAD = 100,   // kilo-cycles (summed over tile visits) staging tiles
  S_KCYC_SWEEP = 101,  // kilo-cycles sweeping
  S_KCYC_STORE = 102,  // kilo-cycles writing back and queueing
  S_KCYC_IDLE_A = 103, // kilo-cycles warps of flood A waited for a tile (tail included)
  S_KCYC_IDLE_B = 104, // the same for flood B's drains
  S_HEAD = 128,      // work-queue tickets handed out (own 128-byte line)
  S_TAIL = 160,      // work-queue entries pushed (own line)
  S_PENDING = 192,   // tiles queued or being processed (own line)
  S_BAR_COUNT = kBarCountSlot,
  S_BAR_GEN = kBarGenSlot,
  S_SIZE = 224
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr int kTile = 32;
constexpr int kRS = 35;           // relay row stride (34 used)
constexpr int kWS = 33;           // W/q row stride
constexpr int kFS = 36;           // flag row stride (bytes)

// Per-warp staged tile.  R: relay values of the tile and its one-cell halo.
// In flood A (modes 0 and 2) every cell that can change relays its own W,
// so W lives in R and only q is kept beside it (Q); flood B keeps (W, q)
// pairs (WQ), since its walls relay +inf whatever their W.  F: flags of the
// tile's own cells.  HC: clean relays of the halo (mode 2): [0] the row
// above and [1] the row below the tile (halo x 0..33), [2] the column left
// and [3] the column right of it (halo y 0..33); 1 = clean and passable.
struct SmemA {
  float R[34 * kRS];
  float Q[kTile * kWS];
  uint8_t F[kTile * kFS];
  uint8_t HC[4][34];
};
struct SmemB {
  float R[34 * kRS];
  float2 WQ[kTile * kWS];
  uint8_t F[kTile * kFS];
};
template <int MODE>
using WarpSmem = typename std::conditional<MODE == 1, SmemB, SmemA>::type;

// Warps per block (one block per SM) of the flood launches.  Flood B runs
// 16 (14.0 KB of shared memory each); flood A runs 16, 20 or 22 (10.0 KB
// each), chosen by FillWork::flood_warps (the autotuner picks it), with the
// register budget the launch bounds give each.
constexpr int kWarpsB = 16;

__device__ __forceinline__ float staged_w(const SmemA& s, int x, int y) {
  return s.R[(y + 1) * kRS + x + 1];
}
__device__ __forceinline__ float staged_w(const SmemB& s, int x, int y) {
  return s.WQ[y * kWS + x].x;
}
__device__ __forceinline__ float staged_q(const SmemA& s, int x, int y) {
  return s.Q[y * kWS + x];
}
__device__ __forceinline__ float staged_q(const SmemB& s, int x, int y) {
  return s.WQ[y * kWS + x].y;
}

size_t fill_workspace_bytes(int W, int H) {
  size_t n = (size_t)W * H;
  size_t nt = (size_t)((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
  return align_up(n, 256) + align_up(nt * 4, 256) + align_up((2 * nt + kRingSlack) * 4, 256) +
         2 * align_up(nt, 256) + 3 * align_up(n * 4, 256) + 1024;
}

FillWork fill_carve(void* base, int W, int H) {
  FillWork w;
  w.W = W;
  w.H = H;
  w.tiles_x = (W + kTile - 1) / kTile;
  w.tiles_y = (H + kTile - 1) / kTile;
  size_t n = (size_t)W * H, nt = (size_t)w.tiles_x * w.tiles_y;
  char* p = (char*)base;
  w.flags = (uint8_t*)p;
  p += align_up(n, 256);
  w.queued = (int*)p;
  p += align_up(nt * 4, 256);
  w.lists = (int*)p;
  p += align_up((2 * nt + kRingSlack) * 4, 256);
  w.tseed = (uint8_t*)p;
  p += align_up(nt, 256);
  w.tconv = (uint8_t*)p;
  p += align_up(nt, 256);
  w.cand = (uint32_t*)p;
  p += align_up(n * 4, 256);
  w.aux = (uint32_t*)p;
  p += align_up(n * 4, 256);
  w.cmin = (uint32_t*)p;
  p += align_up(n * 4, 256);
  w.scal = (unsigned int*)p;
  return w;
}

unsigned int* fill_min_slot(const FillWork& w) { return w.scal + S_MIN; }

// Flood modes: 0 = flood A (every reached cell relays), 2 = flood A that
// also keeps the clean marks (FCLEAN), 1 = flood B (non-passable cells that
// are not confirmed are walls).
template <int MODE>
__device__ __forceinline__ float relay(float w, uint8_t f, float q) {
  if (f & FNODATA) return kInf;
  if (f & FOUTLET) return (f & FNONPASS) ? kInf : q;
  if (MODE != 1 || !(f & FNONPASS)) return w;
  // A clean cell kept flood A's level, which is finite; it is confirmed
  // exactly when it is not below its q (what FCONF records for the others).
  // Every level flood B relays is a passable value (it starts at a passable
  // outlet's q and is only carried or raised to a passable cell's q), never
  // a non-passable q, so a non-passable cell whose level equals its q was
  // reached below it and is a wall: the store that lowered it to q also set
  // FBELOW.  Testing w != q keeps a halo read that sees the new level but
  // not yet the new flags (another SM's write-back stores the two with no
  // order between them) from relaying q.
  return ((f & (FCONF | FCLEAN)) && !(f & FBELOW) && w != q) ? w : kInf;
}

struct FloodArgs {
  const float* q;
  float* Wg;
  FillWork w;
  // Flood B runs as two launches: 1 = seeding and the main drain, 2 = the
  // confirmation phases (the undecided cells found and labelled by plain
  // kernels in between).  3 = the repair flood of a warm-started exact fill
  // (its statistics go to flood B's slots).  Flood A ignores 1 and 2.
  int stage = 0;
};

// ---- asynchronous tile work queue (tilequeue.cuh) --------------------------
// The fill's queue: tile states in w.queued, the ring in w.lists
// (2 * ntiles + kRingSlack slots), counters in the scalar block.
__device__ __forceinline__ TileQueue fill_queue(const FillWork& w) {
  return TileQueue{w.queued,
                   w.lists,
                   2u * (unsigned int)(w.tiles_x * w.tiles_y) + kRingSlack,
                   w.scal + S_HEAD,
                   w.scal + S_TAIL,
                   w.scal + S_PENDING,
                   (int*)(w.scal + S_ERR)};
}

__device__ __forceinline__ void enqueue(const FillWork& w, int t) { tq_enqueue(fill_queue(w), t); }

// Relaxation of staged cell (x, y) given m, the least relay among the
// neighbours it reads, split into its loads (cell_load) and its update
// (cell_store, true if the cell changed) so that the two cells of a sweep
// step are both loaded before either is written.  A cell whose incoming
// level has dropped below its own q (FBELOW) is final in both floods: its
// value is q and its relay can no longer change.
struct CellEval {
  float w, q, m;
  uint8_t f;
};

template <class S>
__device__ __forceinline__ CellEval cell_load(const S& s, int x, int y, float m) {
  return CellEval{staged_w(s, x, y), staged_q(s, x, y), m, s.F[y * kFS + x]};
}

template <int MODE>
__device__ __forceinline__ bool cell_store(WarpSmem<MODE>& s, int x, int y, const CellEval& e) {
  if (e.f & (FNODATA | FOUTLET | FBELOW)) return false;
  const float nw = fminf(e.w, fmaxf(e.q, e.m));
  const bool below = e.m < e.q;  // sets FBELOW, which the cell does not have yet
  if (nw == e.w && !below) return false;
  if constexpr (MODE == 1) s.WQ[y * kWS + x].x = nw;  // in flood A, R below holds W
  // A fall of W withdraws the cell's clean mark (its clean path may not
  // reach the new level); the clean pass after the sweeps derives it again.
  if (MODE == 2 && nw != e.w) s.F[y * kFS + x] = (e.f | (below ? FBELOW : 0)) & (uint8_t)~FCLEAN;
  else if (below) s.F[y * kFS + x] = e.f | FBELOW;
  // relay<MODE>() of a cell that is neither NODATA nor an outlet
  const bool wall = MODE == 1 && (e.f & FNONPASS) && (below || !(e.f & (FCONF | FCLEAN)));
  s.R[(y + 1) * kRS + (x + 1)] = wall ? kInf : nw;
  return true;
}

// Least relay of the three staged cells in relay row ry (tile row ry - 1),
// tile columns x-1..x+1: the neighbours of (x, ry - 2) below it or of
// (x, ry) above it.
template <class S>
__device__ __forceinline__ float row3_min(const S& s, int x, int ry) {
  const float* r = &s.R[ry * kRS + x];
  return fminf(fminf(r[0], r[1]), r[2]);
}

// Least relay of the three staged cells in relay column rx (tile column
// rx - 1), tile rows y-1..y+1.
template <class S>
__device__ __forceinline__ float col3_min(const S& s, int rx, int y) {
  const float* r = &s.R[y * kRS + rx];
  return fminf(fminf(r[0], r[kRS]), r[2 * kRS]);
}

// Per-warp visit statistics (lane 0), added to the scalar block every 64
// visits and when a drain ends: one atomic per counter and flush instead of
// five atomics on one cache line per visit.
struct VisitStats {
  unsigned int tiles = 0, rounds = 0, kload = 0, ksweep = 0, kstore = 0, kidle = 0;
};

template <int MODE>
__device__ __forceinline__ void flush_stats(const FillWork& w, VisitStats& st, bool b_slots) {
  if (!st.tiles && !st.kidle) return;
  b_slots = b_slots || MODE == 1;
  atomicAdd(&w.scal[b_slots ? S_TILES_B : S_TILES_A], st.tiles);
  atomicAdd(&w.scal[b_slots ? S_ROUNDS_B : S_ROUNDS_A], st.rounds);
  atomicAdd(&w.scal[S_KCYC_LOAD], st.kload);
  atomicAdd(&w.scal[S_KCYC_SWEEP], st.ksweep);
  atomicAdd(&w.scal[S_KCYC_STORE], st.kstore);
  if (st.kidle) atomicAdd(&w.scal[b_slots ? S_KCYC_IDLE_B : S_KCYC_IDLE_A], st.kidle);
  st = VisitStats{};
}

// Clean marks of a tile whose W has converged for its halo (flood A with
// clean marks).  A cell turns clean when a neighbour that is clean and
// passable (a relay flood B keeps) offers a level <= its W: that
// neighbour's clean path, extended by the cell, reaches the cell at no more
// than W, and flood B, which never undershoots flood A, then gives it W
// too.  The rule is sound whatever W is, so a cell keeps its mark until its
// W falls (cell_store withdraws it).  Lane = tile column x; per-lane masks
// hold bit y for tile row y.  The eight "offers <= W" tests are made once
// per cell; the marks then spread by bit operations on the column masks
// (neighbour columns by shuffles) until no lane changes, at most
// `max_iter` times.  Returns this lane's column of newly clean cells.
__device__ __forceinline__ unsigned int clean_pass(SmemA& s, int lane, int max_iter) {
  unsigned int qN = 0, qS = 0, qW = 0, qE = 0, qNW = 0, qNE = 0, qSW = 0, qSE = 0;
  unsigned int cl = 0, pas = 0;
  // Relay rows y, y+1, y+2 (tile rows y-1, y, y+1) at columns lane..lane+2.
  float a0 = s.R[lane], a1 = s.R[lane + 1], a2 = s.R[lane + 2];
  float b0 = s.R[kRS + lane], b1 = s.R[kRS + lane + 1], b2 = s.R[kRS + lane + 2];
#pragma unroll 4
  for (int y = 0; y < kTile; y++) {
    const float* rc = &s.R[(y + 2) * kRS + lane];
    const float c0 = rc[0], c1 = rc[1], c2 = rc[2];
    const uint8_t f = s.F[y * kFS + lane];
    const unsigned int bit = 1u << y;
    // b1 is the cell's own relay: its W (every non-outlet cell relays in flood A).
    const float wv = b1;
    if (f & FCLEAN) cl |= bit;
    if (!(f & (FNONPASS | FNODATA))) pas |= bit;
    if (!(f & (FCLEAN | FNODATA)) && wv < kInf) {
      if (a0 <= wv) qNW |= bit;
      if (a1 <= wv) qN |= bit;
      if (a2 <= wv) qNE |= bit;
      if (b0 <= wv) qW |= bit;
      if (b2 <= wv) qE |= bit;
      if (c0 <= wv) qSW |= bit;
      if (c1 <= wv) qS |= bit;
      if (c2 <= wv) qSE |= bit;
    }
    a0 = b0; a1 = b1; a2 = b2;
    b0 = c0; b1 = c1; b2 = c2;
  }
  const unsigned int cl0 = cl;
  if (!__any_sync(0xffffffffu, (qN | qS | qW | qE | qNW | qNE | qSW | qSE) != 0)) return 0u;
  // Clean relays of the halo: this lane's cells of the rows above and below
  // the tile, and the halo columns as 34-bit masks (bit = halo row 0..33).
  const unsigned long long top = s.HC[0][lane + 1], bot = s.HC[1][lane + 1];
  unsigned long long lcol = __ballot_sync(0xffffffffu, s.HC[2][lane] != 0);
  unsigned long long rcol = __ballot_sync(0xffffffffu, s.HC[3][lane] != 0);
  lcol |= ((unsigned long long)s.HC[2][32] << 32) | ((unsigned long long)s.HC[2][33] << 33);
  rcol |= ((unsigned long long)s.HC[3][32] << 32) | ((unsigned long long)s.HC[3][33] << 33);
  for (int it = 0; it < max_iter; it++) {
    // Column mask of clean relays, bit = halo row (tile row + 1).
    const unsigned long long own = ((unsigned long long)(cl & pas) << 1) | top | (bot << 33);
    unsigned long long L = __shfl_up_sync(0xffffffffu, own, 1);
    unsigned long long R = __shfl_down_sync(0xffffffffu, own, 1);
    if (lane == 0) L = lcol;
    if (lane == 31) R = rcol;
    const unsigned int nc =
        cl | (qN & (unsigned int)own) | (qS & (unsigned int)(own >> 2)) |
        (qW & (unsigned int)(L >> 1)) | (qE & (unsigned int)(R >> 1)) | (qNW & (unsigned int)L) |
        (qNE & (unsigned int)R) | (qSW & (unsigned int)(L >> 2)) | (qSE & (unsigned int)(R >> 2));
    const bool changed = nc != cl;
    cl = nc;
    if (!__any_sync(0xffffffffu, changed)) break;
  }
  const unsigned int turned = cl & ~cl0;
  for (unsigned int m = turned; m; m &= m - 1) {
    const int y = __ffs(m) - 1;
    s.F[y * kFS + lane] |= FCLEAN;
  }
  __syncwarp();
  return turned;
}

// Returns whether every cell of the tile is final (NODATA, outlet or FBELOW;
// with clean marks also clean).
template <int MODE>
__device__ bool process_tile(WarpSmem<MODE>& s, const FloodArgs& a, int t, int lane, VisitStats& st) {
  const FillWork& w = a.w;
  const int W = w.W, H = w.H;
  const int tx = t % w.tiles_x, ty = t / w.tiles_x;
  const int x0 = tx * kTile, y0 = ty * kTile;
  const long long c0 = clock64();
  if constexpr (MODE != 1) {
    // Flood A needs q only for the tile's own cells (an outlet's W is its q,
    // which is all its relay needs), and q never changes: asynchronous
    // copies, all in flight while the loop below loads W and the flags.
    for (int idx = lane; idx < kTile * kTile; idx += 32) {
      const int ty_ = idx >> 5, tx_ = idx & 31;
      const int gx = x0 + tx_, gy = y0 + ty_;
      float* dq = &s.Q[ty_ * kWS + tx_];
      if (gx < W && gy < H) cp_async4(dq, a.q + (int64_t)gy * W + gx);
      else *dq = 0.0f;
    }
  }
  // Flood A on a tile whose 32 columns lie inside the grid, with 16-byte
  // aligned rows: its columns' levels and flags by 16-byte and 4-byte loads
  // (8 chunks of 4 cells per staged row, 8.5 per lane, all in flight at
  // once), the two halo columns by scalar loads: about 21 loads per lane
  // instead of 72.  Every load lies inside the grid.
  const bool vec = MODE != 1 && x0 + kTile <= W && (W & 3) == 0 &&
                   ((reinterpret_cast<uintptr_t>(a.Wg) | reinterpret_cast<uintptr_t>(w.flags)) &
                    15u) == 0;
  if (vec) {
    constexpr int kChunks = 34 * (kTile / 4);  // 272
#pragma unroll
    for (int it = 0; it < (kChunks + 31) / 32; it++) {
      const int k = lane + 32 * it;
      if (k < kChunks) {
        const int hy = k >> 3, c = k & 7;
        const int gy = y0 - 1 + hy;
        float4 wv = make_float4(kInf, kInf, kInf, kInf);
        unsigned int f4 = 0x01010101u * FNODATA;
        if (gy >= 0 && gy < H) {
          const int64_t i = (int64_t)gy * W + x0 + 4 * c;
          wv = __ldcg(reinterpret_cast<const float4*>(a.Wg + i));
          f4 = __ldcg(reinterpret_cast<const unsigned int*>(w.flags + i));
        }
        float* r = &s.R[hy * kRS + 1 + 4 * c];
        r[0] = relay<MODE>(wv.x, (uint8_t)f4, wv.x);
        r[1] = relay<MODE>(wv.y, (uint8_t)(f4 >> 8), wv.y);
        r[2] = relay<MODE>(wv.z, (uint8_t)(f4 >> 16), wv.z);
        r[3] = relay<MODE>(wv.w, (uint8_t)(f4 >> 24), wv.w);
        if (hy >= 1 && hy <= kTile)
          *reinterpret_cast<unsigned int*>(&s.F[(hy - 1) * kFS + 4 * c]) = f4;
      }
    }
#pragma unroll
    for (int it = 0; it < 3; it++) {
      const int k = lane + 32 * it;
      if (k < 2 * 34) {
        const int side = k >= 34 ? 1 : 0, hy = k - 34 * side;
        const int hx = side ? kTile + 1 : 0;
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
        float wv = kInf;
        uint8_t fv = FNODATA;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
          const int64_t i = (int64_t)gy * W + gx;
          wv = __ldcg(a.Wg + i);
          fv = __ldcg(w.flags + i);
        }
        s.R[hy * kRS + hx] = relay<MODE>(wv, fv, wv);
      }
    }
  }
#pragma unroll 12
  for (int idx = vec ? 34 * 34 : lane; idx < 34 * 34; idx += 32) {
    int hy = idx / 34, hx = idx - hy * 34;
    int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
    float wv = kInf, qv = 0.0f;
    uint8_t fv = FNODATA;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
      int64_t i = (int64_t)gy * W + gx;
      wv = __ldcg(a.Wg + i);  // L2: written by other SMs with no barrier in between
      if constexpr (MODE == 1) qv = a.q[i];
      fv = __ldcg(w.flags + i);
    }
    s.R[hy * kRS + hx] = relay<MODE>(wv, fv, MODE == 1 ? qv : wv);
    if (hx >= 1 && hx <= kTile && hy >= 1 && hy <= kTile) {
      if constexpr (MODE == 1) s.WQ[(hy - 1) * kWS + hx - 1] = make_float2(wv, qv);
      s.F[(hy - 1) * kFS + hx - 1] = fv;
    }
  }
  if constexpr (MODE != 1) cp_async_wait();
  unsigned int clean0 = 0;  // MODE 2: this lane's column, rows clean when staged
  if constexpr (MODE == 2) {
    // Clean relays of the halo: strips of 34 cells (row above, row below,
    // column left, column right), flags read again from L2, after the
    // levels and a fence.  A clean mark holds for the level it was derived
    // at; a write-back that lowers a clean cell's level (withdrawing or
    // re-deriving its mark) stores the flags, fences, then stores the level.
    // So a halo level read above that is already the new one comes with a
    // flag read here that is at least as new: never a stale clean mark with
    // a lower level, which could mark a neighbour clean too low.
    __threadfence();
    for (int k = lane; k < 4 * 34; k += 32) {
      const int strip = k / 34, j = k - strip * 34;
      const int hx = strip < 2 ? j : (strip == 2 ? 0 : 33);
      const int hy = strip < 2 ? (strip == 0 ? 0 : 33) : j;
      const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
      uint8_t fv = FNODATA;
      if (gx >= 0 && gx < W && gy >= 0 && gy < H) fv = __ldcg(w.flags + (int64_t)gy * W + gx);
      s.HC[strip][j] = (fv & (FCLEAN | FNONPASS | FNODATA)) == FCLEAN;
    }
    __syncwarp();
#pragma unroll 8
    for (int y = 0; y < kTile; y++)
      clean0 |= (s.F[y * kFS + lane] & FCLEAN) ? (1u << y) : 0u;
  }
  __syncwarp();
  const long long c1 = clock64();
  // Sweeps.  Each of the four directions reads only the three neighbours on
  // the side it comes from: down (row by row from the top) the row above,
  // up the row below, right the column to the left, left the column to the
  // right; a round is a vertical phase (down and up interleaved) and a
  // horizontal phase (right and left interleaved).  Together the four read
  // all 8 neighbours.  Warp-uniform masks hold the rows (pd, pu) and
  // columns (pr, pl) each direction still has to evaluate; a bit is cleared
  // when its row or column is evaluated.  A change at (x, y) sets the
  // directions that read it: row y+1 down, y-1 up, column x+1 right, x-1
  // left.  A bit set for a row or column its sweep has already passed stays
  // set into the next round.  When all four masks are empty, every cell has
  // been evaluated against each neighbour since that neighbour last changed:
  // the tile is at a fixpoint for its halo.
  // A tile that converged on an earlier visit is a fixpoint for its old halo:
  // only the rows and columns that read the halo need evaluating first.
  // (written by whichever warp processed the tile last, maybe on another SM)
  const bool revisit = ((volatile uint8_t*)w.tconv)[t] != 0;
  const int max_rounds = w.max_rounds;
  unsigned int pd = revisit ? 1u : ~0u, pu = revisit ? 0x80000000u : ~0u;
  unsigned int pr = pd, pl = pu;
  unsigned int dc = 0;  // this lane's column: rows of the cells changed on this visit
  int rounds = 0;
  // A step evaluates both of its rows (columns) when either is pending: the
  // two cells are loaded before either is stored, so their dependency chains
  // overlap.  Extra evaluations are harmless (any relaxation step is), and
  // at the crossing (k = 16) a cell that reads the other's old value is
  // re-evaluated through the masks like any other.
  for (; rounds < max_rounds && (pd | pu | pr | pl); rounds++) {
    // Step k evaluates row k (down) and row 31 - k (up); steps with neither
    // pending are skipped by a find-first-set over both masks.
    for (int k = 0; k < kTile; k++) {
      const unsigned int m = (pd | __brev(pu)) >> k;
      if (!m) break;
      k += __ffs(m) - 1;
      const int d = k, u = kTile - 1 - k;
      const unsigned int bd = 1u << d, bu = 1u << u;
      pd &= ~bd;
      pu &= ~bu;
      const CellEval ed = cell_load(s, lane, d, row3_min(s, lane, d));
      const CellEval eu = cell_load(s, lane, u, row3_min(s, lane, u + 2));
      const bool cd = cell_store<MODE>(s, lane, d, ed);
      const bool cu = cell_store<MODE>(s, lane, u, eu);
      dc |= (cd ? bd : 0u) | (cu ? bu : 0u);
      const unsigned int b1 = __ballot_sync(0xffffffffu, cd), b2 = __ballot_sync(0xffffffffu, cu);
      if (b1 | b2) {
        const unsigned int rows = (b1 ? bd : 0u) | (b2 ? bu : 0u), cols = b1 | b2;
        pd |= rows << 1;
        pu |= rows >> 1;
        pr |= cols << 1;
        pl |= cols >> 1;
      }
      __syncwarp();
    }
    for (int k = 0; k < kTile; k++) {
      const unsigned int m = (pr | __brev(pl)) >> k;
      if (!m) break;
      k += __ffs(m) - 1;
      const int l = k, r = kTile - 1 - k;
      const unsigned int bl = 1u << l, br = 1u << r;
      pr &= ~bl;
      pl &= ~br;
      const CellEval el = cell_load(s, l, lane, col3_min(s, l, lane));
      const CellEval er = cell_load(s, r, lane, col3_min(s, r + 2, lane));
      const bool cl = cell_store<MODE>(s, l, lane, el);
      const bool cr = cell_store<MODE>(s, r, lane, er);
      const unsigned int b1 = __ballot_sync(0xffffffffu, cl), b2 = __ballot_sync(0xffffffffu, cr);
      if (b1 | b2) {
        const unsigned int cols = (b1 ? bl : 0u) | (b2 ? br : 0u), rows = b1 | b2;
        pr |= cols << 1;
        pl |= cols >> 1;
        pd |= rows << 1;
        pu |= rows >> 1;
        dc |= (lane == l ? b1 : 0u) | (lane == r ? b2 : 0u);
      }
      __syncwarp();
    }
  }
  const bool capped = (pd | pu | pr | pl) != 0;
  // Each round of the clean pass marks at least one more cell, so 1024
  // rounds always reach its fixpoint.
  if constexpr (MODE == 2) dc |= clean_pass(s, lane, kTile * kTile);
  const long long c2 = clock64();
  if (lane == 0) {
    w.tconv[t] = capped ? 0 : 1;
    st.tiles++;
    st.rounds += (unsigned int)rounds;
  }
  // Write back the changed cells, row by row (coalesced); note which
  // borders changed.  Cells outside the grid are NODATA and never change.
  // With clean marks, a changed cell that was clean when staged may have a
  // lower level and a withdrawn or re-derived mark: flags first, a fence,
  // then the levels (the readers' side is in the staging above).
  const unsigned int rows_changed = __reduce_or_sync(0xffffffffu, dc);
  bool flags_first = false;
  if constexpr (MODE == 2) flags_first = __any_sync(0xffffffffu, (dc & clean0) != 0u);
  if (flags_first) {
    for (unsigned int rows = rows_changed; rows; rows &= rows - 1) {
      const int y = __ffs(rows) - 1;
      if ((dc >> y) & 1u) w.flags[(int64_t)(y0 + y) * W + (x0 + lane)] = s.F[y * kFS + lane];
    }
    __threadfence();
  }
  for (unsigned int rows = rows_changed; rows; rows &= rows - 1) {
    const int y = __ffs(rows) - 1;
    if ((dc >> y) & 1u) {
      const int64_t i = (int64_t)(y0 + y) * W + (x0 + lane);
      a.Wg[i] = staged_w(s, lane, y);
      if (!flags_first) w.flags[i] = s.F[y * kFS + lane];
    }
  }
  // The write-back (and a "not converged" mark) is visible before any
  // neighbour is queued or the tile's state changes.  A visit that changed
  // nothing wrote nothing and queues no one.
  if (rows_changed) __threadfence();
  const unsigned int dl = __shfl_sync(0xffffffffu, dc, 0), dr = __shfl_sync(0xffffffffu, dc, 31);
  // 1 L, 2 R, 4 T, 8 B, 16 TL, 32 TR, 64 BL, 128 BR
  const unsigned int sides = (dl ? 1u : 0u) | (dr ? 2u : 0u) | ((rows_changed & 1u) ? 4u : 0u) |
                             ((rows_changed >> 31) ? 8u : 0u) | ((dl & 1u) ? 16u : 0u) |
                             ((dr & 1u) ? 32u : 0u) | ((dl >> 31) ? 64u : 0u) |
                             ((dr >> 31) ? 128u : 0u);
  // Every cell final?  Only a change can make it so after the first visit: a
  // later visit that changed nothing leaves the answer of the visit before.
  bool done = false;
  if (rows_changed || !revisit) {
    bool fin = true;
    for (int idx = lane; idx < kTile * kTile; idx += 32) {
      const uint8_t f = s.F[(idx >> 5) * kFS + (idx & 31)];
      fin &= (f & (FNODATA | FOUTLET | FBELOW)) != 0;
      // With clean marks, a cell that may still turn clean is not final.
      if (MODE == 2) fin &= (f & (FNODATA | FCLEAN)) != 0;
    }
    done = __all_sync(0xffffffffu, fin);
  }
  // Lanes 0..8 queue self (if capped) and the 8 neighbours whose halo changed.
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
    int nx = tx + dx, ny = ty + dy;
    if (want && nx >= 0 && ny >= 0 && nx < w.tiles_x && ny < w.tiles_y)
      enqueue(w, ny * w.tiles_x + nx);
  }
  __syncwarp();
  if (lane == 0) {
    const long long c3 = clock64();
    st.kload += (unsigned int)((c1 - c0) >> 10);
    st.ksweep += (unsigned int)((c2 - c1) >> 10);
    st.kstore += (unsigned int)((c3 - c2) >> 10);
  }
  return done;
}

// Lock-free union-find over the undecided cells (labels in w.aux): links
// always point to a smaller cell index, so no cycle can form; roots are
// hooked with CAS, paths halved with plain stores.  Bounded loops.
__device__ __forceinline__ uint32_t uf_find(uint32_t* lab, uint32_t x) {
  for (int it = 0; it < (1 << 20); it++) {
    uint32_t p = ((volatile uint32_t*)lab)[x];
    if (p == x) return x;
    uint32_t g = ((volatile uint32_t*)lab)[p];
    if (g != p) lab[x] = g;
    x = p;
  }
  return x;
}

// The root without path halving: the flattening pass writes each cell's
// root while other threads walk the same paths, and a halving store that
// landed after such a write would replace the root by an ancestor below
// it -- leaving a cell labelled with a non-root, outside its component's
// minimum.  Plain reads only, so every store of that pass is a root.
__device__ __forceinline__ uint32_t uf_root(const uint32_t* lab, uint32_t x) {
  for (int it = 0; it < (1 << 20); it++) {
    const uint32_t p = ((const volatile uint32_t*)lab)[x];
    if (p == x) return x;
    x = p;
  }
  return x;
}

__device__ __forceinline__ bool uf_unite(uint32_t* lab, uint32_t a, uint32_t b) {
  for (int it = 0; it < (1 << 16); it++) {
    uint32_t ra = uf_find(lab, a), rb = uf_find(lab, b);
    if (ra == rb) return true;
    if (ra > rb) { uint32_t t = ra; ra = rb; rb = t; }
    if (atomicCAS(&lab[rb], rb, ra) == rb) return true;
  }
  return false;
}

// One warp: process queued tiles until no tile is queued or being processed
// anywhere.  During a drain only a warp processing a tile can queue one,
// and that tile keeps `pending` above 0, so pending == 0 means no push can
// come: a ticket still waiting then is abandoned (head and tail are reset
// after the drain).  False on an error or a wait limit.
template <int MODE>
__device__ bool drain(WarpSmem<MODE>& s, const FloodArgs& a, int lane, int ntiles) {
  const FillWork& w = a.w;
  volatile unsigned int* vs = w.scal;
  const unsigned int visit_cap = 1000u * (unsigned int)min(ntiles, 4000000);
  long long ticket = -1;
  unsigned int ns = 32;
  VisitStats st;
  bool ok = true;
  long long idle_from = -1;  // clock when this warp last found no tile (-1: busy)
  for (long long idle = 0;;) {
    int t = -1;
    if (lane == 0) t = tq_try_dequeue(fill_queue(w), &ticket);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= 0) {
      if (lane == 0 && idle_from >= 0) st.kidle += (unsigned int)((clock64() - idle_from) >> 10);
      idle_from = -1;
      const bool done = process_tile<MODE>(s, a, t, lane, st);
      if (lane == 0) {
        tq_finish(fill_queue(w), t, done);
        if (st.tiles >= 64) flush_stats<MODE>(w, st, a.stage == 3);
      }
      __syncwarp();
      idle = 0;
      ns = 32;
      continue;
    }
    if (vs[S_ERR]) {
      ok = false;
      break;
    }
    if (vs[S_PENDING] == 0u) break;
    const bool idle_limit = ++idle > (1LL << 24);
    if (idle_limit || vs[(MODE == 1 || a.stage == 3) ? S_TILES_B : S_TILES_A] > visit_cap) {
      if (lane == 0) atomicCAS((int*)(w.scal + S_ERR), 0, idle_limit ? 2 : 4);
      ok = false;
      break;
    }
    if (idle_from < 0) idle_from = clock64();
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
  }
  if (lane == 0) {
    if (idle_from >= 0) st.kidle += (unsigned int)((clock64() - idle_from) >> 10);
    flush_stats<MODE>(w, st, a.stage == 3);
  }
  __syncwarp();
  return ok;
}

template <int MODE, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 1)
fill_flood_kernel(FloodArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpSmem<MODE>& s = reinterpret_cast<WarpSmem<MODE>*>(smraw)[warp];
  const FillWork& w = a.w;
  const unsigned int nblocks = gridDim.x;
  const int gwarp = blockIdx.x * WARPS + warp, nwarps = gridDim.x * WARPS;
  const int ntiles = w.tiles_x * w.tiles_y;
  GridSync gs{w.scal + S_BAR_COUNT, w.scal + S_BAR_GEN, (int*)(w.scal + S_ERR)};
  volatile unsigned int* vs = w.scal;
  const int p0 = (int)vs[S_PASS] + 2;
  int p = p0;
  int ph = 0;
  const bool phases = MODE == 1 && a.stage == 2;
  const unsigned long long t_start = global_ns();
  // Seed the queue with the tiles that hold a relaying outlet (a tile
  // without one cannot change before a neighbour does, which queues it),
  // one 2x2 parity class of tiles after another with a grid barrier in
  // between, so the ring holds them class by class.  Tiles taken at the
  // same time are then rarely neighbours, and each class starts from the
  // finished borders of the classes before it: in a CPU simulation of the
  // queue (2048^2 realization, 1/29 of the tiles in flight) this took the
  // visits per tile from 3.19 in plain tile order to 2.68.
  bool go = true;
  for (int c = 0; c < 4 && go && !phases; c++) {
    for (int i = gwarp; i < ntiles; i += nwarps) {
      const int tx = i % w.tiles_x, ty = i / w.tiles_x;
      if (lane == 0 && ((tx & 1) | ((ty & 1) << 1)) == c && w.tseed[i]) enqueue(w, i);
    }
    go = grid_barrier(gs, nblocks);
  }
  while (go) {
    const bool drained = drain<MODE>(s, a, lane, ntiles);
    if (!grid_barrier(gs, nblocks) || !drained) break;
    {
      if (!phases) break;  // flood A, or flood B's main drain
      // The queue is empty (abandoned tickets aside): restart its positions.
      // No push comes before the next grid barrier.
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        vs[S_HEAD] = 0u;
        vs[S_TAIL] = 0u;
      }
      // ---- confirmation phase ----
      // Flood A gave a lower bound (W_A in aux, FBELOWA), flood B an upper
      // bound (Wg, FBELOW).  Where they agree the cell is final; the
      // undecided cells (listed in cand, labelled by component in aux by
      // the kernels between the two flood B launches) form 8-connected
      // components that no later change can leave, so each component takes
      // its own phase minimum.
      const int64_t tid0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
      const int64_t tstride = (int64_t)gridDim.x * blockDim.x;
      const unsigned int nu = vs[S_CAND];
      if (blockIdx.x == 0 && threadIdx.x == 0) vs[S_PEND + (ph + 1) % 3] = 0u;
      for (int64_t j = tid0; j < nu; j += tstride) {
        const uint32_t c = w.cand[j], r = w.aux[c];
        if (r == c) w.cmin[c] = 0xffffffffu;
        // Every label is a root: a cell labelled otherwise would take a
        // minimum nothing resets.
        if (ph == 0 && w.aux[r] != r) atomicCAS((int*)(w.scal + S_ERR), 0, 6);
      }
      if (!grid_barrier(gs, nblocks)) break;
      // Flags and levels were written by other SMs' drains, the minima by
      // atomics: all are read from L2 (an L1 line could hold an older value
      // across the grid barrier).
      unsigned int pend = 0, npend = 0;
      for (int64_t j = tid0; j < nu; j += tstride) {
        uint32_t c = w.cand[j];
        uint8_t f = __ldcg(w.flags + c);
        if ((f & FNONPASS) && !(f & (FCONF | FBELOW))) {
          float wv = __ldcg(a.Wg + c);
          if (wv < kInf) {
            atomicMin(&w.cmin[w.aux[c]], float_to_ordered(wv));
            pend = 1;
            npend++;
          }
        }
      }
      npend = __reduce_add_sync(0xffffffffu, npend);
      if (lane == 0 && npend) atomicAdd(&w.scal[S_DBG], npend);
      pend = __reduce_or_sync(0xffffffffu, pend);
      if (lane == 0 && pend) atomicOr(&w.scal[S_PEND + ph % 3], 1u);
      if (!grid_barrier(gs, nblocks)) break;
      if (vs[S_PEND + ph % 3] == 0u) break;
      // Each phase confirms at least one cell of every component with a
      // pending cell (the one holding its minimum level), so there are at
      // most as many phases as undecided cells.
      if (ph > (int)min(nu, 0x7fffff00u) + 8) {
        // Record one pending cell whose level is its component's recorded
        // minimum: [26] cell, [27] level, [28] q, [29] the minimum read
        // back, [30] its label, [31] the label's own label ([24] pending
        // cells counted over the phases, [25] confirmations of the last).
        for (int64_t j = tid0; j < nu; j += tstride) {
          const uint32_t c = w.cand[j];
          const uint8_t f = __ldcg(w.flags + c);
          if (!(f & FNONPASS) || (f & (FCONF | FBELOW))) continue;
          const float wv = __ldcg(a.Wg + c);
          const uint32_t r = w.aux[c];
          const unsigned int mo = __ldcg(w.cmin + r);
          if (wv < kInf && float_to_ordered(wv) == mo &&
              atomicCAS(&w.scal[S_DBG + 2], 0u, c + 1u) == 0u) {
            w.scal[S_DBG + 3] = __float_as_uint(wv);
            w.scal[S_DBG + 4] = __float_as_uint(a.q[c]);
            w.scal[S_DBG + 5] = mo;
            w.scal[S_DBG + 6] = r;
            w.scal[S_DBG + 7] = w.aux[r];
          }
        }
        if (threadIdx.x == 0) atomicCAS((int*)(w.scal + S_ERR), 0, 5);
        break;
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) w.scal[S_DBG + 1] = 0u;
      if (!grid_barrier(gs, nblocks)) break;
      unsigned int nconf = 0;
      for (int64_t j = tid0; j < nu; j += tstride) {
        uint32_t c = w.cand[j];
        uint8_t f = __ldcg(w.flags + c);
        if (!(f & FNONPASS) || (f & (FCONF | FBELOW))) continue;
        const unsigned int mo = __ldcg(w.cmin + w.aux[c]);
        if (mo == 0xffffffffu || !(a.q[c] <= ordered_to_float(mo))) continue;
        nconf++;
        w.flags[c] = f | FCONF;
        if (__ldcg(a.Wg + c) < kInf) {
          // The cell now relays: every tile whose halo holds it must rerun.
          int cx = (int)(c % (uint32_t)w.W), cy = (int)(c / (uint32_t)w.W);
          w.tconv[(cy / kTile) * w.tiles_x + cx / kTile] = 0;  // its neighbours inside must rerun
          int tx0 = max(cx - 1, 0) / kTile, tx1 = min(cx + 1, w.W - 1) / kTile;
          int ty0 = max(cy - 1, 0) / kTile, ty1 = min(cy + 1, w.H - 1) / kTile;
          for (int ty = ty0; ty <= ty1; ty++)
            for (int tx = tx0; tx <= tx1; tx++) enqueue(w, ty * w.tiles_x + tx);
        }
      }
      nconf = __reduce_add_sync(0xffffffffu, nconf);
      if (lane == 0 && nconf) atomicAdd(&w.scal[S_DBG + 1], nconf);
      ph++;
      if (!grid_barrier(gs, nblocks)) break;
    }
    p++;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    vs[S_PASS] = (unsigned int)p;
    const unsigned int us = (unsigned int)((global_ns() - t_start) / 1000);
    if (MODE != 1 && a.stage == 3) {
      vs[S_US_B] = us;
    } else if (MODE != 1) {
      vs[S_PASSES_A] = (unsigned int)(p - p0 + 1);
      vs[S_US_A] = us;
    } else if (!phases) {
      vs[S_PASSES_B] = (unsigned int)(p - p0 + 1);
      vs[S_US_B] = us;
    } else {
      vs[S_PHASES] = (unsigned int)ph;
      vs[S_US_P] = us;
    }
  }
}

// Cells per thread of the elementwise fill kernels (fewer, longer blocks).
constexpr int kCellsPerThread = 4;

__global__ void fill_init_kernel(const float* __restrict__ q, float* __restrict__ Wg,
                                 uint8_t* __restrict__ F, const unsigned int* minslot,
                                 uint8_t* __restrict__ tseed, int tiles_x, int W, int H,
                                 int slab_h, float nodata, int check_only) {
  // Block rows step over the grid's rows (no division to find a cell's x
  // and y); kCellsPerThread cells a block-width apart per thread
  // (coalesced).  A stack of realizations takes each slab's borders and
  // minimum.
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
  const int slab = y / slab_h, ys = y - slab * slab_h;
  const float minE = ordered_to_float(minslot[slab]);
  // After a fused front: its set-up assumed minE = 0.
  if (check_only && minE == 0.0f) continue;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; k++) {
    const int x = (blockIdx.x * kCellsPerThread + k) * blockDim.x + threadIdx.x;
    if (x >= W) break;
    const int64_t i = (int64_t)y * W + x;
    const float qv = q[i];
    const uint8_t f =
        fill_init_flags(qv, nodata, minE, x == 0 || ys == 0 || x == W - 1 || ys == slab_h - 1);
    F[i] = f;
    Wg[i] = (f & (FNODATA | FOUTLET)) ? qv : kInf;
    if ((f & FOUTLET) && !(f & FNONPASS)) tseed[(y / kTile) * tiles_x + x / kTile] = 1;
  }
  }
}

// Exact mode (the reference's GPU fill, src/pitfilling/PitFillingAlgorithmGPUCUDA.cu:201-231):
// NODATA cells keep NODATA and never relay; border cells and cells equal to
// 0 are outlets that keep their elevation and relay it; every other cell
// starts at +inf, or at a warm-start value no lower than its elevation.
__global__ void fill_init_exact_kernel(const float* __restrict__ v, float* __restrict__ Wg,
                                       uint8_t* __restrict__ F, const float* __restrict__ warm,
                                       uint8_t* __restrict__ tseed, int tiles_x, int W, int H,
                                       float nodata) {
  const int y = blockIdx.y;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; k++) {
    const int x = (blockIdx.x * kCellsPerThread + k) * blockDim.x + threadIdx.x;
    if (x >= W) break;
    const int64_t i = (int64_t)y * W + x;
    const float e = v[i];
    uint8_t f = 0;
    if (e == nodata) f = FNODATA;
    else if (x == 0 || y == 0 || x == W - 1 || y == H - 1 || e == 0.0f) f = FOUTLET | FCLEAN;
    F[i] = f;
    Wg[i] = f ? e : (warm ? fmaxf(warm[i], e) : kInf);
    if (f & FOUTLET) tseed[(y / kTile) * tiles_x + x / kTile] = 1;
  }
}

// Verification of a warm-started exact fill.  The warm flood keeps clean
// marks: in exact mode every reached cell relays, so a marked cell's level
// is supported -- a chain of relays from an outlet reaches it with no step
// above its level -- and such a level is never below the exact fill (the
// chain is a path whose highest elevation it covers).  At the flood's
// fixpoint no cell is above the exact fill either (induction along its
// optimal path), so a supported cell holds the answer.  Every other cell
// (started too low, pulled down by one that was, or unreached) restarts
// from +inf and marks its tile for the repair flood; with every start an
// upper bound again, the repair flood ends at the exact fill.  Four
// consecutive cells per thread; the flags are workspace (aligned).  Also
// resets the work queue's positions.
__global__ void fill_unsupported_kernel(float* __restrict__ Wg, uint8_t* __restrict__ F,
                                        uint8_t* __restrict__ tseed, unsigned int* scal,
                                        int tiles_x, int W, int64_t n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_HEAD] = 0u;
    scal[S_TAIL] = 0u;
    scal[S_PENDING] = 0u;
  }
  const int64_t b4 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  unsigned int reset = 0;
  if (b4 < n) {
    uint8_t fv[4];
    if (b4 + 4 <= n) {
      const uchar4 f4 = *reinterpret_cast<const uchar4*>(F + b4);
      fv[0] = f4.x; fv[1] = f4.y; fv[2] = f4.z; fv[3] = f4.w;
    } else {
#pragma unroll
      for (int k = 0; k < 4; k++) fv[k] = b4 + k < n ? F[b4 + k] : FNODATA;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint8_t f = fv[k];
      if (f & (FNODATA | FOUTLET | FCLEAN)) continue;
      const int64_t i = b4 + k;
      Wg[i] = kInf;
      F[i] = f & (uint8_t)~FBELOW;
      const int y = (int)(i / W), x = (int)(i - (int64_t)y * W);
      tseed[(y / kTile) * tiles_x + x / kTile] = 1;
      reset++;
    }
  }
  reset = __reduce_add_sync(0xffffffffu, reset);
  if ((threadIdx.x & 31) == 0 && reset) atomicAdd(&scal[S_RESET], reset);
}

// Cells no outlet reaches keep the reference's initial value.
__global__ void fill_final_exact_kernel(float* __restrict__ Wg, int64_t n) {
#pragma unroll
  for (int k = 0; k < kCellsPerThread; k++) {
    const int64_t i = ((int64_t)blockIdx.x * kCellsPerThread + k) * blockDim.x + threadIdx.x;
    if (i < n && Wg[i] == kInf) Wg[i] = 99990000.0f;
  }
}

// Between the floods.  A clean cell keeps flood A's value and below-q flag,
// which flood B would give it too (every value flood B relays is a passable
// level, so a non-passable cell's incoming level never equals its q, and a
// clean cell's level is reached by a path flood B keeps); nothing of it is
// written.  Every other cell keeps flood A's result (a lower bound) in aux
// and FBELOWA, is confirmed when non-passable and reached at a level >= q,
// restarts from +inf and marks its tile for flood B (tseed).  Four
// consecutive cells per thread; only the flags of clean cells are read.
// Also resets the work queue.
__global__ void fill_classify_kernel(float* __restrict__ Wg, uint8_t* __restrict__ F,
                                     uint32_t* __restrict__ aux, unsigned int* scal,
                                     uint8_t* __restrict__ tseed, int tiles_x, int W, int64_t n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_HEAD] = 0u;
    scal[S_TAIL] = 0u;
    scal[S_PENDING] = 0u;
  }
  const int64_t b4 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (b4 >= n) return;
  uint8_t fv[4];
  if (b4 + 4 <= n) {  // the flags are workspace: 256-byte aligned, b4 % 4 == 0
    const uchar4 f4 = *reinterpret_cast<const uchar4*>(F + b4);
    fv[0] = f4.x; fv[1] = f4.y; fv[2] = f4.z; fv[3] = f4.w;
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++) fv[k] = b4 + k < n ? F[b4 + k] : FNODATA;
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint8_t f = fv[k];
    if (f & (FNODATA | FOUTLET | FCLEAN)) continue;
    const int64_t i = b4 + k;
    const float wa = Wg[i];
    aux[i] = __float_as_uint(wa);
    if ((f & FNONPASS) && !(f & FBELOW) && wa < kInf) f |= FCONF;
    if (f & FBELOW) f |= FBELOWA;
    F[i] = f & (uint8_t)~FBELOW;
    Wg[i] = kInf;
    const int y = (int)(i / W), x = (int)(i - (int64_t)y * W);
    tseed[(y / kTile) * tiles_x + x / kTile] = 1;
  }
}

// Flood B's tile states: a tile without a cell to recompute is done from
// the start (its cells hold flood B's values already); the others are idle.
__global__ void fill_tile_states_kernel(int* __restrict__ queued, const uint8_t* __restrict__ tseed,
                                        int ntiles) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ntiles) queued[t] = tseed[t] ? kIdle : kDone;
}

// Between flood B's two launches: the undecided cells -- flood A's lower
// bound (aux) and flood B's upper bound (Wg) differ in value, or in the
// blocked status of a non-passable cell -- are flagged FUNSURE, labelled
// with their own index and appended to the candidate list.  Only tiles that
// held a cell to recompute (tseed) are read: a clean cell kept flood A's
// value and flag.  One block per tile, one row segment of 4 cells per
// thread; the filled grid is the caller's and is read as float4 only when
// the row segment is 16-byte aligned.
__global__ void fill_undecided_kernel(const float* __restrict__ Wg, uint8_t* __restrict__ F,
                                      uint32_t* __restrict__ aux, uint32_t* __restrict__ cand,
                                      unsigned int* scal, const uint8_t* __restrict__ tseed,
                                      int tiles_x, int W, int H) {
  const int t = blockIdx.x;
  if (!tseed[t]) return;
  const int y = (t / tiles_x) * kTile + (int)(threadIdx.x >> 3);
  const int x = (t % tiles_x) * kTile + (int)(threadIdx.x & 7) * 4;
  if (y >= H || x >= W) return;
  const int64_t b4 = (int64_t)y * W + x;
  uint8_t fv[4];
  float wav[4], wbv[4];
  // b4 % 4 == 0 aligns the workspace arrays (256-byte aligned bases);
  // the caller's grid is checked on its own.
  if (x + 4 <= W && (b4 & 3) == 0 && ((uintptr_t)(Wg + b4) & 15u) == 0) {
    const uchar4 f4 = *reinterpret_cast<const uchar4*>(F + b4);
    const uint4 a4 = *reinterpret_cast<const uint4*>(aux + b4);
    const float4 w4 = *reinterpret_cast<const float4*>(Wg + b4);
    fv[0] = f4.x; fv[1] = f4.y; fv[2] = f4.z; fv[3] = f4.w;
    wav[0] = __uint_as_float(a4.x); wav[1] = __uint_as_float(a4.y);
    wav[2] = __uint_as_float(a4.z); wav[3] = __uint_as_float(a4.w);
    wbv[0] = w4.x; wbv[1] = w4.y; wbv[2] = w4.z; wbv[3] = w4.w;
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const bool in = x + k < W;
      fv[k] = in ? F[b4 + k] : FNODATA;
      wav[k] = in ? __uint_as_float(aux[b4 + k]) : 0.0f;
      wbv[k] = in ? Wg[b4 + k] : 0.0f;
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint8_t f = fv[k];
    // Clean cells agree by construction (their aux and FBELOWA are not kept).
    const bool unsure = !(f & (FNODATA | FOUTLET | FCLEAN)) &&
                        (wav[k] != wbv[k] ||
                         ((f & FNONPASS) && (((f & FBELOWA) != 0) != ((f & FBELOW) != 0))));
    const int64_t i = b4 + k;
    if (unsure) {
      F[i] = f | FUNSURE;
      aux[i] = (uint32_t)i;
    }
    const unsigned int pos = warp_append(&scal[S_CAND], unsure);
    if (unsure) cand[pos] = (uint32_t)i;
  }
}

// Union of undecided neighbours (W, NW, N, NE: each pair once) into
// 8-connected components; labels in aux.
__global__ void fill_unite_kernel(const uint32_t* __restrict__ cand, unsigned int* scal,
                                  const uint8_t* __restrict__ F, uint32_t* aux, int W) {
  const unsigned int nu = ((volatile unsigned int*)scal)[S_CAND];
  bool ok = true;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nu;
       j += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cand[j];
    const int cx = (int)(c % (uint32_t)W), cy = (int)(c / (uint32_t)W);
    for (int k = 0; k < 4; k++) {
      const int nx = cx + (k == 0 ? -1 : k - 2), ny = cy + (k == 0 ? 0 : -1);
      if (nx < 0 || ny < 0 || nx >= W) continue;
      const uint32_t nb = (uint32_t)ny * (uint32_t)W + (uint32_t)nx;
      if (F[nb] & FUNSURE) ok &= uf_unite(aux, c, nb);
    }
  }
  if (!ok) atomicCAS((int*)(scal + S_ERR), 0, 6);
}

// Every undecided cell's label becomes its component's root.
__global__ void fill_flatten_kernel(const uint32_t* __restrict__ cand,
                                    const unsigned int* scal, uint32_t* aux) {
  const unsigned int nu = ((const volatile unsigned int*)scal)[S_CAND];
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nu;
       j += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cand[j];
    aux[c] = uf_root(aux, c);
  }
}

// Cells no outlet reached keep q.  Such a cell was never clean (a clean
// cell's level is finite and flood B keeps it), so only the tiles flood B
// worked on (tseed) are read: one block per tile, a row segment of 4 cells
// per thread.
__global__ void fill_final_kernel(const float* __restrict__ q, float* __restrict__ Wg,
                                  const uint8_t* __restrict__ tseed, int tiles_x, int W, int H) {
  const int t = blockIdx.x;
  if (!tseed[t]) return;
  const int y = (t / tiles_x) * kTile + (int)(threadIdx.x >> 3);
  const int x0 = (t % tiles_x) * kTile + (int)(threadIdx.x & 7) * 4;
  if (y >= H) return;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int x = x0 + k;
    if (x >= W) break;
    const int64_t i = (int64_t)y * W + x;
    if (Wg[i] == kInf) Wg[i] = q[i];
  }
}

__global__ void quantize_min_kernel(float* __restrict__ d, int64_t n, float nodata,
                                    unsigned int* minslot) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float m = kInf;
  if (i < n) {
    float q = fill_quantize(d[i], nodata);
    d[i] = q;
    m = q;
  }
  unsigned int o = float_to_ordered(m);
  o = __reduce_min_sync(0xffffffffu, o);
  // One atomic per block (same-address atomics from every warp queue up).
  __shared__ unsigned int bmin;
  if (threadIdx.x == 0) bmin = 0xffffffffu;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) atomicMin(&bmin, o);
  __syncthreads();
  if (threadIdx.x == 0) atomicMin(minslot, bmin);
}

__global__ void fill_scalars_kernel(unsigned int* s) {
  for (int i = threadIdx.x; i < S_SIZE; i += blockDim.x)
    s[i] = (i == S_MIN || (i >= S_M && i < S_M + 3)) ? 0xffffffffu : 0u;
}

template <int MODE, int WARPS>
static cageo_status launch_flood_warps(const FloodArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(WarpSmem<MODE>) * WARPS;
  auto fn = fill_flood_kernel<MODE, WARPS>;
  CAGEO_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  static PerDevice resident;  // one table per instantiation
  int blocks = 0;
  cageo_status st = per_device(resident, &blocks, [&](int dev, int* v) -> cageo_status {
    return resident_blocks((const void*)fn, WARPS * 32, smem, dev, v);
  });
  if (st) return st;
  FloodArgs args = a;
  void* params[] = {&args};
  // No more blocks than the tiles can keep busy (small grids leave the
  // rest of the GPU idle instead of polling the work queue).
  const int ntiles = a.w.tiles_x * a.w.tiles_y;
  const int grid = std::max(1, std::min(blocks, (ntiles + WARPS - 1) / WARPS));
  CAGEO_CUDA(cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(WARPS * 32), params,
                                         smem, s));
  return CAGEO_OK;
}

bool fill_flood_warps_valid(int warps) { return warps == 16 || warps == 20 || warps == 22; }

template <int MODE>
static cageo_status launch_flood(const FloodArgs& a, cudaStream_t s) {
  if (MODE == 1) return launch_flood_warps<1, kWarpsB>(a, s);
  switch (a.w.flood_warps) {
    case 16: return launch_flood_warps<MODE == 1 ? 0 : MODE, 16>(a, s);
    case 20: return launch_flood_warps<MODE == 1 ? 0 : MODE, 20>(a, s);
    case 22: return launch_flood_warps<MODE == 1 ? 0 : MODE, 22>(a, s);
  }
  set_error("pit filling: %d warps per block is not one of 16, 20, 22", a.w.flood_warps);
  return CAGEO_ERR_ARGUMENT;
}

cageo_status fill_clear_seeds(const FillWork& w, cudaStream_t s) {
  CAGEO_CUDA(cudaMemsetAsync(w.tseed, 0, (size_t)w.tiles_x * w.tiles_y, s));
  return CAGEO_OK;
}

cageo_status fill_reset_scalars(const FillWork& w, cudaStream_t s) {
  fill_scalars_kernel<<<1, 32, 0, s>>>(w.scal);
  CAGEO_CUDA(cudaGetLastError());
  CAGEO_CUDA(cudaMemsetAsync(w.queued, 0, sizeof(int) * w.tiles_x * w.tiles_y, s));
  return CAGEO_OK;
}

cageo_status fill_run(const float* q, float* filled, const FillWork& w, float nodata,
                      cudaStream_t s) {
  const int64_t n = (int64_t)w.W * w.H;
  const unsigned blocks = (unsigned)((n + 256 * kCellsPerThread - 1) / (256 * kCellsPerThread));
  const size_t nt = (size_t)w.tiles_x * w.tiles_y;
  if (!w.front_init) CAGEO_CUDA(cudaMemsetAsync(w.tseed, 0, nt, s));
  const dim3 rows((unsigned)((w.W + 256 * kCellsPerThread - 1) / (256 * kCellsPerThread)),
                   (unsigned)w.H);
  // After a fused front, a few block rows check the slabs' minima and
  // exit (the set-up is redone only where a minimum is not 0).
  const dim3 init_rows(rows.x, std::min(rows.y, w.front_init ? 1024u : 65535u));
  fill_init_kernel<<<init_rows, 256, 0, s>>>(q, filled, w.flags,
                                             w.slab_min ? w.slab_min : w.scal + S_MIN, w.tseed,
                                             w.tiles_x, w.W, w.H, w.slab_h ? w.slab_h : w.H, nodata,
                                             w.front_init ? 1 : 0);
  CAGEO_CUDA(cudaGetLastError());
  FloodArgs a{q, filled, w};
  CAGEO_CUDA(cudaMemsetAsync(w.queued, 0, sizeof(int) * nt, s));  // all idle
  CAGEO_CUDA(cudaMemsetAsync(w.tconv, 0, nt, s));
  CAGEO_CUDA(cudaMemsetAsync(w.lists, 0xff, (2 * nt + kRingSlack) * sizeof(int), s));  // empty ring
  if (w.marks) CAGEO_CUDA(cudaEventRecord(w.marks[0], s));
  cageo_status st = launch_flood<2>(a, s);  // flood A with clean marks
  if (st) return st;
  if (w.marks) CAGEO_CUDA(cudaEventRecord(w.marks[1], s));
  CAGEO_CUDA(cudaMemsetAsync(w.tseed, 0, nt, s));
  const unsigned cblocks = (unsigned)((n + 4 * 256 - 1) / (4 * 256));
  fill_classify_kernel<<<cblocks, 256, 0, s>>>(filled, w.flags, w.aux, w.scal, w.tseed,
                                               w.tiles_x, w.W, n);
  fill_tile_states_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(w.queued, w.tseed,
                                                                       (int)nt);
  CAGEO_CUDA(cudaGetLastError());
  CAGEO_CUDA(cudaMemsetAsync(w.tconv, 0, nt, s));
  a.stage = 1;  // flood B's main drain, from the tiles holding a cell to recompute
  st = launch_flood<1>(a, s);
  if (st) return st;
  fill_undecided_kernel<<<(unsigned)nt, 256, 0, s>>>(filled, w.flags, w.aux, w.cand, w.scal,
                                                     w.tseed, w.tiles_x, w.W, w.H);
  const unsigned ublocks = (unsigned)std::min<int64_t>((n + 255) / 256, 2048);
  fill_unite_kernel<<<ublocks, 256, 0, s>>>(w.cand, w.scal, w.flags, w.aux, w.W);
  fill_flatten_kernel<<<ublocks, 256, 0, s>>>(w.cand, w.scal, w.aux);
  CAGEO_CUDA(cudaGetLastError());
  if (w.marks) CAGEO_CUDA(cudaEventRecord(w.marks[2], s));
  a.stage = 2;  // the confirmation phases
  st = launch_flood<1>(a, s);
  if (st) return st;
  if (w.marks) CAGEO_CUDA(cudaEventRecord(w.marks[3], s));
  fill_final_kernel<<<(unsigned)nt, 256, 0, s>>>(q, filled, w.tseed, w.tiles_x, w.W, w.H);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status fill_run_exact(const float* v, float* filled, const FillWork& w, float nodata,
                            const float* warm, cudaStream_t s) {
  const int64_t n = (int64_t)w.W * w.H;
  const unsigned blocks = (unsigned)((n + 256 * kCellsPerThread - 1) / (256 * kCellsPerThread));
  const size_t nt = (size_t)w.tiles_x * w.tiles_y;
  // A warm start may hold values above the answer anywhere: every tile is
  // visited on the first pass.
  CAGEO_CUDA(cudaMemsetAsync(w.tseed, warm ? 1 : 0, nt, s));
  const dim3 rows((unsigned)((w.W + 256 * kCellsPerThread - 1) / (256 * kCellsPerThread)),
                   (unsigned)w.H);
  fill_init_exact_kernel<<<rows, 256, 0, s>>>(v, filled, w.flags, warm, w.tseed, w.tiles_x, w.W,
                                              w.H, nodata);
  CAGEO_CUDA(cudaGetLastError());
  CAGEO_CUDA(cudaMemsetAsync(w.queued, 0, sizeof(int) * nt, s));  // all idle
  CAGEO_CUDA(cudaMemsetAsync(w.tconv, 0, nt, s));
  CAGEO_CUDA(cudaMemsetAsync(w.lists, 0xff, (2 * nt + kRingSlack) * sizeof(int), s));  // empty ring
  FloodArgs a{v, filled, w};
  if (!warm) {
    cageo_status st = launch_flood<0>(a, s);
    if (st) return st;
  } else {
    // Warm flood with support marks, then the unsupported cells restart
    // from +inf and the repair flood visits their tiles (the others keep
    // their states: a tile done in the warm flood holds the answer).
    cageo_status st = launch_flood<2>(a, s);
    if (st) return st;
    CAGEO_CUDA(cudaMemsetAsync(w.tseed, 0, nt, s));
    const unsigned ublocks = (unsigned)((n + 4 * 256 - 1) / (4 * 256));
    fill_unsupported_kernel<<<ublocks, 256, 0, s>>>(filled, w.flags, w.tseed, w.scal,
                                                    w.tiles_x, w.W, n);
    CAGEO_CUDA(cudaGetLastError());
    CAGEO_CUDA(cudaMemsetAsync(w.tconv, 0, nt, s));
    a.stage = 3;
    if ((st = launch_flood<0>(a, s))) return st;
  }
  fill_final_exact_kernel<<<blocks, 256, 0, s>>>(filled, n);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status fill_quantize_min(float* d, const FillWork& w, float nodata, cudaStream_t s) {
  const int64_t n = (int64_t)w.W * w.H;
  quantize_min_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, n, nodata, w.scal + S_MIN);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

// Adds a warm-started exact fill's counters to acc (device, 9 entries):
// fills, fills that restarted any cell, cells restarted, tile visits and
// sweep rounds of the warm flood, sweep rounds of the repair flood,
// microseconds of the warm and of the repair flood, repair tile visits.
__global__ void fill_warm_stats_kernel(const unsigned int* __restrict__ scal,
                                       unsigned long long* acc) {
  if (threadIdx.x != 0) return;
  const unsigned int reset = scal[S_RESET];
  acc[0] += 1;
  acc[1] += reset ? 1 : 0;
  acc[2] += reset;
  acc[3] += scal[S_TILES_A];
  acc[4] += scal[S_ROUNDS_A];
  acc[5] += scal[S_ROUNDS_B];
  acc[6] += scal[S_US_A];
  acc[7] += scal[S_US_B];
  acc[8] += scal[S_TILES_B];
}

cageo_status fill_accumulate_warm_stats(const FillWork& w, unsigned long long* acc,
                                        cudaStream_t s) {
  fill_warm_stats_kernel<<<1, 32, 0, s>>>(w.scal, acc);
  CAGEO_CUDA(cudaGetLastError());
  return CAGEO_OK;
}

cageo_status fill_check_status(const FillWork& w, int64_t* stats) {
  unsigned int h[S_SIZE];
  CAGEO_CUDA(cudaMemcpy(h, w.scal, sizeof(h), cudaMemcpyDeviceToHost));
  if (stats) {
    stats[0] = h[S_PASS];
    stats[1] = h[S_PHASES];
    stats[2] = h[S_PASSES_A];
    stats[3] = h[S_PASSES_B];
    stats[4] = h[S_US_A];
    stats[5] = h[S_US_B];
    stats[6] = h[S_US_P];
    stats[7] = h[S_TILES_A];
    stats[8] = h[S_ROUNDS_A];
    stats[9] = h[S_TILES_B];
    stats[10] = h[S_ROUNDS_B];
    stats[11] = h[S_KCYC_LOAD];
    stats[12] = h[S_KCYC_SWEEP];
    stats[13] = h[S_KCYC_STORE];
    stats[14] = h[S_KCYC_IDLE_A];
    stats[15] = h[S_KCYC_IDLE_B];
    stats[16] = h[S_RESET];
  }
  if (h[S_ERR]) {
    static const char* what[] = {"",
                                 "a grid-wide wait hit its limit",
                                 "a warp waited for a tile past its limit",
                                 "a tile's queue state kept changing",
                                 "the tile visits passed their limit",
                                 "the confirmation phases passed their limit",
                                 "the labels of the undecided cells are not settled roots"};
    const unsigned int e = h[S_ERR];
    if (e == 5)
      set_error("pit filling: %s (phases %u, undecided cells %u; pending counted %u, confirmed "
                "in the last phase %u; a minimum cell %u: level %.9g, q %.9g, minimum read %.9g, "
                "label %u, its label %u)",
                what[e], h[S_PHASES], h[S_CAND], h[S_DBG], h[S_DBG + 1], h[S_DBG + 2] - 1,
                __builtin_bit_cast(float, h[S_DBG + 3]), __builtin_bit_cast(float, h[S_DBG + 4]),
                ordered_to_float(h[S_DBG + 5]), h[S_DBG + 6], h[S_DBG + 7]);
    else
      set_error("pit filling: %s (pending tiles %u, phases %u, undecided cells %u)",
                e < 7 ? what[e] : "unknown error", h[S_PENDING], h[S_PHASES], h[S_CAND]);
    return CAGEO_ERR_NO_CONVERGENCE;
  }
  return CAGEO_OK;
}

}  // namespace cageo

using namespace cageo;

extern "C" cageo_status cageo_pitfill_exact_warm(const float* d_dem, const float* d_warm,
                                                 float* d_filled, int W, int H, float nodata_dem,
                                                 void* d_workspace, size_t workspace_bytes,
                                                 int64_t* h_stats, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_dem && d_filled && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(W <= 65535 && H <= 65535, "width and height must be <= 65535");
  CAGEO_CHECK_ARG(d_dem != d_filled && d_warm != d_filled, "the filled grid must not alias");
  Scratch ws;
  cageo_status st = ws.acquire(d_workspace, workspace_bytes, fill_workspace_bytes(W, H), stream);
  if (st) return st;
  FillWork w = fill_carve(ws.ptr, W, H);
  if ((st = fill_reset_scalars(w, stream))) return st;
  if ((st = fill_run_exact(d_dem, d_filled, w, nodata_dem, d_warm, stream))) return st;
  CAGEO_CUDA(cudaStreamSynchronize(stream));
  return fill_check_status(w, h_stats);
}

extern "C" size_t cageo_pitfill_workspace_size(int W, int H) {
  if (!valid_dims(W, H)) return 0;
  return fill_workspace_bytes(W, H);
}

extern "C" cageo_status cageo_pitfill(float* d_dem, float* d_filled, int W, int H,
                                      float nodata_dem, int mode, void* d_workspace,
                                      size_t workspace_bytes, cudaStream_t stream) {
  CAGEO_CHECK_ARG(d_dem && d_filled && valid_dims(W, H), "pointers and size");
  CAGEO_CHECK_ARG(W <= 65535 && H <= 65535, "width and height must be <= 65535");
  CAGEO_CHECK_ARG(d_dem != d_filled, "the filled grid must not alias the DEM");
  CAGEO_CHECK_ARG(mode == CAGEO_FILL_CPU_COMPAT || mode == CAGEO_FILL_EXACT, "fill mode");
  Scratch ws;
  cageo_status st = ws.acquire(d_workspace, workspace_bytes, fill_workspace_bytes(W, H), stream);
  if (st) return st;
  FillWork w = fill_carve(ws.ptr, W, H);
  if ((st = fill_reset_scalars(w, stream))) return st;
  if (mode == CAGEO_FILL_EXACT) {
    if ((st = fill_run_exact(d_dem, d_filled, w, nodata_dem, nullptr, stream))) return st;
  } else {
    if ((st = fill_quantize_min(d_dem, w, nodata_dem, stream))) return st;
    if ((st = fill_run(d_dem, d_filled, w, nodata_dem, stream))) return st;
  }
  CAGEO_CUDA(cudaStreamSynchronize(stream));
  return fill_check_status(w, nullptr);
}
