// cageo_oracle.cpp -- CPU restatement of the drainage reference's CPU stage
// algorithms (the `drainage --cpu` path of jsoksane/cageo).
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may
// load it.  The product (libcageo) never links or calls it.
//
// Every function restates one reference stage and cites the file:line it
// follows.  Arithmetic is plain IEEE float32 in the same order as the
// reference; build with -ffp-contract=off so no multiply-add is fused on any
// host (aarch64 g++ contracts by default).
//
// Parity of this restatement is pinned against the reference's own CPU stage
// templates compiled from source (oracle/_ref, see oracle/Makefile and
// oracle/ref_harness.cpp) through the golden fixtures in tests/golden/.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cstdio>
#include <queue>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Neighbour orders used by the reference.  Two different orders exist.
// Pit filling: src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:187-196
const int kFillDx[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
const int kFillDy[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
// Routing / border: N, NE, E, SE, S, SW, W, NW
// src/flowrouting/FlowRoutingAlgorithmCPUOpenMP.h:105-114,
// src/catchmentborder/CatchmentBorderAlgorithmCPUOpenMP.h:54-63
const int kD8Dx[8] = {0, 1, 1, 1, 0, -1, -1, -1};
const int kD8Dy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};

const int kOutside = -9999;  // src/flowtracing/FlowTracingCommon.h:18
const int kLake = -9998;     // src/flowtracing/FlowTracingCommon.h:19
const int kError = -9996;    // src/flowtracing/FlowTracingCommon.h:21
const float kSqrt2 = 1.41421356237309505f;  // src/flowrouting/FlowRoutingCommon.h:18
const int kPrec = 1000;  // src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:38

// toIndex / toElev: src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:56-66.
// float subtract, float multiply by 1000, truncate.  A negative product is
// outside the reference's defined behaviour; it is clamped to 0 here (the
// aarch64 conversion result) and the same clamp is used on the GPU.
inline size_t to_index(float v, float minE) {
  float p = (float)kPrec * (v - minE);
  if (!(p > 0.0f)) return 0;
  return (size_t)p;
}
inline float to_elev(size_t z, float minE) {
  return ((float)z) / (float)kPrec + minE;
}

}  // namespace

extern "C" {

// Convolution, Gaussian (separable) model: column pass into a buffer, then a
// row pass back.  Periodic wrap, ascending tap order, `sum += in*tap` with
// the sum starting at 0.0f.
// src/convolution/ConvolutionAlgorithmCPUOpenMP.h:80-103 (order),
// :164-206 (rows), :207-248 (cols).
// Requires r < W and r < H (the reference wraps by one period only).
int orc_convolve_separable(const float* in, float* out, int W, int H,
                           const float* taps, int r) {
  if (r < 0 || r >= W || r >= H) return -1;
  const int L = 2 * r + 1;
  std::vector<float> tmp((size_t)W * H);
#pragma omp parallel for
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      float sum = 0.0f;
      for (int t = 0; t < L; t++) {
        int sy = y - r + t;
        if (sy < 0) sy += H; else if (sy >= H) sy -= H;
        sum += in[(size_t)sy * W + x] * taps[t];
      }
      tmp[(size_t)y * W + x] = sum;
    }
  }
#pragma omp parallel for
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      float sum = 0.0f;
      for (int t = 0; t < L; t++) {
        int sx = x - r + t;
        if (sx < 0) sx += W; else if (sx >= W) sx -= W;
        sum += tmp[(size_t)y * W + sx] * taps[t];
      }
      out[(size_t)y * W + x] = sum;
    }
  }
  return 0;
}

// Convolution, exponential (full 2D) model: filterY outer, filterX inner.
// src/convolution/ConvolutionAlgorithmCPUOpenMP.h:105-162
int orc_convolve_2d(const float* in, float* out, int W, int H,
                    const float* filt, int r) {
  if (r < 0 || r >= W || r >= H) return -1;
  const int L = 2 * r + 1;
#pragma omp parallel for
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      float sum = 0.0f;
      for (int fy = 0; fy < L; fy++) {
        int sy = y - r + fy;
        if (sy < 0) sy += H; else if (sy >= H) sy -= H;
        for (int fx = 0; fx < L; fx++) {
          int sx = x - r + fx;
          if (sx < 0) sx += W; else if (sx >= W) sx -= W;
          sum += in[(size_t)sy * W + sx] * filt[fy * L + fx];
        }
      }
      out[(size_t)y * W + x] = sum;
    }
  }
  return 0;
}

// Realistic DEM: field[i] = dem[i] + field[i] where dem != NODATA (the
// output aliases the noise buffer, so NODATA cells keep their noise), then
// `x <= 0 && x != NODATA -> 1.0`.
// src/realisticdem/RealisticDemAlgorithm.h:49-70,
// src/utils/addsurfaces/AddSurfacesAlgorithmCPUOpenMP.h:36-56,
// src/utils/removenegativeelevationvalues/RemoveNegativeElevationsAlgorithmCPUOpenMP.h:34-48,
// aliasing at src/main.cpp:200-204.
void orc_realistic_dem(const float* dem, float* field, int64_t n,
                       float nodata_dem) {
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) {
    float d = dem[i];
    if (d != nodata_dem) field[i] = d + field[i];
  }
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) {
    float v = field[i];
    if (v <= 0.0f && v != nodata_dem) field[i] = 1.0f;
  }
}

// Search offsets within the bevel radius sorted by (d^2, y, x); the centre
// excluded.  src/streamburning/StreamBurningAlgorithm.h:140-167,
// src/streamburning/StreamBurningCommon.cpp:13-28.
static std::vector<std::pair<int, int>> burn_offsets(int bevel) {
  struct E { int d, x, y; };
  std::vector<E> v;
  for (int y = -bevel; y <= bevel; y++)
    for (int x = -bevel; x <= bevel; x++) {
      if (x == 0 && y == 0) continue;
      int d2 = x * x + y * y;
      if (d2 <= bevel * bevel) v.push_back({d2, x, y});
    }
  std::stable_sort(v.begin(), v.end(), [](const E& a, const E& b) {
    if (a.d != b.d) return a.d < b.d;
    if (a.y != b.y) return a.y < b.y;
    return a.x < b.x;
  });
  std::vector<std::pair<int, int>> out;
  for (auto& e : v) out.push_back({e.x, e.y});
  return out;
}

// Stream burning, in place.  Stream cells (streams != NODATA_stream) -> 0;
// then the first offset (nearest first) whose cell is a stream with a
// non-NODATA elevation scales the cell by dist/bevel.
// src/streamburning/StreamBurningAlgorithmCPUOpenMP.h:32-82.
// The reference runs this in place with OpenMP; its neighbour elevation
// check reads cells that other threads may have zeroed.  Run serially in
// raster order here; with NODATA_dem != 0 the outcome is the same.
int orc_stream_burn(float* dem, const float* streams, int W, int H, int bevel,
                    float nodata_dem, float nodata_stream) {
  if (bevel < 1 || bevel > 5) return -1;  // MAX_BEVEL_RADIUS, src/streamburning/StreamBurningCommon.h:17
  auto offs = burn_offsets(bevel);
  for (int sy = 0; sy < H; sy++) {
    for (int sx = 0; sx < W; sx++) {
      size_t idx = (size_t)sy * W + sx;
      if (streams[idx] != nodata_stream) dem[idx] = 0.0f;
      for (auto& o : offs) {
        int nx = sx + o.first, ny = sy + o.second;
        if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
        size_t n = (size_t)ny * W + nx;
        if (streams[n] != nodata_stream && dem[n] != nodata_dem) {
          float xd = (float)(sx - nx), yd = (float)(sy - ny);
          float dist = std::sqrt(xd * xd + yd * yd);
          dem[idx] = dem[idx] * (dist / (float)bevel);
          break;
        }
      }
    }
  }
  return 0;
}

// Pit filling, CPU path.  (i) quantize in place to 1/1000 m with the
// "never round a nonzero elevation to 0" rule; (ii) spill = q; minE/maxE;
// (iii) outlets = border cells and cells equal to 0 (STREAM) go to bucket
// toIndex(v,minE); (iv) buckets ascending, FIFO; a popped cell whose value
// is not toElev(z) is skipped; otherwise every unprocessed, non-NODATA
// neighbour gets max(cSpill, spill) and is queued.
// src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:84-109 (quantize),
// :111-118 (minmax, buckets), :120-144 (outlets), :162-237 (sweep).
// dem is overwritten with the quantized grid, as in the reference.
int orc_pitfill(float* dem, float* spill, int W, int H, float nodata) {
  const int64_t N = (int64_t)W * H;
  if (W < 1 || H < 1 || W > 65535 || H > 65535) return -1;
#pragma omp parallel for
  for (int64_t i = 0; i < N; i++) {
    float e = dem[i];
    if (e == nodata) continue;
    size_t qi = to_index(e, 0.0f);
    if (e != 0.0f && qi == 0) qi = 1;
    dem[i] = to_elev(qi, 0.0f);
  }
  std::memcpy(spill, dem, sizeof(float) * N);
  float minE = spill[0], maxE = spill[0];
  for (int64_t i = 1; i < N; i++) {
    if (spill[i] < minE) minE = spill[i];
    if (maxE < spill[i]) maxE = spill[i];
  }
  size_t nb = (size_t)((maxE - minE) * (float)kPrec + 1.0f);
  std::vector<std::vector<uint32_t>> Q(nb);
  std::vector<uint8_t> processed(N, 0);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      int64_t i = (int64_t)y * W + x;
      if (spill[i] == nodata) continue;
      if (x == 0 || x == W - 1 || y == 0 || y == H - 1 || spill[i] == 0.0f) {
        Q[to_index(spill[i], minE)].push_back((uint32_t)i);
        processed[i] = 1;
      }
    }
  for (size_t z = 0; z < nb; z++) {
    const float cSpill = to_elev(z, minE);
    std::vector<uint32_t>& q = Q[z];
    for (size_t k = 0; k < q.size(); k++) {  // FIFO; q may grow while scanned
      uint32_t c = q[k];
      if (cSpill != spill[c]) continue;
      int cx = (int)(c % (uint32_t)W), cy = (int)(c / (uint32_t)W);
      for (int n = 0; n < 8; n++) {
        int nx = cx + kFillDx[n], ny = cy + kFillDy[n];
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        int64_t ni = (int64_t)ny * W + nx;
        float ns = spill[ni];
        if (ns == nodata) continue;
        if (processed[ni]) continue;
        if (ns < cSpill) spill[ni] = cSpill;
        size_t nz = to_index(spill[ni], minE);
        if (nz < nb) Q[nz].push_back((uint32_t)ni);
        processed[ni] = 1;
      }
    }
    std::vector<uint32_t>().swap(q);
  }
  return 0;
}

// Flow routing, first pass + flat surfaces.  dir is 2 int8 per cell (dx,dy)
// like the reference's char2; flatdist as the reference's int grid.
// First pass: src/flowrouting/FlowRoutingAlgorithmCPUOpenMP.h:53-151.
// Flats: :153-249 (layer k assigns flatDist k from neighbours whose
// flatDist is -1 for k = 1, else k-1, and whose elevation is <= the cell's;
// the last matching neighbour in N..NW order wins).
void orc_flow_route(const float* dem, int8_t* dir, int* flatdist, int W,
                    int H) {
  const int64_t N = (int64_t)W * H;
  std::memset(dir, 0, 2 * N);
  std::memset(flatdist, 0, sizeof(int) * N);
  std::vector<uint32_t> flats;
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      int dxi = 0, dyi = 0;
      if (x == 0) dxi = -1; else if (x == W - 1) dxi = 1;
      if (y == 0) dyi = -1; else if (y == H - 1) dyi = 1;
      int64_t i = (int64_t)y * W + x;
      if (dxi != 0 || dyi != 0) {
        dir[2 * i] = (int8_t)dxi; dir[2 * i + 1] = (int8_t)dyi;
        flatdist[i] = -1;
        continue;
      }
      if (dem[i] == 0.0f) { flatdist[i] = -2; continue; }
      float steepest = 0.0f;
      int sdx = 0, sdy = 0;
      for (int n = 0; n < 8; n++) {
        int nx = x + kD8Dx[n], ny = y + kD8Dy[n];
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        float s = dem[i] - dem[(int64_t)ny * W + nx];
        if (s > 0.0f) {
          if (n % 2 == 1) s = s / kSqrt2;
          if (s > steepest) { steepest = s; sdx = kD8Dx[n]; sdy = kD8Dy[n]; }
        }
      }
      if (steepest > 0.0f) {
        dir[2 * i] = (int8_t)sdx; dir[2 * i + 1] = (int8_t)sdy;
        flatdist[i] = -1;
      } else {
        flats.push_back((uint32_t)i);
      }
    }
  }
  int look = -1;
  bool more = true;
  std::vector<uint32_t> next;
  std::vector<std::pair<uint32_t, int>> assign;
  while (more) {
    more = false;
    next.clear();
    assign.clear();
    for (uint32_t c : flats) {
      int cx = (int)(c % (uint32_t)W), cy = (int)(c / (uint32_t)W);
      int got = -1;
      for (int n = 0; n < 8; n++) {
        int nx = cx + kD8Dx[n], ny = cy + kD8Dy[n];
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        int64_t ni = (int64_t)ny * W + nx;
        if (flatdist[ni] == look && dem[ni] <= dem[c]) got = n;
      }
      if (got >= 0) {
        assign.push_back({c, got});
        more = true;
      } else {
        next.push_back(c);
      }
    }
    // Same-layer writes never match `look` (layer values are look+1 or 1 and
    // look is never 0), so applying them after the scan is equivalent.
    int val = (look == -1) ? 1 : look + 1;
    for (auto& a : assign) {
      flatdist[a.first] = val;
      dir[2 * a.first] = (int8_t)kD8Dx[a.second];
      dir[2 * a.first + 1] = (int8_t)kD8Dy[a.second];
    }
    flats.swap(next);
    ++look;
    if (look == 0) look = 1;
  }
}

// Flow tracing: raster order; stream cells (streams >= 0) -> LAKE; other
// cells follow dir until leaving the grid (OUTSIDE), reaching a stream
// (label (int)(-streams)) or an already-labelled cell (copy); a walk over
// 100000 steps gives up and leaves its cells at 0.  Then the connect pass
// copies label[label] for labels >= 0 when that is negative.
// src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:34-113 (trace),
// :115-134 (connect).
void orc_flow_trace(const int8_t* dir, const float* streams, int* label, int W,
                    int H) {
  const int64_t N = (int64_t)W * H;
  std::memset(label, 0, sizeof(int) * N);
  std::vector<int64_t> path;
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      int cx = x, cy = y;
      int64_t idx = (int64_t)y * W + x;
      if (streams[idx] >= 0.0f) { label[idx] = kLake; continue; }
      if (label[idx] < 0) continue;
      int iter = 0;
      path.clear();
      while (true) {
        if (iter > 100000) break;
        path.push_back(idx);
        cx += dir[2 * idx];
        cy += dir[2 * idx + 1];
        idx = (int64_t)cy * W + cx;
        if (cx < 0 || cx >= W || cy < 0 || cy >= H) {
          for (int64_t p : path) label[p] = kOutside;
          break;
        }
        if (streams[idx] >= 0.0f) {
          int l = (int)(-streams[idx]);
          for (int64_t p : path) label[p] = l;
          break;
        }
        if (label[idx] < 0) {
          int l = label[idx];
          for (int64_t p : path) label[p] = l;
          break;
        }
        iter++;
      }
    }
  }
  for (int64_t i = 0; i < N; i++) {
    if (label[i] >= 0) {
      int ni = label[i];
      if (label[ni] < 0) label[i] = label[ni];
    }
  }
}

// Path statistics of a direction grid, for checking the reference walk's
// step cap (src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:66-75: a walk
// that has not terminated after 100001 steps gives up, and its cells take
// cell 0's label in the connect pass).  A walk from cell c ends within its
// path's length, the number of moves from c until one leaves the grid or
// enters a stream cell.  out[0] = the longest such length over cells whose
// path terminates; out[1] = the cells whose path never terminates (it
// reaches a cell without a direction or a cycle).  Stream cells count as
// length 0.  Iterative, memoized: O(W*H).
void orc_trace_path_stats(const int8_t* dir, const float* streams, int W, int H,
                          int64_t* out) {
  const int64_t N = (int64_t)W * H;
  const int32_t kUnknown = -1, kOnStack = -2, kNever = -3;
  std::vector<int32_t> len(N, kUnknown);
  std::vector<int64_t> stack;
  int64_t longest = 0, never = 0;
  for (int64_t s = 0; s < N; s++) {
    if (len[s] != kUnknown) continue;
    stack.clear();
    int64_t c = s;
    int32_t tail;  // length at the end of the stacked chain, or kNever
    while (true) {
      if (streams[c] >= 0.0f) { len[c] = 0; tail = 0; break; }
      if (len[c] >= 0 || len[c] == kNever) { tail = len[c]; break; }
      if (len[c] == kOnStack) { tail = kNever; break; }
      len[c] = kOnStack;
      stack.push_back(c);
      const int cx = (int)(c % W) + dir[2 * c], cy = (int)(c / W) + dir[2 * c + 1];
      if (cx < 0 || cx >= W || cy < 0 || cy >= H) { tail = 0; break; }
      c = (int64_t)cy * W + cx;
    }
    // A chain that ran off the grid: its last stacked cell's move left the
    // grid (length 1); otherwise the chain's next cell has length `tail`.
    for (size_t k = stack.size(); k-- > 0;) {
      const int64_t v = stack[k];
      if (tail == kNever) {
        len[v] = kNever;
        never++;
      } else {
        len[v] = tail + 1;
        tail = len[v];
        if (tail > longest) longest = tail;
      }
    }
  }
  out[0] = longest;
  out[1] = never;
}

// Catchment border: border = 1 where the label is not LAKE and some N8
// neighbour has a larger, non-LAKE label; the Monte Carlo grid adds it
// (float).  The reference's border grid comes from an uninitialised
// allocation; zero-initialised here.
// src/catchmentborder/CatchmentBorderAlgorithmCPUOpenMP.h:30-82,
// src/catchmentborder/CatchmentBorderAlgorithm.h:53-74.
void orc_border_accumulate(const int* label, float* mc, int W, int H) {
  const int64_t N = (int64_t)W * H;
  std::vector<float> border(N, 0.0f);
#pragma omp parallel for
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      int64_t i = (int64_t)y * W + x;
      int c = label[i];
      if (c == kLake) continue;
      for (int n = 0; n < 8; n++) {
        int nx = x + kD8Dx[n], ny = y + kD8Dy[n];
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        int v = label[(int64_t)ny * W + nx];
        if (c < v && v != kLake) { border[i] = 1.0f; break; }
      }
    }
  }
#pragma omp parallel for
  for (int64_t i = 0; i < N; i++) {
    if (mc[i] != -1.0f) mc[i] = mc[i] + border[i];
  }
}

// ---- The reference's GPU path semantics ("exact" mode) -------------------

// Pit filling, GPU path: an exact float fill, no quantization.
// Initialisation, src/pitfilling/PitFillingAlgorithmGPUCUDA.cu:201-231:
// NODATA cells keep NODATA; border cells and cells equal to STREAM (0) keep
// their elevation and are the sources; every other cell starts at 99990000.
// Relaxation, :275-380: a source c lowers each interior neighbour n
// (1 <= x <= W-2, 1 <= y <= H-2) whose value is not NODATA, is above c's
// and is not its own elevation, to max(c, dem[n]), and n becomes a source.
// The limit does not depend on the order of the updates: every reached cell
// ends at the least, over 8-connected paths of non-NODATA cells from a
// source, of the largest elevation along the path; unreached cells keep
// 99990000.  It is computed here by a priority flood on that path maximum.
int orc_pitfill_exact(const float* dem, float* filled, int W, int H, float nodata) {
  const int64_t N = (int64_t)W * H;
  if (W < 1 || H < 1) return -1;
  typedef std::pair<float, int64_t> E;
  std::priority_queue<E, std::vector<E>, std::greater<E>> pq;
  std::vector<uint8_t> done(N, 0);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const int64_t i = (int64_t)y * W + x;
      const float v = dem[i];
      if (v == nodata) {
        filled[i] = v;
        done[i] = 1;
      } else if (v == 0.0f || x == 0 || y == 0 || x == W - 1 || y == H - 1) {
        filled[i] = v;
        pq.push(E(v, i));
      } else {
        filled[i] = 99990000.0f;
      }
    }
  while (!pq.empty()) {
    const E e = pq.top();
    pq.pop();
    const int64_t c = e.second;
    if (done[c] || e.first != filled[c]) continue;
    done[c] = 1;
    const int cx = (int)(c % W), cy = (int)(c / W);
    for (int n = 0; n < 8; n++) {
      const int nx = cx + kFillDx[n], ny = cy + kFillDy[n];
      if (nx <= 0 || nx >= W - 1 || ny <= 0 || ny >= H - 1) continue;
      const int64_t ni = (int64_t)ny * W + nx;
      if (done[ni]) continue;
      const float nv = std::max(filled[c], dem[ni]);
      if (nv < filled[ni]) {
        filled[ni] = nv;
        pq.push(E(nv, ni));
      }
    }
  }
  return 0;
}

// Flow routing, GPU path.  First pass,
// src/flowrouting/FlowRoutingAlgorithmGPUCUDAOriginal.cu:200-271: border
// cells point outward (flatDist -1, whatever their value), cells equal to 0
// are streams (-2), NODATA cells -3; others take the steepest strictly
// descending non-NODATA neighbour in N..NW order (diagonal drops divided by
// sqrt 2, first maximum wins).  Flats, :391-437 with the loop at :98-121:
// iteration k = 1, 2, ... gives each still-flat cell (flatDist 0) the first
// neighbour, in the order N, W, E, S, NW, NE, SW, SE, that either has a
// negative flatDist and a non-NODATA elevation <= the cell's, or was given
// a direction in an earlier iteration (1 <= flatDist <= k-1); flatDist = k.
// Values written in iteration k are not read in it, so applying them after
// the scan is the same.  The reference repeats until every flat cell has a
// direction; flats without an outlet would never finish there and are left
// at flatDist 0 with no direction here.
void orc_flow_route_gpu(const float* dem, int8_t* dir, int* flatdist, int W, int H,
                        float nodata) {
  const int64_t N = (int64_t)W * H;
  std::memset(dir, 0, 2 * N);
  std::memset(flatdist, 0, sizeof(int) * N);
  std::vector<uint32_t> flats;
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      int dxi = 0, dyi = 0;
      if (x == 0) dxi = -1; else if (x == W - 1) dxi = 1;
      if (y == 0) dyi = -1; else if (y == H - 1) dyi = 1;
      const int64_t i = (int64_t)y * W + x;
      if (dxi != 0 || dyi != 0) {
        dir[2 * i] = (int8_t)dxi; dir[2 * i + 1] = (int8_t)dyi;
        flatdist[i] = -1;
        continue;
      }
      if (dem[i] == 0.0f) { flatdist[i] = -2; continue; }
      if (dem[i] == nodata) { flatdist[i] = -3; continue; }
      float steepest = 0.0f;
      int sdx = 0, sdy = 0;
      for (int n = 0; n < 8; n++) {
        const int64_t ni = (int64_t)(y + kD8Dy[n]) * W + (x + kD8Dx[n]);
        if (dem[ni] == nodata) continue;
        float s = dem[i] - dem[ni];
        if (s > 0.0f) {
          if (n % 2 == 1) s = s / kSqrt2;
          if (s > steepest) { steepest = s; sdx = kD8Dx[n]; sdy = kD8Dy[n]; }
        }
      }
      if (steepest > 0.0f) {
        dir[2 * i] = (int8_t)sdx; dir[2 * i + 1] = (int8_t)sdy;
        flatdist[i] = -1;
      } else {
        flats.push_back((uint32_t)i);
      }
    }
  }
  static const int odx[8] = {0, -1, 1, 0, -1, 1, -1, 1};
  static const int ody[8] = {-1, 0, 0, 1, -1, -1, 1, 1};
  std::vector<uint32_t> next;
  std::vector<std::pair<uint32_t, int>> assign;
  for (int k = 1; !flats.empty(); k++) {
    next.clear();
    assign.clear();
    for (uint32_t c : flats) {
      const int cx = (int)(c % (uint32_t)W), cy = (int)(c / (uint32_t)W);
      const float e = dem[c];
      int got = -1;
      for (int n = 0; n < 8 && got < 0; n++) {
        const int nx = cx + odx[n], ny = cy + ody[n];
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        const int64_t ni = (int64_t)ny * W + nx;
        const int f = flatdist[ni];
        if ((f < 0 && dem[ni] != nodata && e >= dem[ni]) || (f >= 1 && f + 1 <= k)) got = n;
      }
      if (got >= 0) assign.push_back({c, got});
      else next.push_back(c);
    }
    if (assign.empty()) break;
    for (auto& a : assign) {
      flatdist[a.first] = k;
      dir[2 * a.first] = (int8_t)odx[a.second];
      dir[2 * a.first + 1] = (int8_t)ody[a.second];
    }
    flats.swap(next);
  }
}

// Flow tracing with dead ends reported: stream cells (streams >= 0) are
// LAKE; every other cell follows its direction to the grid edge (OUTSIDE) or
// a stream cell s (label (int)(-streams[s])); a cell without a direction, and
// every cell whose path reaches one, is ERROR.  The reference's GPU tracing
// marks the cell without a direction ERROR
// (src/flowtracing/FlowTracingAlgorithmGPUCUDA.cu:139-143) and leaves the
// cells upstream of it at a value that depends on its block layout; ERROR
// is used for them here.  A label-0 terminal takes cell 0's label, as in
// the CPU connect pass (src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:115-134).
void orc_flow_trace_gpu(const int8_t* dir, const float* streams, int* label, int W, int H) {
  const int64_t N = (int64_t)W * H;
  const int kUnset = 1;  // labels are <= 0
  std::vector<int> lab(N, kUnset);
  std::vector<int64_t> path;
  for (int64_t start = 0; start < N; start++) {
    if (lab[start] != kUnset) continue;
    path.clear();
    int64_t idx = start;
    int l = kUnset;
    while (true) {
      if (lab[idx] != kUnset) { l = lab[idx]; break; }
      if (streams[idx] >= 0.0f) { lab[idx] = kLake; l = kLake; break; }
      const int dx = dir[2 * idx], dy = dir[2 * idx + 1];
      if (dx == 0 && dy == 0) { path.push_back(idx); l = kError; break; }
      path.push_back(idx);
      const int cx = (int)(idx % W) + dx, cy = (int)(idx / W) + dy;
      if (cx < 0 || cx >= W || cy < 0 || cy >= H) { l = kOutside; break; }
      const int64_t ni = (int64_t)cy * W + cx;
      if (streams[ni] >= 0.0f) { l = (int)(-streams[ni]); break; }
      if ((int64_t)path.size() > N) { l = kError; break; }
      idx = ni;
    }
    for (int64_t p : path) lab[p] = l;
  }
  const int l0 = lab[0];
  for (int64_t i = 0; i < N; i++) label[i] = lab[i] >= 0 ? (l0 >= 0 ? 0 : l0) : lab[i];
}

// One realization of the GPU path semantics after the noise: convolution,
// realistic DEM and burning as in the CPU path (they agree when no NODATA
// is present), exact fill, GPU routing, tracing with dead ends reported,
// border accumulation.
int orc_realization_exact(const float* dem, const float* streams, float* field, int W, int H,
                          int model, const float* filt, int r, int bevel, float nodata_dem,
                          float nodata_stream, float* mc, float* filled_out, int8_t* dir_out,
                          int* label_out) {
  const int64_t N = (int64_t)W * H;
  std::vector<float> conv(N);
  int rc = model == 1 ? orc_convolve_separable(field, conv.data(), W, H, filt, r)
                      : orc_convolve_2d(field, conv.data(), W, H, filt, r);
  if (rc) return rc;
  orc_realistic_dem(dem, conv.data(), N, nodata_dem);
  rc = orc_stream_burn(conv.data(), streams, W, H, bevel, nodata_dem, nodata_stream);
  if (rc) return rc;
  std::vector<float> filled(N);
  rc = orc_pitfill_exact(conv.data(), filled.data(), W, H, nodata_dem);
  if (rc) return rc;
  std::vector<int8_t> dir(2 * N);
  std::vector<int> fd(N);
  orc_flow_route_gpu(filled.data(), dir.data(), fd.data(), W, H, nodata_dem);
  std::vector<int> label(N);
  orc_flow_trace_gpu(dir.data(), streams, label.data(), W, H);
  orc_border_accumulate(label.data(), mc, W, H);
  if (filled_out) std::memcpy(filled_out, filled.data(), sizeof(float) * N);
  if (dir_out) std::memcpy(dir_out, dir.data(), 2 * N);
  if (label_out) std::memcpy(label_out, label.data(), sizeof(int) * N);
  return 0;
}

// One realization after the noise: convolution (model 1 = Gaussian taps of
// length 2r+1, model 0 = exponential (2r+1)^2 filter), realistic DEM,
// burning, pit fill, routing, tracing, border accumulation.  `field` holds
// the injected noise on entry.  Mirrors the stage order of
// src/main.cpp:186-244.  Optional stage outputs are written when non-null.
int orc_realization(const float* dem, const float* streams, float* field,
                    int W, int H, int model, const float* filt, int r,
                    int bevel, float nodata_dem, float nodata_stream,
                    float* mc, float* filled_out, int8_t* dir_out,
                    int* label_out) {
  const int64_t N = (int64_t)W * H;
  std::vector<float> conv(N);
  int rc = model == 1 ? orc_convolve_separable(field, conv.data(), W, H, filt, r)
                      : orc_convolve_2d(field, conv.data(), W, H, filt, r);
  if (rc) return rc;
  orc_realistic_dem(dem, conv.data(), N, nodata_dem);
  rc = orc_stream_burn(conv.data(), streams, W, H, bevel, nodata_dem, nodata_stream);
  if (rc) return rc;
  std::vector<float> filled(N);
  rc = orc_pitfill(conv.data(), filled.data(), W, H, nodata_dem);
  if (rc) return rc;
  std::vector<int8_t> dir(2 * N);
  std::vector<int> fd(N);
  orc_flow_route(filled.data(), dir.data(), fd.data(), W, H);
  std::vector<int> label(N);
  orc_flow_trace(dir.data(), streams, label.data(), W, H);
  orc_border_accumulate(label.data(), mc, W, H);
  if (filled_out) std::memcpy(filled_out, filled.data(), sizeof(float) * N);
  if (dir_out) std::memcpy(dir_out, dir.data(), 2 * N);
  if (label_out) std::memcpy(label_out, label.data(), sizeof(int) * N);
  return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
