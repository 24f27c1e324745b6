// synth.cpp -- host helper for the synthetic inputs used by the tests and the
// benchmark: a stream raster derived from a DEM by priority-flood routing and
// D8 flow accumulation.
//
// Not part of the drainage pipeline itself.  The reference ships no sample
// data (its DEM/*.bin are missing), so seeded synthetic DEMs stand in for it.
//
// Method: priority-flood (Barnes, Lehman & Mulla 2014) from the grid border;
// each cell drains to the cell that first reached it, which gives every cell
// (pits and flats included) a receiver; flow accumulation then runs in
// reverse pop order.  Cells whose accumulation exceeds `threshold` become
// stream cells, numbered per 8-connected stream component (1, 2, ...) or all
// 1.0; the rest get `nodata`.
//
// Returns 0, 1 for a grid below 3 x 3 or of 2^32 cells or more (cell
// indices are uint32), 2 when host memory runs out (no C++ exception
// leaves the library).
#include <cstdint>
#include <cstring>
#include <new>
#include <queue>
#include <vector>

static int synth_streams(const float* dem, int W, int H, int threshold, int per_component_ids,
                         float nodata, float* streams_out, int* accum_out) {
  if (W < 3 || H < 3 || (int64_t)W * H >= ((int64_t)1 << 32)) return 1;
  const int64_t N = (int64_t)W * H;
  // The flood pops cells in ascending (level, push order).  A level never
  // falls, so every cell pushed at the level being processed goes after the
  // ones already queued at that level: those wait in a FIFO, and only cells
  // above the level enter the heap.  The heap key packs the level's order-
  // preserving bits above the push counter, so one 64-bit compare orders it.
  struct Item {
    uint64_t key;  // ordered float bits << 32 | push order (N < 2^32)
    uint32_t i;
  };
  struct Cmp {
    bool operator()(const Item& a, const Item& b) const { return a.key > b.key; }
  };
  auto ordered = [](float z) {
    uint32_t u;
    std::memcpy(&u, &z, 4);
    if (u == 0x80000000u) u = 0;  // -0 and +0 are one level
    return (uint64_t)((u & 0x80000000u) ? ~u : (u | 0x80000000u));
  };
  std::priority_queue<Item, std::vector<Item>, Cmp> pq;
  std::vector<uint32_t> level_fifo;
  size_t fifo_head = 0;
  std::vector<uint8_t> seen(N, 0);
  std::vector<float> zc(N);  // level at which each cell was pushed
  std::vector<uint32_t> recv(N, 0xffffffffu), pop_order;
  pop_order.reserve(N);
  uint64_t order = 0;
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++)
      if (x == 0 || y == 0 || x == W - 1 || y == H - 1) {
        uint32_t i = (uint32_t)((int64_t)y * W + x);
        zc[i] = dem[i];
        pq.push({ordered(dem[i]) << 32 | order++, i});
        seen[i] = 1;
      }
  static const int dx[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  static const int dy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
  uint64_t level = 0;  // ordered bits of the level being processed
  while (!pq.empty() || fifo_head < level_fifo.size()) {
    uint32_t ci;
    if (!pq.empty() && (fifo_head == level_fifo.size() || (pq.top().key >> 32) == level)) {
      ci = pq.top().i;
      level = pq.top().key >> 32;
      pq.pop();
    } else {
      ci = level_fifo[fifo_head++];
      if (fifo_head == level_fifo.size()) {
        level_fifo.clear();
        fifo_head = 0;
      }
    }
    const float cz = zc[ci];
    pop_order.push_back(ci);
    int cx = (int)(ci % (uint32_t)W), cy = (int)(ci / (uint32_t)W);
    for (int n = 0; n < 8; n++) {
      int nx = cx + dx[n], ny = cy + dy[n];
      if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
      uint32_t ni = (uint32_t)((int64_t)ny * W + nx);
      if (seen[ni]) continue;
      seen[ni] = 1;
      recv[ni] = ci;
      float z = dem[ni] < cz ? cz : dem[ni];
      zc[ni] = z;
      if (ordered(z) == level) {
        level_fifo.push_back(ni);
        order++;
      } else {
        pq.push({ordered(z) << 32 | order++, ni});
      }
    }
  }
  std::vector<int> acc(N, 1);
  for (int64_t k = N - 1; k >= 0; k--) {
    uint32_t i = pop_order[k];
    if (recv[i] != 0xffffffffu) acc[recv[i]] += acc[i];
  }
  for (int64_t i = 0; i < N; i++) streams_out[i] = acc[i] > threshold ? 1.0f : nodata;
  if (per_component_ids) {
    std::vector<int> comp(N, 0);
    int next = 0;
    std::vector<uint32_t> stack;
    for (int64_t s = 0; s < N; s++) {
      if (streams_out[s] == nodata || comp[s]) continue;
      comp[s] = ++next;
      stack.assign(1, (uint32_t)s);
      while (!stack.empty()) {
        uint32_t c = stack.back();
        stack.pop_back();
        int cx = (int)(c % (uint32_t)W), cy = (int)(c / (uint32_t)W);
        for (int n = 0; n < 8; n++) {
          int nx = cx + dx[n], ny = cy + dy[n];
          if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
          uint32_t ni = (uint32_t)((int64_t)ny * W + nx);
          if (streams_out[ni] == nodata || comp[ni]) continue;
          comp[ni] = next;
          stack.push_back(ni);
        }
      }
    }
    for (int64_t i = 0; i < N; i++)
      if (comp[i]) streams_out[i] = (float)comp[i];
  }
  if (accum_out)
    for (int64_t i = 0; i < N; i++) accum_out[i] = acc[i];
  return 0;
}

extern "C" int cageo_synth_streams(const float* dem, int W, int H, int threshold,
                                   int per_component_ids, float nodata, float* streams_out,
                                   int* accum_out) {
  try {
    return synth_streams(dem, W, H, threshold, per_component_ids, nodata, streams_out,
                         accum_out);
  } catch (const std::bad_alloc&) {
    return 2;
  }
}
