// jpeg.cpp -- baseline (sequential DCT, Huffman) grayscale JPEG writer for
// the drainage count image (`-o result.jpg`, src/main.cpp:258-271, which
// uses the jpge library with its default quality 85).
//
// Written from the JPEG standard (ITU-T T.81): quantization and Huffman
// tables are the example tables of Annex K (K.1 luminance quantization,
// K.3 luminance DC/AC Huffman codes), scaled for quality the usual way
// (scale = 5000/q below 50, 200-2q above).  Blocks are 8x8, edge-replicated
// at the right and bottom borders; the forward DCT is the separable
// floating-point definition.  Output is a JFIF file.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>
#include "cageo.h"
#include "guard.h"

namespace {

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// Annex K.1, luminance (natural order).
const uint8_t kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};

// Annex K.3: code-length counts (1..16) and symbol values.
const uint8_t kDcBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kAcBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kAcVals[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61,
    0x07, 0x22, 0x71, 0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52,
    0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72, 0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25,
    0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45,
    0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59, 0x5a, 0x63, 0x64,
    0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99,
    0x9a, 0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6,
    0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3,
    0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8,
    0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

struct Huff {
  uint16_t code[256];
  uint8_t len[256];
};

// Canonical codes from (counts, symbols) (T.81 Annex C).
Huff make_huff(const uint8_t bits[16], const uint8_t* vals) {
  Huff h{};
  uint16_t code = 0;
  int k = 0;
  for (int l = 1; l <= 16; l++) {
    for (int i = 0; i < bits[l - 1]; i++, k++) {
      h.code[vals[k]] = code++;
      h.len[vals[k]] = (uint8_t)l;
    }
    code <<= 1;
  }
  return h;
}

struct BitWriter {
  std::vector<uint8_t>& out;
  uint32_t acc = 0;
  int n = 0;
  explicit BitWriter(std::vector<uint8_t>& o) : out(o) {}
  void put(uint32_t bits, int len) {
    for (int i = len - 1; i >= 0; i--) {
      acc = (acc << 1) | ((bits >> i) & 1u);
      if (++n == 8) {
        out.push_back((uint8_t)acc);
        if ((uint8_t)acc == 0xFF) out.push_back(0x00);  // byte stuffing
        acc = 0;
        n = 0;
      }
    }
  }
  void flush() {
    while (n) put(1, 1);  // pad with 1-bits
  }
};

int magnitude_bits(int v) {
  int a = v < 0 ? -v : v, n = 0;
  while (a) { n++; a >>= 1; }
  return n;
}

void put16(std::vector<uint8_t>& o, int v) {
  o.push_back((uint8_t)(v >> 8));
  o.push_back((uint8_t)v);
}

}  // namespace

static cageo_status write_jpeg(const char* path, const uint8_t* h_gray, int W, int H,
                               int quality) {
  if (!path || !h_gray || W <= 0 || H <= 0 || W > 65535 || H > 65535) {
    cageo::set_error("invalid argument: JPEG path, image or size (1..65535 per side)");
    return CAGEO_ERR_ARGUMENT;
  }
  if (quality < 1 || quality > 100) {
    cageo::set_error("invalid argument: JPEG quality must be 1..100");
    return CAGEO_ERR_ARGUMENT;
  }
  const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  uint8_t q[64];
  for (int i = 0; i < 64; i++) {
    int v = (kLumaQ[i] * scale + 50) / 100;
    q[i] = (uint8_t)(v < 1 ? 1 : (v > 255 ? 255 : v));
  }
  const Huff dc = make_huff(kDcBits, kDcVals), ac = make_huff(kAcBits, kAcVals);
  double cosv[8][8];
  for (int x = 0; x < 8; x++)
    for (int u = 0; u < 8; u++) cosv[x][u] = std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16);

  std::vector<uint8_t> o;
  o.reserve((size_t)W * H / 4 + 1024);
  o.insert(o.end(), {0xFF, 0xD8});                                    // SOI
  o.insert(o.end(), {0xFF, 0xE0, 0x00, 0x10, 'J', 'F', 'I', 'F', 0x00, 0x01, 0x01, 0x00,
                     0x00, 0x01, 0x00, 0x01, 0x00, 0x00});            // APP0 JFIF 1.1
  o.insert(o.end(), {0xFF, 0xDB, 0x00, 0x43, 0x00});                  // DQT, table 0
  for (int i = 0; i < 64; i++) o.push_back(q[kZigzag[i]]);
  o.insert(o.end(), {0xFF, 0xC0, 0x00, 0x0B, 0x08});                  // SOF0
  put16(o, H);
  put16(o, W);
  o.insert(o.end(), {0x01, 0x01, 0x11, 0x00});
  o.insert(o.end(), {0xFF, 0xC4});                                    // DHT
  put16(o, 2 + 1 + 16 + 12 + 1 + 16 + 162);
  o.push_back(0x00);
  o.insert(o.end(), kDcBits, kDcBits + 16);
  o.insert(o.end(), kDcVals, kDcVals + 12);
  o.push_back(0x10);
  o.insert(o.end(), kAcBits, kAcBits + 16);
  o.insert(o.end(), kAcVals, kAcVals + 162);
  o.insert(o.end(), {0xFF, 0xDA, 0x00, 0x08, 0x01, 0x01, 0x00, 0x00, 0x3F, 0x00});  // SOS

  BitWriter bw(o);
  int prev_dc = 0;
  for (int by = 0; by < H; by += 8) {
    for (int bx = 0; bx < W; bx += 8) {
      double blk[8][8], tmp[8][8];
      for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
          int sy = by + y < H ? by + y : H - 1, sx = bx + x < W ? bx + x : W - 1;
          blk[y][x] = (double)h_gray[(size_t)sy * W + sx] - 128.0;
        }
      for (int y = 0; y < 8; y++)  // rows
        for (int u = 0; u < 8; u++) {
          double s = 0;
          for (int x = 0; x < 8; x++) s += blk[y][x] * cosv[x][u];
          tmp[y][u] = s * (u == 0 ? std::sqrt(0.125) : 0.5);
        }
      int coef[64];
      for (int v = 0; v < 8; v++)  // columns
        for (int u = 0; u < 8; u++) {
          double s = 0;
          for (int y = 0; y < 8; y++) s += tmp[y][u] * cosv[y][v];
          s *= (v == 0 ? std::sqrt(0.125) : 0.5);
          const double qv = s / q[v * 8 + u];
          coef[v * 8 + u] = (int)std::lround(qv);
        }
      // DC
      const int diff = coef[0] - prev_dc;
      prev_dc = coef[0];
      const int dn = magnitude_bits(diff);
      bw.put(dc.code[dn], dc.len[dn]);
      if (dn) bw.put((uint32_t)(diff < 0 ? diff - 1 : diff) & ((1u << dn) - 1u), dn);
      // AC
      int run = 0;
      for (int k = 1; k < 64; k++) {
        const int v = coef[kZigzag[k]];
        if (v == 0) { run++; continue; }
        while (run > 15) { bw.put(ac.code[0xF0], ac.len[0xF0]); run -= 16; }
        const int n = magnitude_bits(v);
        const int sym = (run << 4) | n;
        bw.put(ac.code[sym], ac.len[sym]);
        bw.put((uint32_t)(v < 0 ? v - 1 : v) & ((1u << n) - 1u), n);
        run = 0;
      }
      if (run) bw.put(ac.code[0x00], ac.len[0x00]);  // EOB
    }
  }
  bw.flush();
  o.insert(o.end(), {0xFF, 0xD9});  // EOI
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    cageo::set_error("unable to open \"%s\" for writing", path);
    return CAGEO_ERR_IO;
  }
  const size_t put = std::fwrite(o.data(), 1, o.size(), f);
  const bool closed = std::fclose(f) == 0;
  if (put != o.size() || !closed) {
    cageo::set_error("short write to \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  return CAGEO_OK;
}

extern "C" cageo_status cageo_write_jpeg(const char* path, const uint8_t* h_gray, int W, int H,
                                         int quality) {
  return cageo::guarded("cageo_write_jpeg",
                        [&] { return write_jpeg(path, h_gray, W, H, quality); });
}
