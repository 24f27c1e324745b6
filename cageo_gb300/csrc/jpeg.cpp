// jpeg.cpp -- the drainage count image as a JPEG file (`-o result.jpg`).
//
// The reference writes it with the jpge encoder, called on the one-channel
// byte image with the encoder's default parameters (src/main.cpp:258-271,
// src/jpge/jpge.cpp:951-972; defaults in src/jpge/jpge.h:21: quality 85,
// H2V2 subsampling, standard Huffman tables).  This writer produces the same
// bytes.  It is written from the JPEG standard (ITU-T T.81) and from what
// that encoder does with those parameters:
//
//  * Three components, Y Cb Cr, sampled 2x2, 1x1, 1x1 (src/jpge/jpge.cpp:
//    439-507): the luma plane is the byte image itself, both chroma planes
//    the constant 128 (the grey-to-YCbCr expansion, :97-100 and :804-847),
//    so every chroma block is all zero after the level shift.
//  * Minimum coded units of 16x16 pixels: a row is extended to a multiple of
//    16 by repeating its last pixel, the image to a multiple of 16 rows by
//    repeating its last row (:838-847, :785-803).  Within a unit the four
//    luma blocks go top-left, top-right, bottom-left, bottom-right, then Cb,
//    then Cr (:731-764).
//  * Quantization: the example tables of Annex K.1 (luma) and K.2 (chroma)
//    scaled for quality (5000/q below 50, 200-2q from 50; (t*s+50)/100
//    clamped to 1..255, :401-414); coefficients rounded half away from zero,
//    (|c| + t/2) / t (:571-594).
//  * Forward DCT: the Loeffler-Ligtenberg-Moschytz factorisation in 13-bit
//    fixed point, as published with the Independent JPEG Group's integer
//    DCT, with the encoder's scaling (:102-138): the row pass keeps two
//    fraction bits (its sums shifted left by 2, its rotations descaled by
//    2^11), the column pass removes them and the factor 8 (sums descaled by
//    2^5, rotations by 2^18).  The encoder truncates each operand of a
//    constant multiply to 16 bits; for 8-bit samples no operand exceeds
//    32640 in magnitude (a column of eight row sums of +-4096 at most), so
//    the truncation never changes a value, and no 32-bit sum overflows.
//    Both are kept here as the encoder's arithmetic defines them.
//  * Entropy coding: the Huffman tables of Annex K.3-K.6, DC differences per
//    component, zero runs of 16 as 0xF0, end of block when the block ends in
//    zeros, 0xFF bytes followed by 0x00, the last byte padded with 1-bits
//    (:604-616, :657-719, :776-783).
//  * Markers: SOI, JFIF APP0 (version 1.1, no units, density 1x1), one DQT
//    segment per table, SOF0, one DHT segment per table (luma DC, luma AC,
//    chroma DC, chroma AC), SOS, EOI (:244-365).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>
#include "cageo.h"
#include "guard.h"

namespace {

// Position in natural (row-major) order of the k-th coefficient in zigzag order.
const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// Annex K.1 (luminance) and K.2 (chrominance) quantization, natural order.
const uint8_t kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kChromaQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                              24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

// Annex K.3-K.6: number of codes of each length 1..16, then the symbols.
const uint8_t kLumaDcBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kChromaDcBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kLumaAcBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kLumaAcVals[162] = {
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
const uint8_t kChromaAcBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
const uint8_t kChromaAcVals[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61,
    0x71, 0x13, 0x22, 0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33,
    0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1, 0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18,
    0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36, 0x37, 0x38, 0x39, 0x3a, 0x43, 0x44,
    0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59, 0x5a, 0x63,
    0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97,
    0x98, 0x99, 0x9a, 0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4,
    0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca,
    0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7,
    0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

struct HuffTable {
  const uint8_t* bits;  // counts for lengths 1..16
  const uint8_t* vals;
  int nvals;
  uint16_t code[256];
  uint8_t len[256];
};

// Canonical codes (T.81 Annex C): consecutive codes within a length, the
// next length starting at twice the code after the last one.
HuffTable make_table(const uint8_t bits[16], const uint8_t* vals, int nvals) {
  HuffTable h{bits, vals, nvals, {}, {}};
  uint32_t code = 0;
  int k = 0;
  for (int l = 1; l <= 16; l++) {
    for (int i = 0; i < bits[l - 1]; i++, k++) {
      h.code[vals[k]] = (uint16_t)code++;
      h.len[vals[k]] = (uint8_t)l;
    }
    code <<= 1;
  }
  return h;
}

// The twelve rotation constants of the LLM factorisation, round(x * 2^13),
// with c(k) = cos(k*pi/16).
struct DctConsts {
  int32_t k0298, k0390, k0541, k0765, k0899, k1175, k1501, k1847, k1961, k2053, k2562, k3072;
};

DctConsts make_dct_consts() {
  auto c = [](int k) { return std::cos(k * 3.14159265358979323846 / 16.0); };
  auto fix = [](double x) { return (int32_t)(x * 8192.0 + 0.5); };
  const double r2 = std::sqrt(2.0);
  DctConsts d;
  d.k0298 = fix(r2 * (-c(1) + c(3) + c(5) - c(7)));
  d.k0390 = fix(r2 * (c(3) - c(5)));
  d.k0541 = fix(r2 * c(6));
  d.k0765 = fix(r2 * (c(2) - c(6)));
  d.k0899 = fix(r2 * (c(3) - c(7)));
  d.k1175 = fix(r2 * c(3));
  d.k1501 = fix(r2 * (c(1) + c(3) - c(5) - c(7)));
  d.k1847 = fix(r2 * (c(2) + c(6)));
  d.k1961 = fix(r2 * (c(3) + c(5)));
  d.k2053 = fix(r2 * (c(1) + c(3) - c(5) + c(7)));
  d.k2562 = fix(r2 * (c(1) + c(3)));
  d.k3072 = fix(r2 * (c(1) + c(3) + c(5) - c(7)));
  return d;
}

// 32-bit two's-complement results, as the encoder's int32 arithmetic gives
// them (computed in 64 bits, so no signed overflow occurs here).
inline int32_t wrap32(int64_t v) { return (int32_t)(uint32_t)(uint64_t)v; }
// An operand truncated to 16 bits, times a constant.
inline int64_t mul16(int64_t v, int32_t k) { return (int64_t)(int16_t)(uint16_t)(uint64_t)v * k; }
inline int32_t round_shift(int32_t v, int n) {
  return wrap32((int64_t)v + ((int64_t)1 << (n - 1))) >> n;
}

// One 8-point transform of p[0], p[s], ..., p[7s] in place.  The even sums
// (outputs 0 and 4) come out unscaled, the rotations scaled by 2^13; the
// caller's `sum_shl` / `sum_shr` and `rot_shr` rescale them.
inline void llm8(int32_t* p, int s, const DctConsts& k, int sum_shl, int sum_shr, int rot_shr) {
  const int64_t x0 = p[0], x1 = p[s], x2 = p[2 * s], x3 = p[3 * s];
  const int64_t x4 = p[4 * s], x5 = p[5 * s], x6 = p[6 * s], x7 = p[7 * s];
  const int64_t a0 = wrap32(x0 + x7), a7 = wrap32(x0 - x7), a1 = wrap32(x1 + x6),
                a6 = wrap32(x1 - x6), a2 = wrap32(x2 + x5), a5 = wrap32(x2 - x5),
                a3 = wrap32(x3 + x4), a4 = wrap32(x3 - x4);
  const int64_t e0 = wrap32(a0 + a3), e3 = wrap32(a0 - a3), e1 = wrap32(a1 + a2),
                e2 = wrap32(a1 - a2);
  // Even part.
  const int32_t s0 = wrap32(e0 + e1), s4 = wrap32(e0 - e1);
  const int64_t r = mul16(e2 + e3, k.k0541);
  const int32_t s2 = wrap32(r + mul16(e3, k.k0765)), s6 = wrap32(r - mul16(e2, k.k1847));
  // Odd part.
  const int64_t z1 = wrap32(a4 + a7), z2 = wrap32(a5 + a6), z3 = wrap32(a4 + a6),
                z4 = wrap32(a5 + a7);
  const int64_t z5 = mul16(z3 + z4, k.k1175);
  const int64_t m4 = mul16(a4, k.k0298), m5 = mul16(a5, k.k2053), m6 = mul16(a6, k.k3072),
                m7 = mul16(a7, k.k1501);
  const int64_t n1 = -mul16(z1, k.k0899), n2 = -mul16(z2, k.k2562);
  const int64_t n3 = wrap32(-mul16(z3, k.k1961) + z5), n4 = wrap32(-mul16(z4, k.k0390) + z5);
  const int32_t s1 = wrap32(m7 + n1 + n4), s3 = wrap32(m6 + n2 + n3), s5 = wrap32(m5 + n2 + n4),
                s7 = wrap32(m4 + n1 + n3);
  auto sum = [&](int32_t v) {
    return sum_shl ? (int32_t)((uint32_t)v << sum_shl) : round_shift(v, sum_shr);
  };
  p[0] = sum(s0);
  p[4 * s] = sum(s4);
  p[s] = round_shift(s1, rot_shr);
  p[2 * s] = round_shift(s2, rot_shr);
  p[3 * s] = round_shift(s3, rot_shr);
  p[5 * s] = round_shift(s5, rot_shr);
  p[6 * s] = round_shift(s6, rot_shr);
  p[7 * s] = round_shift(s7, rot_shr);
}

// Rows keep 2 fraction bits; columns remove them and the factor 8.
void forward_dct(int32_t* blk, const DctConsts& k) {
  for (int r = 0; r < 8; r++) llm8(blk + 8 * r, 1, k, 2, 0, 13 - 2);
  for (int c = 0; c < 8; c++) llm8(blk + c, 8, k, 0, 2 + 3, 13 + 2 + 3);
}

struct BitSink {
  std::vector<uint8_t>& out;
  uint64_t acc = 0;  // pending bits, right-aligned
  int n = 0;
  explicit BitSink(std::vector<uint8_t>& o) : out(o) {}
  void put(uint32_t bits, int len) {
    acc = (acc << len) | (bits & ((1u << len) - 1u));
    n += len;
    while (n >= 8) {
      const uint8_t b = (uint8_t)(acc >> (n - 8));
      out.push_back(b);
      if (b == 0xFF) out.push_back(0x00);
      n -= 8;
    }
  }
  void pad() {
    if (n) put(0x7Fu, 8 - n);  // the last byte's remaining bits are 1
  }
};

inline int magnitude_bits(int v) {
  unsigned a = (unsigned)(v < 0 ? -v : v);
  int n = 0;
  while (a) { n++; a >>= 1; }
  return n;
}

// Quantize (zigzag order) and entropy-code one transformed block.
void code_block(const int32_t* dct, const uint8_t* qz, const HuffTable& dc, const HuffTable& ac,
                int& prev_dc, BitSink& bs) {
  int coef[64];
  for (int i = 0; i < 64; i++) {
    const int32_t c = dct[kZigzag[i]], t = qz[i];
    const int32_t a = (c < 0 ? -c : c) + (t >> 1);
    const int32_t v = a < t ? 0 : a / t;
    coef[i] = (int)(int16_t)(c < 0 ? -v : v);
  }
  const int diff = coef[0] - prev_dc;
  prev_dc = coef[0];
  const int dn = magnitude_bits(diff);
  bs.put(dc.code[dn], dc.len[dn]);
  if (dn) bs.put((uint32_t)(diff < 0 ? diff - 1 : diff), dn);
  int run = 0;
  for (int i = 1; i < 64; i++) {
    const int v = coef[i];
    if (v == 0) {
      run++;
      continue;
    }
    for (; run >= 16; run -= 16) bs.put(ac.code[0xF0], ac.len[0xF0]);
    const int n = magnitude_bits(v);
    const int sym = (run << 4) | n;
    bs.put(ac.code[sym], ac.len[sym]);
    bs.put((uint32_t)(v < 0 ? v - 1 : v), n);
    run = 0;
  }
  if (run) bs.put(ac.code[0x00], ac.len[0x00]);
}

void put16(std::vector<uint8_t>& o, int v) {
  o.push_back((uint8_t)(v >> 8));
  o.push_back((uint8_t)v);
}

void put_dqt(std::vector<uint8_t>& o, int id, const uint8_t* qz) {
  o.insert(o.end(), {0xFF, 0xDB, 0x00, 0x43, (uint8_t)id});
  o.insert(o.end(), qz, qz + 64);
}

void put_dht(std::vector<uint8_t>& o, int cls_id, const HuffTable& h) {
  o.insert(o.end(), {0xFF, 0xC4});
  put16(o, 2 + 1 + 16 + h.nvals);
  o.push_back((uint8_t)cls_id);
  o.insert(o.end(), h.bits, h.bits + 16);
  o.insert(o.end(), h.vals, h.vals + h.nvals);
}

// Quality-scaled table in zigzag order (the order it is stored and used in).
void scaled_table(const uint8_t* natural, int quality, uint8_t* qz) {
  const int32_t s = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  for (int i = 0; i < 64; i++) {
    const int32_t v = ((int32_t)natural[kZigzag[i]] * s + 50) / 100;
    qz[i] = (uint8_t)(v < 1 ? 1 : (v > 255 ? 255 : v));
  }
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
  uint8_t qy[64], qc[64];
  scaled_table(kLumaQ, quality, qy);
  scaled_table(kChromaQ, quality, qc);
  const HuffTable ydc = make_table(kLumaDcBits, kDcVals, 12);
  const HuffTable yac = make_table(kLumaAcBits, kLumaAcVals, 162);
  const HuffTable cdc = make_table(kChromaDcBits, kDcVals, 12);
  const HuffTable cac = make_table(kChromaAcBits, kChromaAcVals, 162);
  const DctConsts k = make_dct_consts();

  std::vector<uint8_t> o;
  o.reserve((size_t)W * H / 4 + 1024);
  o.insert(o.end(), {0xFF, 0xD8});                                      // SOI
  o.insert(o.end(), {0xFF, 0xE0, 0x00, 0x10, 'J', 'F', 'I', 'F', 0x00,  // APP0: JFIF 1.1,
                     0x01, 0x01, 0x00, 0x00, 0x01, 0x00, 0x01, 0x00, 0x00});  // no units, 1x1
  put_dqt(o, 0, qy);
  put_dqt(o, 1, qc);
  o.insert(o.end(), {0xFF, 0xC0, 0x00, 0x11, 0x08});  // SOF0, 8-bit samples
  put16(o, H);
  put16(o, W);
  o.insert(o.end(), {0x03, 0x01, 0x22, 0x00, 0x02, 0x11, 0x01, 0x03, 0x11, 0x01});
  put_dht(o, 0x00, ydc);
  put_dht(o, 0x10, yac);
  put_dht(o, 0x01, cdc);
  put_dht(o, 0x11, cac);
  o.insert(o.end(), {0xFF, 0xDA, 0x00, 0x0C, 0x03, 0x01, 0x00, 0x02, 0x11, 0x03, 0x11, 0x00,
                     0x3F, 0x00});  // SOS: all three components, full spectrum

  // A band of 16 rows, each extended to a multiple of 16 by its last pixel;
  // rows past the image repeat its last row.
  const int W16 = (W + 15) & ~15;
  std::vector<uint8_t> band((size_t)16 * W16);
  BitSink bs(o);
  int prev_y = 0, prev_cb = 0, prev_cr = 0;
  int32_t blk[64];
  int32_t zero[64] = {0};  // a chroma block: 128 - 128 everywhere, and so its transform
  for (int y0 = 0; y0 < H; y0 += 16) {
    for (int r = 0; r < 16; r++) {
      const int y = y0 + r < H ? y0 + r : H - 1;
      uint8_t* row = &band[(size_t)r * W16];
      const uint8_t* src = h_gray + (size_t)y * W;
      for (int x = 0; x < W16; x++) row[x] = src[x < W ? x : W - 1];
    }
    for (int x0 = 0; x0 < W16; x0 += 16) {
      for (int b = 0; b < 4; b++) {
        const int bx = x0 + 8 * (b & 1), by = 8 * (b >> 1);
        for (int r = 0; r < 8; r++)
          for (int c = 0; c < 8; c++) blk[8 * r + c] = (int32_t)band[(size_t)(by + r) * W16 + bx + c] - 128;
        forward_dct(blk, k);
        code_block(blk, qy, ydc, yac, prev_y, bs);
      }
      code_block(zero, qc, cdc, cac, prev_cb, bs);
      code_block(zero, qc, cdc, cac, prev_cr, bs);
    }
  }
  bs.pad();
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
