"""Minimal baseline (sequential, Huffman) JPEG decoder used to check the
library's JPEG writer: interleaved components with their sampling factors,
one quantization and Huffman table pair per component; returns the first
(luma) component.  Test infrastructure only."""
import numpy as np

ZIGZAG = [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34,
          27, 20, 13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37,
          44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63]


def _huff(bits, vals):
    table, code, k = {}, 0, 0
    for length in range(1, 17):
        for _ in range(bits[length - 1]):
            table[(length, code)] = vals[k]
            code += 1
            k += 1
        code <<= 1
    return table


class _Bits:
    def __init__(self, data):
        out, i = bytearray(), 0
        while i < len(data):
            b = data[i]
            if b == 0xFF:
                nxt = data[i + 1]
                if nxt == 0x00:
                    out.append(0xFF)
                    i += 2
                    continue
                break  # a marker ends the scan
            out.append(b)
            i += 1
        self.data, self.pos = bytes(out), 0

    def bit(self):
        b = (self.data[self.pos >> 3] >> (7 - (self.pos & 7))) & 1
        self.pos += 1
        return b

    def bits(self, n):
        v = 0
        for _ in range(n):
            v = (v << 1) | self.bit()
        return v

    def symbol(self, table):
        code = 0
        for length in range(1, 17):
            code = (code << 1) | self.bit()
            if (length, code) in table:
                return table[(length, code)]
        raise ValueError("bad Huffman code")


def _extend(v, n):
    return v - (1 << n) + 1 if n and v < (1 << (n - 1)) else v


def parse(path):
    """Markers of a baseline file: (quant tables, Huffman tables, frame
    components [(id, h, v, tq)], scan components [(id, td, ta)], W, H, scan
    bytes)."""
    with open(path, "rb") as f:
        data = f.read()
    assert data[:2] == b"\xff\xd8", "SOI"
    i, quant, tables, comps, W, H = 2, {}, {}, [], None, None
    while True:
        assert data[i] == 0xFF
        marker = data[i + 1]
        if marker == 0xD9:
            break
        seglen = int.from_bytes(data[i + 2:i + 4], "big")
        seg = data[i + 4:i + 2 + seglen]
        if marker == 0xDB:
            j = 0
            while j < len(seg):
                assert seg[j] >> 4 == 0, "8-bit tables"
                q = np.zeros(64)
                for k in range(64):
                    q[ZIGZAG[k]] = seg[j + 1 + k]
                quant[seg[j] & 15] = q
                j += 65
        elif marker == 0xC0:
            H, W = int.from_bytes(seg[1:3], "big"), int.from_bytes(seg[3:5], "big")
            comps = [(seg[6 + 3 * c], seg[7 + 3 * c] >> 4, seg[7 + 3 * c] & 15, seg[8 + 3 * c])
                     for c in range(seg[5])]
        elif marker == 0xC4:
            j = 0
            while j < len(seg):
                tc_th = seg[j]
                bits = list(seg[j + 1:j + 17])
                n = sum(bits)
                tables[tc_th] = _huff(bits, list(seg[j + 17:j + 17 + n]))
                j += 17 + n
        elif marker == 0xDA:
            scan = [(seg[1 + 2 * c], seg[2 + 2 * c] >> 4, seg[2 + 2 * c] & 15)
                    for c in range(seg[0])]
            return quant, tables, comps, scan, W, H, data[i + 2 + seglen:]
        i += 2 + seglen
    raise ValueError("no scan")


def decode(path):
    quant, tables, comps, scan, W, H, data = parse(path)
    assert [c[0] for c in comps] == [s[0] for s in scan], "one interleaved scan"
    hmax, vmax = max(c[1] for c in comps), max(c[2] for c in comps)
    mw, mh = 8 * hmax, 8 * vmax
    nx, ny = (W + mw - 1) // mw, (H + mh - 1) // mh
    c = np.array([[np.cos((2 * x + 1) * u * np.pi / 16) for u in range(8)] for x in range(8)])
    a = np.array([np.sqrt(0.125)] + [0.5] * 7)
    basis = c * a[None, :]  # basis[x, u]
    _, h0, v0, _ = comps[0]
    luma = np.zeros((ny * 8 * v0, nx * 8 * h0))
    bs = _Bits(data)
    prev = [0] * len(comps)
    for my in range(ny):
        for mx in range(nx):
            for ci, ((_, h, v, tq), (_, td, ta)) in enumerate(zip(comps, scan)):
                for by in range(v):
                    for bx in range(h):
                        coef = np.zeros(64)
                        s = bs.symbol(tables[td])
                        prev[ci] += _extend(bs.bits(s), s)
                        coef[0] = prev[ci]
                        k = 1
                        while k < 64:
                            rs = bs.symbol(tables[0x10 | ta])
                            r, s = rs >> 4, rs & 15
                            if s == 0:
                                if r == 15:
                                    k += 16
                                    continue
                                break
                            k += r
                            coef[ZIGZAG[k]] = _extend(bs.bits(s), s)
                            k += 1
                        if ci:
                            continue  # chroma is decoded only to advance the stream
                        blk = (coef * quant[tq]).reshape(8, 8)  # [v][u]
                        pix = (basis @ blk.T @ basis.T).T + 128
                        y0, x0 = (my * v + by) * 8, (mx * h + bx) * 8
                        luma[y0:y0 + 8, x0:x0 + 8] = pix
    return np.clip(np.rint(luma[:H, :W]), 0, 255).astype(np.uint8)
