"""CPU restatement of the learned warm start's network (test infrastructure).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the ``cageo_gb300``
package.  It restates, in float64 numpy, the features, the forward pass and
the backward pass that ``cageo_gb300/csrc/learned.cu`` implements, so the
GPU gradients can be checked against an independent computation.  The
network has no counterpart in the drainage reference.

Layout: parameters W1[32][4][9], b1[32], W2[32][32][9], b2[32], W3[1][32][9],
b3[1]; tap t = (dy+1)*3 + (dx+1) reads the input at (y+dy, x+dx); zero
padding outside the grid; weights and biases are rounded to bf16 before use.
"""
import numpy as np

N_PARAMS = 10721
_SHAPES = [("W1", (32, 4, 9)), ("b1", (32,)), ("W2", (32, 32, 9)), ("b2", (32,)),
           ("W3", (1, 32, 9)), ("b3", (1,))]


def bf16_round(x):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    a = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (a >> 16) & 1
    r = ((a + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(params, rounded=True):
    """Split the parameter vector; rounded=False keeps float64 values (for
    finite-difference checks of this restatement itself)."""
    out, k = {}, 0
    for name, shp in _SHAPES:
        n = int(np.prod(shp))
        w = params[k:k + n]
        w = bf16_round(w).astype(np.float64) if rounded else np.asarray(w, np.float64)
        out[name] = w.reshape(shp)
        k += n
    return out


def features(v, nodata=-9999.0):
    """[H][W] float32 -> [4][H][W] float32 with the kernel's float32 order."""
    v = np.asarray(v, np.float32)
    H, W = v.shape
    f = np.zeros((4, H, W), np.float32)
    for y in range(H):
        for x in range(W):
            c = v[y, x]
            if c == np.float32(nodata):
                continue
            mn3 = mn7 = mx7 = c
            s = np.float32(0.0)
            cnt = 0
            for dy in range(-3, 4):
                for dx in range(-3, 4):
                    yy, xx = y + dy, x + dx
                    if not (0 <= yy < H and 0 <= xx < W):
                        continue
                    e = v[yy, xx]
                    if e == np.float32(nodata):
                        continue
                    mn7, mx7 = min(mn7, e), max(mx7, e)
                    s = np.float32(s + e)
                    cnt += 1
                    if abs(dy) <= 1 and abs(dx) <= 1:
                        mn3 = min(mn3, e)
            f[:, y, x] = [c - mn3, c - mn7, mx7 - c, c - np.float32(s / np.float32(cnt))]
    return f


def _shift(a, dy, dx):
    """out[..., y, x] = a[..., y+dy, x+dx], zero outside."""
    out = np.zeros_like(a)
    H, W = a.shape[-2:]
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    out[..., ys:ye, xs:xe] = a[..., ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def _conv(a, w, b):
    """a [B][Cin][H][W], w [Cout][Cin][9] -> [B][Cout][H][W]."""
    out = np.zeros((a.shape[0], w.shape[0]) + a.shape[2:])
    for t in range(9):
        s = _shift(a, t // 3 - 1, t % 3 - 1)
        out += np.einsum("oc,bchw->bohw", w[:, :, t], s)
    return out + (b[None, :, None, None] if b is not None else 0.0)


def forward(params, feat, rounded=True):
    """feat [B][4][H][W] -> (a1, a2, y [B][H][W]) in float64."""
    p = unpack(params, rounded)
    x = np.asarray(feat, np.float64)
    a1 = np.maximum(_conv(x, p["W1"], p["b1"]), 0.0)
    a2 = np.maximum(_conv(a1, p["W2"], p["b2"]), 0.0)
    y = _conv(a2, p["W3"], p["b3"])[:, 0]
    return a1, a2, y


def _wgrad(dz, a):
    """dW[o][c][t] = sum dz[b][o](y,x) a[b][c](y+dy,x+dx)."""
    g = np.zeros((dz.shape[1], a.shape[1], 9))
    for t in range(9):
        s = _shift(a, t // 3 - 1, t % 3 - 1)
        g[:, :, t] = np.einsum("bohw,bchw->oc", dz, s)
    return g


def _dinput(dz, w):
    """Gradient of a correlation with respect to its input."""
    out = np.zeros((dz.shape[0], w.shape[1]) + dz.shape[2:])
    for t in range(9):
        out += _shift(np.einsum("oc,bohw->bchw", w[:, :, t], dz), 1 - t // 3, 1 - t % 3)
    return out


def backward(params, feat, dy, rounded=True):
    """Gradient of sum(dy * y) with respect to the parameter vector (float64)."""
    p = unpack(params, rounded)
    x = np.asarray(feat, np.float64)
    a1, a2, _ = forward(params, feat, rounded)
    dz3 = np.asarray(dy, np.float64)[:, None]
    gW3, gb3 = _wgrad(dz3, a2), dz3.sum(axis=(0, 2, 3))
    dz2 = _dinput(dz3, p["W3"]) * (a2 > 0)
    gW2, gb2 = _wgrad(dz2, a1), dz2.sum(axis=(0, 2, 3))
    dz1 = _dinput(dz2, p["W2"]) * (a1 > 0)
    gW1, gb1 = _wgrad(dz1, x), dz1.sum(axis=(0, 2, 3))
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
