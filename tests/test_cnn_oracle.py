"""The CPU restatement of the warm-start network checks itself: its
analytic gradients against central finite differences (float64), and its
bf16 rounding against the definition (nearest, ties to even)."""
import numpy as np

import cnn_oracle as co


def test_bf16_round():
    x = np.array([1.0, 1.00390625, 1.01171875, -3.3, 65504.0, 1e-3], np.float32)
    r = co.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.015625)  # ties to even
    bits = r.view(np.uint32)
    assert np.all(bits & 0xFFFF == 0)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.standard_normal(co.N_PARAMS) * 0.3
    feat = rng.standard_normal((2, 4, 7, 6))
    dy = rng.standard_normal((2, 7, 6))
    g = co.backward(p, feat, dy, rounded=False)
    idx = rng.choice(co.N_PARAMS, 40, replace=False)
    idx = np.concatenate([idx, [1152, 10400, 10720, 10432]])  # biases and a W3 tap
    for k in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp = (dy * co.forward(pp, feat, rounded=False)[2]).sum()
        lm = (dy * co.forward(pm, feat, rounded=False)[2]).sum()
        num = (lp - lm) / (2 * h)
        assert abs(num - g[k]) <= 1e-5 * max(1.0, abs(num)), (k, num, g[k])


def test_features_small():
    v = np.array([[5, 4, 3], [4, 1, 2], [3, 2, 9]], np.float32)
    f = co.features(v)
    assert f[0, 1, 1] == 0.0           # the centre is the 3x3 minimum
    assert f[2, 1, 1] == 8.0           # 7x7 maximum 9 minus 1
    assert np.isclose(f[3, 1, 1], 1 - v.mean(), atol=1e-6)
