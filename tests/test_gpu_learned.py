"""The learned warm start's kernels against the CPU restatement of the
network (oracle/cnn_oracle.py): features, forward pass, gradients of every
parameter, the fused bf16 tensor-core inference, loss and optimizer."""
import numpy as np
import pytest

import cnn_oracle as co
from cases import make_case

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _params(seed, scale=1.0):
    from cageo_gb300 import learned
    p = learned.init_params(seed) * scale
    p[1152:1184] = 0.05  # small positive biases keep some ReLUs active
    p[10400:10432] = 0.05
    return p


def test_features_match_oracle(cuda):
    from cageo_gb300 import api
    dem, _ = make_case(23, 17, seed=2, nodata_cells=12)
    got = api.ws_features(_t(dem))[0].cpu().numpy()
    ref = co.features(dem)
    assert np.array_equal(got, ref)


def test_forward_and_gradients_match_oracle(cuda):
    from cageo_gb300 import api
    import torch
    rng = np.random.default_rng(5)
    p = _params(1)
    feat = (rng.standard_normal((2, 4, 13, 11)) * 0.7).astype(np.float32)
    a1, a2, out = api.ws_forward(_t(p), _t(feat))
    _, _, ref = co.forward(p, feat)
    assert np.allclose(out.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
    dy = rng.standard_normal((2, 13, 11)).astype(np.float32)
    grad = torch.zeros(co.N_PARAMS, device="cuda")
    api.ws_backward(_t(p), _t(feat), a1, a2, _t(dy), grad)
    g = grad.cpu().numpy()
    gr = co.backward(p, feat, dy)
    for lo, hi in [(0, 1152), (1152, 1184), (1184, 10400), (10400, 10432), (10432, 10720),
                   (10720, 10721)]:
        assert np.allclose(g[lo:hi], gr[lo:hi], rtol=2e-3, atol=2e-3 * np.abs(gr[lo:hi]).max()), lo


def test_fused_inference_matches_training_forward(cuda):
    """The fused kernel keeps hidden activations in bf16 (the training pass
    in fp32): outputs agree to bf16 precision; the warm start follows the
    threshold exactly."""
    from cageo_gb300 import api
    import torch
    dem, streams = make_case(150, 101, seed=7)
    v = _t(dem)
    p = _t(_params(3, 0.5))
    _, _, out = api.ws_forward(p, api.ws_features(v))
    warm, depth = api.ws_infer(p, v, threshold=0.0, want_warm=True, want_depth=True)
    ref = out[0]
    scale = float(ref.abs().max()) + 1e-3
    assert float((depth - ref).abs().max()) <= 0.03 * scale
    inf = torch.full_like(v, float("inf"))
    assert torch.equal(warm, torch.where(depth < 0.0, v, inf))


def test_mse_and_adam(cuda):
    from cageo_gb300 import api
    import torch
    rng = np.random.default_rng(9)
    y = rng.standard_normal((2, 12, 10)).astype(np.float32)
    t = rng.standard_normal((2, 12, 10)).astype(np.float32)
    dy = torch.empty((2, 12, 10), device="cuda")
    loss = torch.zeros(1, device="cuda")
    api.ws_mse(_t(y), _t(t), dy, loss, margin=3)
    m = np.zeros((12, 10), bool)
    m[3:9, 3:7] = True
    cnt = 2 * m.sum()
    d = (y - t) * m
    assert np.allclose(dy.cpu().numpy(), 2 * d / cnt, rtol=1e-6, atol=1e-9)
    assert np.isclose(float(loss), (d ** 2).sum() / cnt, rtol=1e-5)
    p = _t(np.ones(5))
    g = _t(np.array([1, -1, 2, 0, 0.5]))
    m1, m2 = torch.zeros(5, device="cuda"), torch.zeros(5, device="cuda")
    api.ws_adam(p, g, m1, m2, 0.1, 1)
    # First bias-corrected Adam step moves each parameter by lr * sign(g).
    ref = 1 - 0.1 * np.sign([1, -1, 2, 0, 0.5])
    assert np.allclose(p.cpu().numpy(), ref, atol=1e-6)
