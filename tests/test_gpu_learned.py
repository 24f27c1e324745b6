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


@pytest.mark.parametrize("which", ["trained", "untrained"])
def test_learned_pipeline_equals_plain_exact(cuda, which):
    """Warm-started realizations are verified and repaired: counts, filled
    surface, directions and labels equal the plain exact pipeline's, also
    for an untrained network whose warm starts are mostly wrong."""
    from cageo_gb300 import api, learned
    dem, streams = make_case(300, 257, seed=12)
    kw = dict(error_stddev=1.5, seed=5, fill_mode=api.FILL_EXACT)
    plain = api.Pipeline(dem, streams, **kw)
    plain.run(0, 4)
    lp = api.Pipeline(dem, streams, **kw)
    if which == "trained":
        lp.set_warmstart(learned.load_params(), 0.005)
    else:
        lp.set_warmstart(learned.init_params(7), 0.5)
    lp.run(0, 4)
    assert np.array_equal(lp.counts(), plain.counts())
    for a, b in zip(lp.last_stages(), plain.last_stages()):
        assert np.array_equal(a, b)
    st = lp.warmstart_stats()
    assert st["realizations"] == 4
    if which == "untrained":
        assert st["repaired"] >= 1 and st["reset_cells"] > 0
    lp.set_warmstart(None, 0.0)
    lp.run(4, 1)
    plain.run(4, 1)
    assert np.array_equal(lp.counts(), plain.counts())


def test_trained_network_saves_fill_sweeps(cuda):
    """What the trained network gains: its warm start (before verification)
    needs fewer sweep rounds than the cold fill, and far fewer of the cells it
    starts at their own elevation are wrong (wet cells marked dry, each of
    which forces a repair) than with the untrained network."""
    from cageo_gb300 import api, learned
    import torch
    src = learned.PairSource(size=512, tiles=2, seed=4242)
    trained, untrained = learned.load_params(), learned.init_params(3)
    rounds = {}
    for name, prm in (("trained", trained), ("untrained", untrained)):
        p = torch.from_numpy(prm).cuda()
        tot = dict(cold=0, warm=0, dry_hits=0, false_dry=0)
        for j in range(3):
            v = src.realization(j % 2, 500 + j)
            filled = api.pitfill(v, mode=api.FILL_EXACT)
            warm, _ = api.ws_infer(p, v, threshold=0.005)
            _, sc = api.pitfill_exact_warm(v)
            _, sw = api.pitfill_exact_warm(v, warm)
            marked = torch.isfinite(warm)
            tot["cold"] += sc["rounds"]
            tot["warm"] += sw["rounds"]
            tot["dry_hits"] += int((marked & (filled == v)).sum())
            tot["false_dry"] += int((marked & (filled > v)).sum())
        rounds[name] = tot
    print("warm-start sweep rounds:", rounds)
    assert rounds["trained"]["warm"] < rounds["trained"]["cold"]
    share = {k: r["false_dry"] / max(1, r["false_dry"] + r["dry_hits"]) for k, r in rounds.items()}
    assert share["trained"] < share["untrained"] / 3
