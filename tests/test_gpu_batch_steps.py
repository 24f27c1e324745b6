"""Batched steps (cageo_pipeline_set_batch): realizations processed K at a
time, their fills sharing one stacked grid, give the same counts and stage
outputs as single realizations and as the oracle, bit for bit."""
import numpy as np
import pytest

from cases import bits, make_case

pytestmark = pytest.mark.gpu


def _oracle(oracle, dem, streams, seed, reals, rng_m=60.0, sigma=1.5):
    import torch
    from cageo_gb300 import api
    r = api.filter_radius(rng_m, 10.0)
    taps = api.filter_build(api.FILTER_GAUSSIAN, rng_m, 10.0, r)
    mc = np.zeros(dem.shape, np.float32)
    noise = torch.empty(dem.shape, dtype=torch.float32, device="cuda")
    last = None
    for k in reals:
        api.noise_philox(noise, seed, k, 0.0, sigma)
        mc, f, d, lab = oracle.realization(dem, streams, noise.cpu().numpy(), taps, r, 1, mc)
        last = (f, d, lab)
    return mc, last


@pytest.mark.parametrize("W,H,K,count,graphs", [(128, 96, 2, 5, True), (257, 131, 3, 7, True),
                                                (200, 150, 4, 8, False), (512, 512, 4, 9, True),
                                                (65, 33, 5, 5, True), (40, 2000, 40, 41, True)])
def test_batched_equals_oracle(cuda, oracle, W, H, K, count, graphs):
    """Counts after `count` realizations in steps of K (plus the remainder
    singly), and the last realization's stage outputs."""
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=W + K)
    p = api.Pipeline(dem, streams, error_stddev=1.5, seed=17, use_graphs=graphs)
    p.set_batch(K)
    p.run(0, count)
    got = p.counts()
    f, d, lab = p.last_stages()
    ref, (rf, rd, rl) = _oracle(oracle, dem, streams, 17, range(count))
    assert np.array_equal(got, ref)
    assert np.array_equal(bits(f), bits(rf))
    assert np.array_equal(d, rd)
    assert np.array_equal(lab, rl)
    # A second run continues the same counts, batched steps and all.
    p.run(count, K)
    ref2, _ = _oracle(oracle, dem, streams, 17, range(count + K))
    assert np.array_equal(p.counts(), ref2)
    p.close()


def test_batched_equals_single(cuda):
    """Several batch sizes against the single-realization pipeline."""
    from cageo_gb300 import api
    dem, streams = make_case(300, 200, seed=61, plateaus=0.2)
    single = api.Pipeline(dem, streams, error_stddev=2.0, seed=3)
    single.run(10, 12)
    want = single.counts()
    fw, dw, lw = single.last_stages()
    for K in (2, 3, 6, 12):
        p = api.Pipeline(dem, streams, error_stddev=2.0, seed=3)
        p.set_batch(K)
        p.run(10, 12)
        assert np.array_equal(p.counts(), want), K
        f, d, lab = p.last_stages()
        assert np.array_equal(bits(f), bits(fw)) and np.array_equal(d, dw)
        assert np.array_equal(lab, lw)
        p.set_batch(1)  # back to single realizations
        p.run(22, 1)
        p.close()


def test_batch_refusals(cuda):
    from cageo_gb300 import api
    dem, streams = make_case(96, 80, seed=5)
    p = api.Pipeline(dem, streams, seed=1)
    for bad in (0, 65):
        with pytest.raises(api.CageoError):
            p.set_batch(bad)
    big = api.Pipeline(np.zeros((8192, 8192), np.float32) + 50.0,
                       np.full((8192, 8192), -9999.0, np.float32), seed=1)
    with pytest.raises(api.CageoError, match="2\\^31"):
        big.set_batch(32)
    big.close()
    exact = api.Pipeline(dem, streams, seed=1, fill_mode=api.FILL_EXACT)
    with pytest.raises(api.CageoError, match="CPU-compatible"):
        exact.set_batch(2)
