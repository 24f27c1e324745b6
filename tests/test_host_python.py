"""Host-side Python helpers that need no GPU: the synthetic workloads, the
batched job mix and the warm-start network's parameter layout."""
import numpy as np

from cageo_gb300 import api, batch, learned, synth


def test_workload_is_seeded_and_shaped():
    d1, s1, p1 = synth.workload("plain-512")
    d2, s2, p2 = synth.workload("plain-512")
    assert d1.shape == s1.shape == (512, 512) and d1.dtype == s1.dtype == np.float32
    assert np.array_equal(d1, d2) and np.array_equal(s1, s2) and p1 == p2
    assert set(np.unique(s1)) <= {1.0, -9999.0} and (s1 >= 0).sum() > 0
    assert float(d1.min()) >= 80.0 - 3.0 - 1e-3 and float(d1.max()) <= 180.0 + 1e-3  # relief minus pits
    small, _, ps = synth.workload("plain-4096", scale=1 / 16)
    assert small.shape == (256, 256) and ps["pits"] == max(int(2000 / 256), 1)


def test_mixed_jobs_cover_every_dem_with_drawn_filters():
    jobs = batch.mixed_jobs(4, 256, seed=5)
    assert jobs == batch.mixed_jobs(4, 256, seed=5)
    assert [j[0] for j in jobs[:8]] == [0, 1, 2, 3, 0, 1, 2, 3]
    assert [j[1] for j in jobs] == list(range(256))
    assert all(j[2] == api.FILTER_EXPONENTIAL and j[4] == 0.0 for j in jobs)
    rng_m = np.array([j[3] for j in jobs])
    sd = np.array([j[5] for j in jobs])
    assert 30.0 <= rng_m.min() and rng_m.max() <= 120.0 and 1.0 <= sd.min() and sd.max() <= 3.0
    radii = {api.filter_radius(float(r), 10.0) for r in rng_m}
    assert min(radii) >= 8 and max(radii) <= 30


def test_warmstart_parameter_layout():
    """He-scaled weights of the three 3x3 layers (4 -> 32 -> 32 -> 1), zero
    biases, 10721 values in the kernels' order: w1, b1, w2, b2, w3, b3."""
    p = learned.init_params(seed=1)
    assert p.shape == (learned.N_PARAMS,) and p.dtype == np.float32
    w1, b1 = p[0:1152], p[1152:1184]
    w2, b2 = p[1184:10400], p[10400:10432]
    w3, b3 = p[10432:10720], p[10720:]
    assert not b1.any() and not b2.any() and not b3.any() and b3.size == 1
    assert abs(w1.std() - np.sqrt(2 / 36)) < 0.05 and abs(w2.std() - np.sqrt(2 / 288)) < 0.01
    assert abs(w3.std() - np.sqrt(1 / 288)) < 0.02
    trained = learned.load_params()
    assert trained.shape == p.shape and np.isfinite(trained).all()
    meta = learned.load_meta()
    assert meta["steps"] > 0 and "evaluation" in meta


def test_plateaus_cover_their_share():
    """Lake plateaus: discs flattened to their centre elevation until the
    requested share of the area is flat (the stress workload asks 20% in
    discs of radius 50-400 cells at 16384^2, Gaussian 90 m: radius 23)."""
    dem = synth.fbm_dem(600, 500, 0.8, 3, 0.0, 300.0)
    flat = synth.add_plateaus(dem, 0.2, seed=3, radius=(5, 40))
    assert np.array_equal(synth.add_plateaus(dem, 0.2, seed=3, radius=(5, 40)), flat)
    changed = np.count_nonzero(flat != dem) / dem.size
    # Each disc keeps its centre's value; the last disc may overshoot by its area.
    assert 0.2 - 0.01 <= changed <= 0.2 + np.pi * 40 ** 2 / dem.size
    # Flattened cells equal a neighbour exactly (the fBm surface alone almost never does).
    eq = np.zeros(dem.shape, bool)
    for dy, dx in ((0, 1), (0, -1), (1, 0), (-1, 0)):
        eq |= flat == np.roll(flat, (dy, dx), axis=(0, 1))
    assert np.count_nonzero(eq) / dem.size >= 0.19
    p = synth.WORKLOADS["stress-16384"]
    assert (p["width"], p["height"], p["plateaus"], p["range_m"]) == (16384, 16384, 0.2, 90.0)
    assert api.filter_radius(p["range_m"], p["cell"]) == 23
