"""Parity at the benchmark configurations' full sizes: the fused, graph-captured
pipeline against the oracle's realization loop on the same Philox noise --
border counts, filled surface, flow directions and basin labels bit-exact.

* plain-4096: 4096^2 fBm DEM (seed 1, Hurst 0.75, 0-300 m, 2000 pits),
  streams at accumulation 2000, Gaussian 60 m, sd 1.5 m; 3 realizations,
  single and as one batched step of 3.
* eval-8192: 8192^2 (Hurst 0.8, 20000 pits), Gaussian 60 m; 2 realizations,
  single and as one batched step of 2.
* the batched workload's four grids at full size (2048^2, 257x1013,
  1500x733, 3001x401) with exponential filters of radius 8, 19 and 30.
* stress-16384: 16384^2 with 20 % flat lake plateaus (discs of 50-400
  cells), Gaussian 90 m; 1 realization.  The longest terminating trace path
  is measured and must stay within the reference walk's step cap
  (src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:66-75).

Stream rasters carry per-component ids so the labels tell basins apart.
These are the slow GPU tests: the oracle runs the reference's serial
bucket fill and walk at full size."""
import numpy as np
import pytest

from cases import bits

pytestmark = pytest.mark.gpu

# The reference walk gives up once a path has taken more than 100000 steps.
TRACE_STEP_CAP = 100000


def _oracle_run(oracle, dem, streams, seed, reals, model, rng_m, sigma):
    import torch
    from cageo_gb300 import api
    H, W = dem.shape
    r = api.filter_radius(rng_m, 10.0)
    taps = api.filter_build(model, rng_m, 10.0, r)
    mc = np.zeros((H, W), np.float32)
    noise = torch.empty((H, W), dtype=torch.float32, device="cuda")
    last = None
    for k in reals:
        api.noise_philox(noise, seed, k, 0.0, sigma)
        mc, filled, dirs, lab = oracle.realization(dem, streams, noise.cpu().numpy(), taps, r,
                                                   model, mc)
        last = (filled, dirs, lab)
    return mc, last


def _check_workload(oracle, name, reals, seed, batch=1):
    """The pipeline (single realizations, and with batch > 1 also in batched
    steps of `batch`) against the oracle."""
    from cageo_gb300 import api, synth
    dem, streams, p = synth.workload(name, ids="components")
    runs = []
    for b in sorted({1, batch}):
        pipe = api.Pipeline(dem, streams, cell_size=p["cell"], filter_model=api.FILTER_GAUSSIAN,
                            practical_range=p["range_m"], error_stddev=p["sigma"], seed=seed)
        pipe.set_batch(b)
        pipe.run(0, reals)
        runs.append((b, pipe.counts(), pipe.last_stages()))
        pipe.close()
    ref, (rf, rd, rl) = _oracle_run(oracle, dem, streams, seed, range(reals), 1, p["range_m"],
                                    p["sigma"])
    for b, got, (f, d, lab) in runs:
        assert np.array_equal(bits(f), bits(rf)), "filled surface (batch %d)" % b
        assert np.array_equal(d, rd), "flow directions (batch %d)" % b
        assert np.array_equal(lab, rl), "basin labels (batch %d)" % b
        assert np.array_equal(got, ref), "border counts (batch %d)" % b
    return dem, streams, rd


def test_plain_4096(cuda, oracle):
    _check_workload(oracle, "plain-4096", 3, seed=1, batch=3)


def test_eval_8192(cuda, oracle):
    _check_workload(oracle, "eval-8192", 2, seed=3, batch=2)


# (grid index in the batched workload, practical range in m -> radius)
BATCH_JOBS = [(0, 120.0), (1, 30.0), (2, 76.0), (3, 120.0), (0, 30.0), (3, 76.0)]


def test_batched_grids_full_size(cuda, oracle):
    """Every batch grid at its full size, exponential filters of radius 8
    (30 m), 19 (76 m) and 30 (120 m), through the batch runner."""
    from cageo_gb300 import api, batch, synth
    assert sorted({api.filter_radius(m, 10.0) for _, m in BATCH_JOBS}) == [8, 19, 30]
    grids = synth.batched_grids(seed=5, ids="components")
    jobs = [(k, 100 + j, api.FILTER_EXPONENTIAL, m, 0.0, 2.0) for j, (k, m) in
            enumerate(BATCH_JOBS)]
    b = batch.Batch(grids, seed=21)
    b.run(jobs)
    got = b.counts()
    b.close()
    ref = [np.zeros_like(d) for d, _ in grids]
    for k, real, model, rng_m, mean, sd in jobs:
        dem, streams = grids[k]
        mc, _ = _oracle_run(oracle, dem, streams, 21, [real], model, rng_m, sd)
        ref[k] = ref[k] + mc
    for k, (g, r_) in enumerate(zip(got, ref)):
        assert np.array_equal(g, r_), "grid %d" % k


def test_stress_16384_plateaus(cuda, oracle):
    dem, streams, dirs = _check_workload(oracle, "stress-16384", 1, seed=5)
    longest, never = oracle.trace_path_stats(dirs, streams)
    print("stress-16384: longest terminating trace path %d moves, %d cells without an "
          "outlet" % (longest, never))
    assert longest <= TRACE_STEP_CAP
