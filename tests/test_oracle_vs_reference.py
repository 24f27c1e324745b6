"""The oracle's restatement against the reference's own CPU stage code
(oracle/_ref, compiled from the reference sources where they are present),
stage by stage, on every golden fixture and on further seeded cases:
uneven shapes, plateaus, NODATA DEM cells, both filter models and every
bevel radius.  Skipped where the reference harness is not built."""
import os

import numpy as np
import pytest

from cases import bits, gaussian_noise, make_case


@pytest.fixture(scope="module")
def ref():
    from oracle import Reference
    if not os.path.exists(Reference.path):
        pytest.skip("reference harness not built here")
    return Reference()


def _stages(impl, dem, noise, streams, taps, r, model, bevel, nodata_dem=-9999.0,
            nodata_stream=-9999.0):
    conv = impl.convolve(noise, taps, r, model)
    real = impl.realistic_dem(dem, conv, nodata_dem)
    burned = impl.stream_burn(real, streams, bevel, nodata_dem, nodata_stream)
    q, filled = impl.pitfill(burned, nodata_dem)
    dirs = impl.flow_route(filled)
    labels = impl.flow_trace(dirs, streams)
    mc = impl.border_accumulate(labels, np.full(dem.shape, 2.0, np.float32))
    return dict(conv=conv, realistic=real, burned=burned, quantized=q, filled=filled,
                dirs=dirs, labels=labels, border=mc)


def _same(a, b):
    return np.array_equal(bits(a), bits(b))


def test_reference_regenerates_every_fixture(ref):
    from test_golden import GOLDEN
    for path in GOLDEN:
        g = np.load(path)
        got = _stages(ref, g["dem"], g["noise"], g["streams"], g["taps"], int(g["radius"]),
                      int(g["model"]), 2)
        for k, v in got.items():
            want = g[k] if k != "border" else g["border"] + 2.0
            assert _same(v, want), (os.path.basename(path), k)


CASES = [
    # W, H, seed, model, bevel, extra case options
    (97, 61, 1, 1, 2, {}),
    (131, 257, 2, 0, 1, {}),
    (200, 150, 3, 1, 5, dict(plateaus=0.3)),
    (160, 120, 4, 1, 3, dict(nodata_cells=60)),
    (64, 300, 5, 0, 4, dict(hurst=0.6, lo=0.0, hi=40.0)),
]


@pytest.mark.parametrize("W,H,seed,model,bevel,opts", CASES,
                         ids=["%dx%d-m%d-b%d" % (c[0], c[1], c[3], c[4]) for c in CASES])
def test_port_matches_reference_seeded(oracle, ref, W, H, seed, model, bevel, opts):
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=seed, **opts)
    rng_m = 60.0 if model == 1 else 30.0
    r = api.filter_radius(rng_m, 10.0)
    taps = api.filter_build(model, rng_m, 10.0, r)
    noise = gaussian_noise(W, H, 100 + seed, 1.5)
    a = _stages(oracle, dem, noise, streams, taps, r, model, bevel)
    b = _stages(ref, dem, noise, streams, taps, r, model, bevel)
    for k in a:
        assert _same(a[k], b[k]), k
    # the cases reach the paths they are meant to
    if opts.get("plateaus"):
        assert (b["filled"] > b["quantized"]).any()
    if opts.get("nodata_cells"):
        nod = dem == -9999.0
        assert np.array_equal(b["realistic"][nod], np.where(b["conv"][nod] <= 0, 1.0,
                                                            b["conv"][nod]).astype(np.float32))


@pytest.mark.parametrize("noise_seed", [7, 8])
def test_port_matches_reference_plain512(oracle, ref, noise_seed):
    """The 512 x 512 workload (Hurst 0.8, 80-180 m, 200 pits, streams above
    500 cells, Gaussian 60 m, sigma 1.5) at full size."""
    from cageo_gb300 import api, synth
    dem, streams, p = synth.workload("plain-512")
    r = api.filter_radius(p["range_m"], p["cell"])
    taps = api.filter_build(api.FILTER_GAUSSIAN, p["range_m"], p["cell"], r)
    noise = gaussian_noise(p["width"], p["height"], noise_seed, p["sigma"])
    a = _stages(oracle, dem, noise, streams, taps, r, 1, 2)
    b = _stages(ref, dem, noise, streams, taps, r, 1, 2)
    for k in a:
        assert _same(a[k], b[k]), k


def test_port_matches_reference_uneven_tiles(oracle, ref):
    """The batch's uneven grids (257 x 1013, 1500 x 733, 3001 x 401) at full
    size with the exponential filter at 30, 75 and 120 m (radius 8, 19, 30)."""
    from cageo_gb300 import api, synth
    for (dem, streams), rng_m in zip(synth.batched_grids()[1:], (30.0, 75.0, 120.0)):
        H, W = dem.shape
        r = api.filter_radius(rng_m, 10.0)
        taps = api.filter_build(api.FILTER_EXPONENTIAL, rng_m, 10.0, r)
        noise = gaussian_noise(W, H, 3, 2.0)
        a = _stages(oracle, dem, noise, streams, taps, r, 0, 2)
        b = _stages(ref, dem, noise, streams, taps, r, 0, 2)
        for k in a:
            assert _same(a[k], b[k]), (W, H, k)


@pytest.mark.parametrize("nodata_dem, nodata_stream", [(0.0, -9999.0), (-9999.0, 0.0), (-1.0, -1.0)])
def test_port_matches_reference_other_nodata(oracle, ref, nodata_dem, nodata_stream):
    """NODATA values other than -9999 in the DEM and the stream raster.
    With a DEM NODATA of 0 the burned stream cells equal NODATA, and the
    reference's in-place OpenMP burn reads neighbours that other threads
    may already have zeroed (src/streamburning/StreamBurningAlgorithmCPUOpenMP.h:46-71):
    its result then depends on the thread schedule.  The port burns in
    raster order, which is what the reference gives on one thread, so the
    reference runs on one OpenMP thread here."""
    import ctypes
    from cageo_gb300 import api
    dem, streams = make_case(120, 90, seed=3, nodata_cells=30)
    dem[dem == -9999.0] = nodata_dem
    streams = np.where(streams == -9999.0, np.float32(nodata_stream), streams).astype(np.float32)
    taps = api.filter_build(api.FILTER_GAUSSIAN, 60.0, 10.0, 15)
    noise = gaussian_noise(120, 90, 4, 1.5)
    a = _stages(oracle, dem, noise, streams, taps, 15, 1, 2, nodata_dem, nodata_stream)
    gomp = ctypes.CDLL("libgomp.so.1")
    threads = gomp.omp_get_max_threads()
    gomp.omp_set_num_threads(1)
    try:
        b = _stages(ref, dem, noise, streams, taps, 15, 1, 2, nodata_dem, nodata_stream)
    finally:
        gomp.omp_set_num_threads(threads)
    for k in a:
        assert _same(a[k], b[k]), k


def test_port_matches_reference_stream_values(oracle, ref):
    """Stream rasters with fractional, zero and negative (non-NODATA) ids:
    burning treats every non-NODATA value as a stream, tracing only values
    >= 0, and labels are -(int)id (src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:58-99)."""
    from cageo_gb300 import api
    dem, streams = make_case(140, 100, seed=8)
    ids = streams >= 0
    vals = np.random.default_rng(5).choice(np.array([2.7, 0.0, -5.0, 3.0, 0.4], np.float32),
                                           size=int(ids.sum()))
    streams[ids] = vals
    taps = api.filter_build(api.FILTER_GAUSSIAN, 60.0, 10.0, 15)
    noise = gaussian_noise(140, 100, 9, 1.5)
    a = _stages(oracle, dem, noise, streams, taps, 15, 1, 2)
    b = _stages(ref, dem, noise, streams, taps, 15, 1, 2)
    for k in a:
        assert _same(a[k], b[k]), k


def test_port_matches_reference_trace_dead_ends(oracle, ref):
    """Directions with dead ends (no direction off the border) and label-0
    streams: the reference's walk gives up after its step limit and the
    connect pass copies cell 0's label (src/flowtracing/FlowTracingAlgorithmCPUOpenMP.h:66-75,115-134)."""
    rng = np.random.default_rng(5)
    H, W = 40, 50
    dirs = rng.integers(-1, 2, size=(H, W, 2)).astype(np.int8)
    dirs[..., 0] = -1
    dirs[rng.random((H, W)) < 0.05] = 0
    st = np.full((H, W), -9999.0, np.float32)
    st[rng.random((H, W)) < 0.05] = 0.0
    st[rng.random((H, W)) < 0.05] = 2.0
    assert np.array_equal(oracle.flow_trace(dirs, st), ref.flow_trace(dirs, st))


@pytest.mark.parametrize("H,W", [(1, 1), (1, 7), (7, 1), (2, 2), (3, 3), (2, 9), (5, 4), (33, 1)])
def test_port_matches_reference_tiny_grids(oracle, ref, H, W):
    """Grids that are all or almost all border, single rows and columns:
    fill, routing, tracing and border counts."""
    rng = np.random.default_rng(H * 100 + W)
    for _ in range(5):
        dem = np.round(rng.uniform(0, 5, (H, W)), 2).astype(np.float32)
        dem[rng.random((H, W)) < 0.1] = 0.0
        streams = np.where(rng.random((H, W)) < 0.1, np.float32(1.0), np.float32(-9999.0))
        qa, fa = oracle.pitfill(dem)
        qb, fb = ref.pitfill(dem)
        assert _same(qa, qb) and _same(fa, fb)
        da, db = oracle.flow_route(fa), ref.flow_route(fb)
        assert np.array_equal(da, db)
        la, lb = oracle.flow_trace(da, streams), ref.flow_trace(db, streams)
        assert np.array_equal(la, lb)
        zero = np.zeros((H, W), np.float32)
        assert _same(oracle.border_accumulate(la, zero), ref.border_accumulate(lb, zero))
