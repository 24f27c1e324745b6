"""The fused, graph-captured pipeline equals the oracle's realization loop
(border counts bit-exact) on the same Philox noise."""
import numpy as np
import pytest

from cases import bits, make_case

pytestmark = pytest.mark.gpu


def _oracle_counts(oracle, dem, streams, seed, reals, model, rng_m, sigma, mean=0.0):
    import torch
    from cageo_gb300 import api
    H, W = dem.shape
    r = api.filter_radius(rng_m, 10.0)
    taps = api.filter_build(model, rng_m, 10.0, r)
    mc = np.zeros((H, W), np.float32)
    noise = torch.empty((H, W), dtype=torch.float32, device="cuda")
    last = None
    for k in reals:
        api.noise_philox(noise, seed, k, mean, sigma)
        mc, filled, dirs, lab = oracle.realization(dem, streams, noise.cpu().numpy(), taps, r,
                                                   model, mc)
        last = (filled, dirs, lab)
    return mc, last


@pytest.mark.parametrize("W,H,model,graphs", [(128, 96, 1, True), (257, 131, 1, False),
                                             (200, 150, 0, True), (512, 512, 1, True)])
def test_pipeline_counts(cuda, oracle, W, H, model, graphs):
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=W)
    rng_m = 60.0 if model == 1 else 30.0
    p = api.Pipeline(dem, streams, filter_model=model, practical_range=rng_m, error_stddev=1.5,
                     seed=77, use_graphs=graphs)
    p.run(0, 3)
    p.run(3, 2)
    got = p.counts()
    f, d, lab = p.last_stages()
    ref, (rf, rd, rl) = _oracle_counts(oracle, dem, streams, 77, range(5), model, rng_m, 1.5)
    assert np.array_equal(got, ref)
    assert np.array_equal(bits(f), bits(rf))
    assert np.array_equal(d, rd)
    assert np.array_equal(lab, rl)
    p.close()


@pytest.mark.parametrize("W,H,rng_m", [(2, 2, 4.0), (3, 40, 4.0), (40, 3, 4.0), (33, 33, 30.0),
                                       (31, 65, 30.0), (65, 31, 10.0)])
def test_pipeline_small_and_thin_grids(cuda, oracle, W, H, rng_m):
    """Grids smaller than a 32x32 tile, a tile and one cell, or a few cells
    thin: partial tiles on every side, the whole grid a border."""
    from cageo_gb300 import api, synth
    dem = synth.fbm_dem(W, H, 0.8, 7 * W + H, 80.0, 180.0)
    streams = np.full((H, W), -9999.0, np.float32)
    streams[H // 2, W // 2] = 1.0  # one stream cell
    p = api.Pipeline(dem, streams, filter_model=1, practical_range=rng_m, error_stddev=1.5,
                     seed=5, use_graphs=True)
    p.run(0, 3)
    got = p.counts()
    f, d, lab = p.last_stages()
    ref, (rf, rd, rl) = _oracle_counts(oracle, dem, streams, 5, range(3), 1, rng_m, 1.5)
    assert np.array_equal(got, ref)
    assert np.array_equal(bits(f), bits(rf))
    assert np.array_equal(d, rd)
    assert np.array_equal(lab, rl)
    p.close()


def test_pipeline_nodata_zero_uses_stage_path(cuda, oracle):
    from cageo_gb300 import api
    dem, streams = make_case(96, 80, seed=5)
    p = api.Pipeline(dem, streams, nodata_dem=0.0, error_stddev=1.0, seed=3)
    p.run(0, 2)
    got = p.counts()
    import torch
    r = api.filter_radius(60.0, 10.0)
    taps = api.filter_build(1, 60.0, 10.0, r)
    mc = np.zeros_like(dem)
    noise = torch.empty(dem.shape, dtype=torch.float32, device="cuda")
    for k in range(2):
        api.noise_philox(noise, 3, k, 0.0, 1.0)
        mc, *_ = oracle.realization(dem, streams, noise.cpu().numpy(), taps, r, 1, mc,
                                    nodata_dem=0.0)
    assert np.array_equal(got, mc)


def test_pipeline_graph_equals_direct(cuda):
    from cageo_gb300 import api
    dem, streams = make_case(300, 200, seed=12)
    a = api.Pipeline(dem, streams, seed=5, use_graphs=True)
    b = api.Pipeline(dem, streams, seed=5, use_graphs=False)
    a.run(0, 6)
    b.run(0, 6)
    assert np.array_equal(a.counts(), b.counts())
    assert a.counts().max() <= 6


def test_graph_kernel_count(cuda):
    """The captured realization's kernel launches are counted from the graph
    itself; a pipeline that has not captured one refuses."""
    from cageo_gb300 import api
    dem, streams = make_case(160, 128, seed=14)
    p = api.Pipeline(dem, streams, seed=2, use_graphs=True)
    with pytest.raises(api.CageoError):
        p.graph_kernels()
    p.run(0, 3)
    n = p.graph_kernels()
    assert 10 <= n <= 64
    q = api.Pipeline(dem, streams, seed=2, use_graphs=False)
    q.run(0, 1)
    with pytest.raises(api.CageoError):
        q.graph_kernels()


def test_checkpoint_resume(cuda, tmp_path):
    from cageo_gb300 import api
    dem, streams = make_case(120, 90, seed=31)
    a = api.Pipeline(dem, streams, seed=4)
    a.run(0, 5)
    b = api.Pipeline(dem, streams, seed=4)
    b.run(0, 3)
    b.save(str(tmp_path / "ck.bin"), 3)
    c = api.Pipeline(dem, streams, seed=4)
    assert c.load(str(tmp_path / "ck.bin")) == 3
    c.run(3, 2)
    assert np.array_equal(a.counts(), c.counts())
    other = api.Pipeline(dem, streams, seed=5)
    with pytest.raises(api.CageoError, match="seed"):
        other.load(str(tmp_path / "ck.bin"))


@pytest.mark.parametrize("change,field", [
    (dict(practical_range=80.0), "practical range"),
    (dict(error_stddev=2.0), "error standard deviation"),
    (dict(filter_model=0, practical_range=30.0), "filter model"),
    (dict(bevel_radius=3), "bevel radius"),
    (dict(fill_mode=1), "fill mode"),
    (dict(nodata_stream=-1.0), "NODATA"),
    ("dem", "DEM or stream grid"),
    ("streams", "DEM or stream grid"),
])
def test_checkpoint_refuses_another_run(cuda, tmp_path, change, field):
    """A checkpoint records every setting the counts depend on and a digest
    of the input grids; loading it into a pipeline that differs in any of
    them is refused (its counts would mix two distributions)."""
    from cageo_gb300 import api
    dem, streams = make_case(96, 72, seed=33)
    a = api.Pipeline(dem, streams, seed=4)
    a.run(0, 1)
    a.save(str(tmp_path / "ck.bin"), 1)
    kw, d2, s2 = dict(seed=4), dem, streams
    if change == "dem":
        d2 = dem.copy()
        d2[10, 10] += 0.5
    elif change == "streams":
        s2 = streams.copy()
        s2[5, 7] = 1.0 if s2[5, 7] < 0 else -9999.0
    else:
        kw.update(change)
    b = api.Pipeline(d2, s2, **kw)
    with pytest.raises(api.CageoError, match=field):
        b.load(str(tmp_path / "ck.bin"))
    same = api.Pipeline(dem, streams, seed=4)
    assert same.load(str(tmp_path / "ck.bin")) == 1


def test_checkpoint_survives_an_interrupted_save(cuda, tmp_path):
    """A save writes "<path>.tmp" and renames it over the checkpoint: a save
    killed part-way (a truncated .tmp left behind) leaves the previous
    checkpoint whole, and the next save replaces both."""
    from cageo_gb300 import api
    dem, streams = make_case(96, 72, seed=35)
    a = api.Pipeline(dem, streams, seed=6)
    a.run(0, 2)
    ck = tmp_path / "ck.bin"
    a.save(str(ck), 2)
    size = ck.stat().st_size
    (tmp_path / "ck.bin.tmp").write_bytes(ck.read_bytes()[: size // 3])
    b = api.Pipeline(dem, streams, seed=6)
    assert b.load(str(ck)) == 2
    assert np.array_equal(a.counts(), b.counts())
    a.run(2, 1)
    a.save(str(ck), 3)
    assert not (tmp_path / "ck.bin.tmp").exists()
    assert b.load(str(ck)) == 3
    # a truncated checkpoint itself is refused, not half-loaded
    (tmp_path / "cut.bin").write_bytes(ck.read_bytes()[: size - 4])
    with pytest.raises(api.CageoError, match="not a complete checkpoint"):
        b.load(str(tmp_path / "cut.bin"))


def test_autotune_keeps_counts(cuda):
    """The autotuner only changes launch settings (the fill's sweep rounds
    per tile visit and warps per SM of its lower-bound flood, the front's
    convolution tile): counts, filled surface and labels equal an untuned
    pipeline's under every setting."""
    from cageo_gb300 import api
    dem, streams = make_case(300, 200, seed=44)
    a = api.Pipeline(dem, streams, error_stddev=1.5, seed=9)
    best, ms = a.autotune(1000, trials=2)
    cands = api.autotune_candidates()
    fill = [c for c in cands if c["fill_rounds"]]
    assert len(ms) == len(cands) and all(v > 0 for _, v in ms)  # Gaussian: every tile applies
    assert {c["fill_warps"] for c in fill} == {16, 20, 22}
    assert {c["conv_tile"] for c in cands} == set(range(len(api.CONV_TILES)))
    assert dict(best, conv_tile=0) in fill and 0 <= best["conv_tile"] < len(api.CONV_TILES)
    assert a.tuning() == best
    a.run(0, 3)
    b = api.Pipeline(dem, streams, error_stddev=1.5, seed=9)
    b.run(0, 3)
    assert np.array_equal(a.counts(), b.counts())
    fb = b.last_stages()
    for rounds, warps, tile in [(1, 16, 0), (4, 22, 1), (1024, 20, 2), (16, 20, 3)]:
        c = api.Pipeline(dem, streams, error_stddev=1.5, seed=9)
        c.set_tuning(rounds, warps, tile)
        c.run(0, 3)
        assert np.array_equal(c.counts(), b.counts())
        fc = c.last_stages()
        assert np.array_equal(bits(fc[0]), bits(fb[0])) and np.array_equal(fc[2], fb[2])
    with pytest.raises(api.CageoError):
        c.set_tuning(32, 18)
    with pytest.raises(api.CageoError):
        c.set_tuning(32, 20, len(api.CONV_TILES))


@pytest.mark.parametrize("range_m", [60.0, 90.0, 40.0])
def test_conv_tiles_same_results(cuda, range_m):
    """Every convolution tile shape of the fused front gives the same counts,
    filled surface, directions and labels, single and in batched steps, for
    the unrolled radii (15 and 23) and the generic kernel (10), on a grid
    whose sides are multiples of no tile."""
    from cageo_gb300 import api
    dem, streams = make_case(333, 211, seed=46)
    runs = []
    for tile in range(len(api.CONV_TILES)):
        for batch in (1, 3):
            p = api.Pipeline(dem, streams, practical_range=range_m, error_stddev=1.5, seed=12)
            p.set_tuning(64, 20, tile)
            p.set_batch(batch)
            p.run(0, 6)
            runs.append(((tile, batch), p.counts(), p.last_stages()))
            p.close()
    (_, c0, (f0, d0, l0)) = runs[0]
    assert c0.max() > 0
    for key, c, (f, d, lab) in runs[1:]:
        assert np.array_equal(c, c0), key
        assert np.array_equal(bits(f), bits(f0)) and np.array_equal(d, d0), key
        assert np.array_equal(lab, l0), key


def test_conv_tiles_exponential(cuda):
    """Exponential filters run the 2D kernel: only the first tile applies;
    the autotuner skips the others (0 ms)."""
    from cageo_gb300 import api
    dem, streams = make_case(200, 150, seed=47)
    p = api.Pipeline(dem, streams, filter_model=api.FILTER_EXPONENTIAL, practical_range=50.0,
                     error_stddev=1.5, seed=3)
    with pytest.raises(api.CageoError):
        p.set_tuning(64, 20, 1)
    best, ms = p.autotune(0, trials=1)
    assert best["conv_tile"] == 0
    assert [v for c, v in ms if c["conv_tile"]] == [0.0] * (len(api.CONV_TILES) - 1)
    assert all(v > 0 for c, v in ms if not c["conv_tile"])


@pytest.mark.parametrize("batch", [1, 3])
def test_pipeline_nodata_cells(cuda, oracle, batch):
    """NODATA DEM cells make the fill's minimum -9999: the set-up the fused
    front makes (which assumes a minimum of 0) is redone by the fill."""
    import torch
    from cageo_gb300 import api
    dem, streams = make_case(150, 110, seed=43, nodata_cells=40)
    p = api.Pipeline(dem, streams, error_stddev=1.5, seed=12)
    p.set_batch(batch)
    p.run(0, 6)
    got = p.counts()
    f, d, lab = p.last_stages()
    r = api.filter_radius(60.0, 10.0)
    taps = api.filter_build(1, 60.0, 10.0, r)
    mc = np.zeros_like(dem)
    noise = torch.empty(dem.shape, dtype=torch.float32, device="cuda")
    for k in range(6):
        api.noise_philox(noise, 12, k, 0.0, 1.5)
        mc, rf, rd, rl = oracle.realization(dem, streams, noise.cpu().numpy(), taps, r, 1, mc)
    assert np.array_equal(got, mc)
    assert np.array_equal(bits(f), bits(rf)) and np.array_equal(d, rd)
    assert np.array_equal(lab, rl)
