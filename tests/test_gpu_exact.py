"""Exact mode (the reference GPU path's semantics: exact float fill, GPU flat
order, dead ends reported) on the GPU against the oracle, bit-exact."""
import numpy as np
import pytest

from cases import bits, make_case

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("W,H,seed,plateaus,nod", [(96, 80, 1, 0.0, 0), (257, 131, 2, 0.2, 0),
                                                   (300, 200, 3, 0.0, 200), (512, 512, 4, 0.1, 0),
                                                   (1500, 733, 5, 0.0, 0)])
def test_exact_fill(cuda, oracle, W, H, seed, plateaus, nod):
    from cageo_gb300 import api
    dem, _ = make_case(W, H, seed=seed, plateaus=plateaus, nodata_cells=nod)
    d = _t(dem)
    got = api.pitfill(d, mode=api.FILL_EXACT).cpu().numpy()
    assert np.array_equal(bits(d.cpu().numpy()), bits(dem))  # input untouched
    ref = oracle.pitfill_exact(dem)
    assert np.array_equal(bits(got), bits(ref))


def test_exact_fill_unreached_cells(cuda, oracle):
    from cageo_gb300 import api
    dem = np.full((70, 90), 50.0, np.float32)
    dem[30:40, 30:40] = -9999.0
    dem[33:37, 33:37] = 10.0  # enclosed by NODATA
    got = api.pitfill(_t(dem), mode=api.FILL_EXACT).cpu().numpy()
    assert np.all(got[33:37, 33:37] == np.float32(99990000.0))
    assert np.array_equal(bits(got), bits(oracle.pitfill_exact(dem)))


def test_exact_fill_static(cuda, oracle):
    import torch
    from cageo_gb300 import api
    dem, _ = make_case(400, 300, seed=9)
    d = _t(dem)
    out = torch.empty_like(d)
    api._check(api.lib().cageo_pitfill_static(api._ptr(d), api._ptr(out), 400, 300, -9999.0,
                                              api.FILL_EXACT, api._stream()))
    assert np.array_equal(bits(out.cpu().numpy()), bits(oracle.pitfill_exact(dem)))


@pytest.mark.parametrize("W,H,seed,plateaus,nod", [(128, 96, 1, 0.3, 0), (301, 257, 2, 0.2, 100),
                                                   (640, 480, 3, 0.25, 0)])
def test_gpu_order_routing(cuda, oracle, W, H, seed, plateaus, nod):
    from cageo_gb300 import api
    dem, _ = make_case(W, H, seed=seed, plateaus=plateaus, nodata_cells=nod)
    filled = oracle.pitfill_exact(dem)
    d, fd = api.route_d8(_t(filled), with_flatdist=True, mode=api.ROUTE_GPU_ORDER)
    rd, rfd = oracle.flow_route_gpu(filled, with_flatdist=True)
    assert np.array_equal(fd.cpu().numpy(), rfd)
    assert np.array_equal(d.cpu().numpy(), rd)
    # Unfilled grids hold closed flats: they stay unresolved in both.
    d2, fd2 = api.route_d8(_t(dem), with_flatdist=True, mode=api.ROUTE_GPU_ORDER)
    rd2, rfd2 = oracle.flow_route_gpu(dem, with_flatdist=True)
    assert np.array_equal(fd2.cpu().numpy(), rfd2)
    assert np.array_equal(d2.cpu().numpy(), rd2)


def test_dead_end_tracing(cuda, oracle):
    from cageo_gb300 import api
    dem, streams = make_case(200, 160, seed=6, plateaus=0.2)
    rd = oracle.flow_route_gpu(dem)  # unfilled: pits are dead ends
    assert (np.abs(rd).sum(axis=2) == 0).sum() > 0
    lab = api.trace(_t(rd), _t(streams), mode=api.TRACE_DEAD_END_ERROR).cpu().numpy()
    ref = oracle.flow_trace_gpu(rd, streams)
    assert (ref == api.ERROR).sum() > 0
    assert np.array_equal(lab, ref)


@pytest.mark.parametrize("W,H,model,graphs", [(128, 96, 1, True), (257, 131, 1, False),
                                             (200, 150, 0, True), (512, 512, 1, True)])
def test_exact_pipeline(cuda, oracle, W, H, model, graphs):
    import torch
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=W + 1)
    rng_m = 60.0 if model == 1 else 30.0
    p = api.Pipeline(dem, streams, filter_model=model, practical_range=rng_m, error_stddev=1.5,
                     seed=21, use_graphs=graphs, fill_mode=api.FILL_EXACT)
    p.run(0, 2)
    p.run(2, 2)
    got = p.counts()
    f, d, lab = p.last_stages()
    r = api.filter_radius(rng_m, 10.0)
    taps = api.filter_build(model, rng_m, 10.0, r)
    mc = np.zeros((H, W), np.float32)
    noise = torch.empty((H, W), dtype=torch.float32, device="cuda")
    for k in range(4):
        api.noise_philox(noise, 21, k, 0.0, 1.5)
        mc, rf, rd, rl = oracle.realization_exact(dem, streams, noise.cpu().numpy(), taps, r,
                                                  model, mc)
    assert np.array_equal(got, mc)
    assert np.array_equal(bits(f), bits(rf))
    assert np.array_equal(d, rd)
    assert np.array_equal(lab, rl)
    p.close()


@pytest.mark.parametrize("start", ["all_dry", "random", "answer", "above"])
def test_warm_exact_fill_verifies_itself(cuda, oracle, start):
    """Any warm start gives the exact fill: cells whose level no chain of
    relays from an outlet supports restart from +inf inside the fill."""
    import torch
    from cageo_gb300 import api
    from cases import make_case
    dem, _ = make_case(300, 220, seed=71, plateaus=0.2)
    v = torch.from_numpy(dem).to(cuda)
    ref = oracle.pitfill_exact(dem)
    rng = np.random.default_rng(5)
    if start == "all_dry":
        warm = v.clone()  # every cell at its own elevation: every pit too low
    elif start == "random":
        warm = v + torch.from_numpy(rng.uniform(-3, 3, dem.shape).astype(np.float32)).to(cuda)
    elif start == "answer":
        warm = torch.from_numpy(ref).to(cuda)
    else:
        warm = torch.from_numpy(ref + 1.0).to(cuda)
    filled, st = api.pitfill_exact_warm(v, warm)
    assert np.array_equal(filled.cpu().numpy().view(np.int32), ref.view(np.int32))
    if start in ("answer", "above"):
        assert st["reset_cells"] == 0  # every start is supported once relaxed
    if start == "all_dry":
        assert st["reset_cells"] > 0
