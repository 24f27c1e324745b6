"""Stage-by-stage parity of the CUDA kernels (through the C ABI) against the
oracle on identical inputs.  Integer and direction outputs must be equal;
float outputs bit-for-bit equal (the kernels reproduce the CPU path's float
operation order), i.e. tolerance 0."""
import numpy as np
import pytest

from cases import bits, gaussian_noise, make_case

pytestmark = pytest.mark.gpu

SHAPES = [(64, 64), (97, 61), (257, 131), (512, 512), (1013, 257)]


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("W,H", SHAPES)
@pytest.mark.parametrize("model", [1, 0])
def test_convolution(cuda, oracle, W, H, model):
    from cageo_gb300 import api
    rng_m = 60.0 if model == 1 else 40.0
    r = api.filter_radius(rng_m, 10.0)
    taps = api.filter_build(model, rng_m, 10.0, r)
    x = gaussian_noise(W, H, 3)
    got = api.convolve(_t(x, cuda), model, taps, r).cpu().numpy()
    ref = oracle.convolve(x, taps, r, model)
    assert np.array_equal(bits(got), bits(ref))


@pytest.mark.parametrize("W,H", SHAPES)
def test_realistic_and_burn(cuda, oracle, W, H):
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=W + H)
    field = gaussian_noise(W, H, 4, 3.0)
    f = _t(field, cuda)
    api.realistic_dem(_t(dem, cuda), f)
    ref = oracle.realistic_dem(dem, field)
    assert np.array_equal(bits(f.cpu().numpy()), bits(ref))
    for bevel in (2, 1, 5):
        g = f.clone()
        api.stream_burn(g, _t(streams, cuda), bevel)
        assert np.array_equal(bits(g.cpu().numpy()), bits(oracle.stream_burn(ref, streams, bevel)))


@pytest.mark.parametrize("W,H", SHAPES)
@pytest.mark.parametrize("seed", [0, 1])
def test_pitfill(cuda, oracle, W, H, seed):
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=seed)
    rdem = oracle.stream_burn(oracle.realistic_dem(dem, gaussian_noise(W, H, 10 + seed)), streams)
    q_ref, f_ref = oracle.pitfill(rdem)
    d = _t(rdem, cuda)
    filled = api.pitfill(d)
    assert np.array_equal(bits(d.cpu().numpy()), bits(q_ref)), "quantized DEM"
    assert np.array_equal(bits(filled.cpu().numpy()), bits(f_ref)), "filled DEM"


def test_pitfill_unaligned_grids(cuda, oracle):
    """A grid that starts 4 bytes past a 16-byte boundary (a tensor view)
    fills the same.  A workspace off its 256-byte boundary is refused before
    any launch."""
    import torch
    from cageo_gb300 import api
    W, H = 512, 96
    dem, streams = make_case(W, H, seed=5)
    rdem = oracle.stream_burn(oracle.realistic_dem(dem, gaussian_noise(W, H, 12)), streams)
    q_ref, f_ref = oracle.pitfill(rdem)
    buf = torch.empty(W * H + 1, dtype=torch.float32, device=cuda)
    d = buf[1:].view(H, W)
    d.copy_(_t(rdem, cuda))
    assert d.data_ptr() % 16 == 4
    filled = api.pitfill(d)
    assert np.array_equal(bits(d.cpu().numpy()), bits(q_ref)), "quantized DEM"
    assert np.array_equal(bits(filled.cpu().numpy()), bits(f_ref)), "filled DEM"
    need = api.lib().cageo_pitfill_workspace_size(W, H)
    ws = torch.empty(need + 256, dtype=torch.uint8, device=cuda)[4:]
    with pytest.raises(api.CageoError) as e:
        api.pitfill(_t(rdem, cuda), workspace=ws)
    assert e.value.status == 1 and "256-byte" in str(e.value)  # CAGEO_ERR_ARGUMENT
    # The filled grid off a 16-byte boundary too, through the C ABI.
    d2 = _t(rdem, cuda)
    fbuf = torch.empty(W * H + 1, dtype=torch.float32, device=cuda)
    f2 = fbuf[1:].view(H, W)
    assert f2.data_ptr() % 16 == 4
    st = api.lib().cageo_pitfill(api._ptr(d2), api._ptr(f2), W, H, -9999.0, api.FILL_CPU_COMPAT,
                                 None, 0, api._stream())
    assert st == 0, api.lib().cageo_last_error_string()
    assert np.array_equal(bits(f2.cpu().numpy()), bits(f_ref)), "filled DEM (unaligned output)"


def test_noise_into_unaligned_field(cuda):
    """Noise written to a field that starts 4 bytes past a 16-byte boundary
    equals the noise written to an aligned one."""
    import torch
    from cageo_gb300 import api
    W, H = 301, 77
    a = torch.empty((H, W), dtype=torch.float32, device=cuda)
    api.noise_philox(a, 91, 4, 0.5, 1.5)
    buf = torch.empty(W * H + 1, dtype=torch.float32, device=cuda)
    b = buf[1:].view(H, W)
    assert b.data_ptr() % 16 == 4
    api.noise_philox(b, 91, 4, 0.5, 1.5)
    assert torch.equal(a, b)


@pytest.mark.parametrize("realization", range(4))
def test_pitfill_philox_noise(cuda, oracle, realization):
    """Fill of realistic DEMs made from the library's own Philox noise (the
    inputs the pipeline sees), 512 x 512."""
    import torch
    from cageo_gb300 import api
    W = H = 512
    dem, streams = make_case(W, H, seed=W)
    r = api.filter_radius(60.0, 10.0)
    taps = api.filter_build(api.FILTER_GAUSSIAN, 60.0, 10.0, r)
    noise = torch.empty((H, W), dtype=torch.float32, device=cuda)
    api.noise_philox(noise, 77, realization, 0.0, 1.5)
    conv = oracle.convolve(noise.cpu().numpy(), taps, r, 1)
    rdem = oracle.stream_burn(oracle.realistic_dem(dem, conv), streams)
    _, f_ref = oracle.pitfill(rdem)
    filled = api.pitfill(_t(rdem, cuda))
    assert np.array_equal(bits(filled.cpu().numpy()), bits(f_ref))


def test_pitfill_no_streams_and_nodata(cuda, oracle):
    """minE != 0 (no stream cell) and NODATA cells change the round-trip test."""
    from cageo_gb300 import api
    dem, _ = make_case(160, 120, seed=7)
    dem = dem + np.float32(3.25)
    dem.reshape(-1)[np.random.default_rng(1).choice(dem.size, 40, replace=False)] = -9999.0
    q_ref, f_ref = oracle.pitfill(dem)
    d = _t(dem, cuda)
    filled = api.pitfill(d)
    assert np.array_equal(bits(filled.cpu().numpy()), bits(f_ref))


@pytest.mark.parametrize("W,H", SHAPES)
def test_routing(cuda, oracle, W, H):
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=3)
    rdem = oracle.stream_burn(oracle.realistic_dem(dem, gaussian_noise(W, H, 5)), streams)
    _, filled = oracle.pitfill(rdem)
    dirs = api.route_d8(_t(filled, cuda)).cpu().numpy()
    assert np.array_equal(dirs, oracle.flow_route(filled))


def test_routing_plateaus(cuda, oracle):
    """Large flat areas exercise the layered flat BFS and its tie rule."""
    from cageo_gb300 import api
    dem, streams = make_case(300, 220, seed=9, plateaus=0.3)
    _, filled = oracle.pitfill(oracle.stream_burn(dem, streams))
    dirs = api.route_d8(_t(filled, cuda)).cpu().numpy()
    assert np.array_equal(dirs, oracle.flow_route(filled))


@pytest.mark.parametrize("W,H", SHAPES)
def test_trace_and_border(cuda, oracle, W, H):
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=4)
    rdem = oracle.stream_burn(oracle.realistic_dem(dem, gaussian_noise(W, H, 6)), streams)
    _, filled = oracle.pitfill(rdem)
    dirs = oracle.flow_route(filled)
    lab = api.trace(_t(dirs, cuda), _t(streams, cuda))
    ref = oracle.flow_trace(dirs, streams)
    assert np.array_equal(lab.cpu().numpy(), ref)
    import torch
    mc = torch.full((H, W), 3.0, device=cuda)
    api.border_accumulate(lab, mc)
    assert np.array_equal(mc.cpu().numpy(), oracle.border_accumulate(ref, np.full((H, W), 3.0, np.float32)))


@pytest.mark.parametrize("x0", [5, 31])
def test_trace_cycle_is_an_error(cuda, x0):
    """Directions that form a cycle never reach an outlet: tracing reports
    CAGEO_ERR_NO_CONVERGENCE, whether the cycle stays inside a 32x32 tile
    (x0 = 5) or crosses into the next one (x0 = 31)."""
    from cageo_gb300 import api
    H, W = 40, 70
    dirs = np.zeros((H, W, 2), np.int8)
    dirs[..., 1] = -1  # everything flows north, out of the grid
    dirs[10, x0] = (1, 0)      # (x0, 10) -> (x0 + 1, 10)
    dirs[10, x0 + 1] = (-1, 0)  # and back
    streams = np.full((H, W), -9999.0, np.float32)
    with pytest.raises(api.CageoError) as e:
        api.trace(_t(dirs, cuda), _t(streams, cuda))
    assert e.value.status == 3  # CAGEO_ERR_NO_CONVERGENCE


def test_trace_dead_ends(cuda, oracle):
    """Cells without a direction never terminate in the reference; they and
    label-0 streams take cell 0's label in its connect pass."""
    from cageo_gb300 import api
    rng = np.random.default_rng(2)
    H, W = 40, 50
    dirs = rng.integers(-1, 2, size=(H, W, 2)).astype(np.int8)
    # make directions acyclic: point everything left/up-ish except some dead ends
    dirs[..., 0] = -1
    dirs[rng.random((H, W)) < 0.05] = 0
    streams = np.full((H, W), -9999.0, np.float32)
    streams[rng.random((H, W)) < 0.05] = 0.0   # label-0 streams
    streams[rng.random((H, W)) < 0.05] = 2.0
    lab = api.trace(_t(dirs, cuda), _t(streams, cuda)).cpu().numpy()
    assert np.array_equal(lab, oracle.flow_trace(dirs, streams))
