"""Host-side behaviour of the C ABI that needs no GPU: argument validation
(refused before any device work), error strings, raster I/O."""
import ctypes

import numpy as np
import pytest

from cageo_gb300 import api

P = ctypes.c_void_p


def _err():
    return api.lib().cageo_last_error_string().decode()


def test_argument_checks_refuse_before_device_work():
    L = api.lib()
    a, b = P(4096), P(8192)  # never dereferenced: every call below fails its checks first
    assert L.cageo_convolve(a, b, 10, 10, 1, a, 10, None) == 1 and "radius" in _err()
    assert L.cageo_convolve(a, a, 10, 10, 1, a, 2, None) == 1 and "in place" in _err()
    assert L.cageo_convolve(a, b, 10, 10, 7, a, 2, None) == 1
    assert L.cageo_pitfill(a, b, 70000, 10, -9999.0, 0, None, 0, None) == 1 and "65535" in _err()
    assert L.cageo_pitfill(a, a, 10, 10, -9999.0, 0, None, 0, None) == 1
    assert L.cageo_pitfill(a, b, 10, 10, -9999.0, 3, None, 0, None) == 1
    assert L.cageo_stream_burn(a, b, 10, 10, 6, -9999.0, -9999.0, None) == 1 and "bevel" in _err()
    assert L.cageo_noise_philox(None, 10, 10, 1, 0, 0.0, 1.0, None) == 1
    assert L.cageo_pitfill_static(a, b, 4096, 4096, -9999.0, 0, None) == 1
    cfg = api.PipelineConfig(64, 64, 10.0, 9, 60.0, 0.0, 1.0, 2, -9999.0, -9999.0, 1, 1)
    p = P()
    assert L.cageo_pipeline_create(ctypes.byref(p), ctypes.byref(cfg), a, b) == 1
    cfg.filter_model = 1
    cfg.practical_range = 400.0  # radius 100 >= 64
    assert L.cageo_pipeline_create(ctypes.byref(p), ctypes.byref(cfg), a, b) == 1
    assert not p.value


def test_mode_and_workspace_checks_refuse_before_device_work():
    """Unknown modes, aliasing outputs, and caller workspaces that are too
    small or off their 256-byte boundary are refused on the host."""
    L = api.lib()
    a, b, c = P(4096), P(8192), P(12288)  # never dereferenced
    assert L.cageo_route_d8_mode(a, b, c, 10, 10, -9999.0, 5, None, 0, None) == 1
    assert "routing mode" in _err()
    assert L.cageo_trace_mode(a, b, c, 10, 10, 7, None, 0, None) == 1 and "tracing mode" in _err()
    assert L.cageo_pitfill_exact_warm(a, b, b, 10, 10, -9999.0, None, 0, None, None) == 1
    assert "alias" in _err()
    need = L.cageo_pitfill_workspace_size(64, 64)
    assert L.cageo_pitfill(a, b, 64, 64, -9999.0, 0, P(1 << 20), need - 1, None) == 1
    assert "smaller" in _err()
    assert L.cageo_pitfill(a, b, 64, 64, -9999.0, 0, P((1 << 20) + 4), need, None) == 1
    assert "256-byte" in _err()
    need_t = L.cageo_trace_workspace_size(64, 64)
    assert L.cageo_trace_mode(a, b, c, 64, 64, 0, P((1 << 20) + 64), need_t, None) == 1
    assert "256-byte" in _err()
    cfg = api.PipelineConfig(64, 64, 10.0, 1, 60.0, 0.0, 1.0, 2, -9999.0, -9999.0, 1, 1, 0)
    p = P()
    for field, bad, word in (("bevel_radius", 6, "bevel"), ("fill_mode", 2, "fill mode"),
                             ("width", 1, "grid size"), ("height", 70000, "65535")):
        good = getattr(cfg, field)
        setattr(cfg, field, bad)
        assert L.cageo_pipeline_create(ctypes.byref(p), ctypes.byref(cfg), a, b) == 1, field
        assert word in _err(), (field, _err())
        setattr(cfg, field, good)
    assert not p.value


def test_workspace_sizes_scale_with_grid():
    L = api.lib()
    s1, s2 = L.cageo_pitfill_workspace_size(512, 512), L.cageo_pitfill_workspace_size(1024, 1024)
    assert 0 < s1 < s2
    assert L.cageo_pitfill_workspace_size(0, 10) == 0
    assert L.cageo_trace_workspace_size(100, 100) > 4 * 100 * 100
    assert L.cageo_route_workspace_size(100, 100) > 4 * 100 * 100


def test_raster_roundtrip(tmp_path):
    hdr = tmp_path / "dem.hdr"
    api.write_header(str(hdr), 7, 5, 10.0, -9999.0, xll=3383178.75, yll=6720450.0)
    info = api.read_header(str(hdr))
    assert (info.ncols, info.nrows, info.cellsize, info.nodata_value) == (7, 5, 10.0, -9999.0)
    assert info.xllcorner == pytest.approx(3383178.75)
    data = np.arange(35, dtype=np.float32).reshape(5, 7)
    api.write_raster(str(tmp_path / "dem.bin"), data)
    assert np.array_equal(api.read_raster(str(tmp_path / "dem.bin"), (5, 7)), data)


def test_raster_errors(tmp_path):
    api.write_raster(str(tmp_path / "x.bin"), np.zeros(10, np.float32))
    with pytest.raises(api.CageoError) as e:
        api.read_raster(str(tmp_path / "x.bin"), (3, 4))
    assert e.value.status == 5
    with pytest.raises(api.CageoError) as e:
        api.read_raster(str(tmp_path / "missing.bin"), (3, 4))
    assert e.value.status == 4
    (tmp_path / "bad.hdr").write_text("ncols 4\nnrows 4\ncolour blue\n")
    with pytest.raises(api.CageoError) as e:
        api.read_header(str(tmp_path / "bad.hdr"))
    assert e.value.status == 5 and "colour" in _err()
    (tmp_path / "bo.hdr").write_text("ncols 4\nnrows 4\nbyteorder VAX\n")
    with pytest.raises(api.CageoError):
        api.read_header(str(tmp_path / "bo.hdr"))
    # the reference's sample header parses
    (tmp_path / "ref.hdr").write_text("ncols\t\t1560\nnrows\t\t1341\nxllcorner\t3383178.7509533\n"
                                      "yllcorner\t6720450\ncellsize\t10\nNODATA_value\t-9999\n"
                                      "byteorder\tLSBFIRST\n")
    i = api.read_header(str(tmp_path / "ref.hdr"))
    assert (i.ncols, i.nrows, i.byteorder_msb) == (1560, 1341, 0)


def test_synthetic_streams_follow_accumulation():
    from cageo_gb300 import synth
    dem = synth.add_pits(synth.fbm_dem(64, 48, 0.8, 2, 10.0, 60.0), 5, 2)
    s, acc = synth.make_streams(dem, 40, ids="components", return_accum=True)
    assert np.all((s >= 0) == (acc > 40))
    assert acc.max() <= 64 * 48 and acc.min() >= 1
    assert s[s >= 0].min() >= 1  # stream ids start at 1 (0 would alias index 0 in tracing)


def test_host_refusals_set_the_error_string(tmp_path):
    L = api.lib()
    out = (ctypes.c_float * 9)()
    assert L.cageo_filter_build(7, 60.0, 10.0, 1, out) == 1 and "filter model" in _err()
    assert L.cageo_filter_build(1, 60.0, 10.0, -1, out) == 1 and "radius" in _err()
    img = np.zeros((8, 8), np.uint8)
    p = str(tmp_path / "x.jpg").encode()
    assert L.cageo_write_jpeg(p, img.ctypes.data_as(P), 8, 8, 0) == 1 and "quality" in _err()
    assert L.cageo_write_jpeg(p, None, 8, 8, 85) == 1 and "JPEG" in _err()
    assert L.cageo_read_header(None, None) == 1 and "header" in _err()
    assert L.cageo_write_raster(None, None, 0) == 1 and "raster" in _err()


_OOM_CHILD = r"""
import ctypes, resource, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from cageo_gb300 import api
L = api.lib()
W = H = 40000
img = np.zeros(W * H, np.uint8)  # reserved, not touched
def vm_bytes():
    with open("/proc/self/status") as f:
        for line in f:
            if line.startswith("VmSize:"):
                return int(line.split()[1]) * 1024
lim = vm_bytes() + (64 << 20)
resource.setrlimit(resource.RLIMIT_AS, (lim, lim))
st = L.cageo_write_jpeg(sys.argv[2].encode(), img.ctypes.data_as(ctypes.c_void_p), W, H, 85)
print(st, L.cageo_last_error_string().decode())
"""


def test_host_allocation_failure_is_a_status_not_an_abort(tmp_path):
    """The JPEG writer's output buffer cannot be allocated under a small
    address-space limit: the call returns CAGEO_ERR_HOST with a message
    instead of letting std::bad_alloc terminate the process."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _OOM_CHILD, root, str(tmp_path / "big.jpg")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    status, msg = r.stdout.strip().split(" ", 1)
    assert int(status) == 6 and "out of host memory" in msg, r.stdout


def test_autotune_candidates_layout():
    """Host-only: the fill settings (first convolution tile), then the other
    convolution tiles with fill fields 0 (run with the chosen fill setting)."""
    c = api.autotune_candidates()
    fill = [x for x in c if x["fill_rounds"]]
    assert len(fill) == 9 and all(x["conv_tile"] == 0 for x in fill)
    assert {(x["fill_rounds"], x["fill_warps"]) for x in fill} == \
        {(r, w) for r in (16, 32, 64) for w in (16, 20, 22)}
    tiles = [x for x in c if not x["fill_rounds"]]
    assert [x["conv_tile"] for x in tiles] == list(range(1, len(api.CONV_TILES)))
    assert all(x["fill_warps"] == 0 for x in tiles) and len(c) == 9 + len(tiles)
