"""The drainage command line (reference options and file formats) and the
Philox noise generator."""
import os
import subprocess

import numpy as np
import pytest

from cases import make_case, philox_np

pytestmark = pytest.mark.gpu


def _write_inputs(tmp_path, dem, streams, nodata=-9999.0):
    from cageo_gb300 import api
    H, W = dem.shape
    d = tmp_path / "DEM"
    d.mkdir()
    for name, grid in (("dem10", dem), ("streams", streams)):
        api.write_header(str(d / (name + ".hdr")), W, H, 10.0, nodata)
        api.write_raster(str(d / (name + ".bin")), grid)
    return d


def test_drainage_cli_matches_oracle(cuda, oracle, tmp_path):
    import torch
    from cageo_gb300 import _build, api
    dem, streams = make_case(160, 120, seed=21)
    d = _write_inputs(tmp_path, dem, streams)
    cmd = [_build.DRAINAGE, "--dem-path", str(d), "--filter-type", "Gaussian",
           "--practical-range", "60", "--error-standard-deviation", "1.5", "-i", "3",
           "--seed", "9", "-o", "counts.bin"]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "DEM size: 160 x 120" in r.stdout
    got = api.read_raster(str(tmp_path / "counts.bin"), dem.shape)
    rr = api.filter_radius(60.0, 10.0)
    taps = api.filter_build(api.FILTER_GAUSSIAN, 60.0, 10.0, rr)
    noise = torch.empty(dem.shape, dtype=torch.float32, device=cuda)
    mc = np.zeros_like(dem)
    for k in range(3):
        api.noise_philox(noise, 9, k, 0.0, 1.5)
        mc, *_ = oracle.realization(dem, streams, noise.cpu().numpy(), taps, rr, 1, mc)
    assert np.array_equal(got, mc)


def test_drainage_cli_frames_and_refusals(cuda, tmp_path):
    from cageo_gb300 import _build, api
    dem, streams = make_case(64, 48, seed=22)
    d = _write_inputs(tmp_path, dem, streams)
    base = [_build.DRAINAGE, "--dem-path", str(d), "-i", "2", "--seed", "3"]
    r = subprocess.run(base + ["-o", "f.bin", "--output-option", "frames"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f0 = api.read_raster(str(tmp_path / "f_0000.bin"), dem.shape)
    f1 = api.read_raster(str(tmp_path / "f_0001.bin"), dem.shape)
    assert np.all(f1 >= f0) and f1.max() <= 2
    assert subprocess.run(base + ["--cpu"], cwd=tmp_path, capture_output=True).returncode != 0
    assert subprocess.run(base + ["--filter-type", "Spherical"], cwd=tmp_path,
                          capture_output=True).returncode != 0
    assert subprocess.run(base + ["--bogus"], cwd=tmp_path, capture_output=True).returncode != 0
    # header mismatch between DEM and streams
    api.write_header(str(d / "streams.hdr"), 65, 48, 10.0, -9999.0)
    r = subprocess.run(base, cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "don't match" in r.stdout


def test_noise_matches_philox_restatement(cuda):
    import torch
    from cageo_gb300 import api
    H, W, seed, real = 64, 96, 0x1234_5678_9ABC, 7
    t = torch.empty((H, W), dtype=torch.float32, device=cuda)
    api.noise_philox(t, seed, real, 2.0, 0.5)
    got = t.cpu().numpy().reshape(-1)
    g = np.arange(H * W // 4, dtype=np.uint64)
    c = philox_np([g, np.full_like(g, real), np.full_like(g, 0x63616765), np.zeros_like(g)],
                   (seed & 0xFFFFFFFF, seed >> 32))
    u = [((x >> np.uint64(8)).astype(np.float64) + 0.5) / 16777216.0 for x in c]
    z = np.empty(H * W)
    rad0, rad1 = np.sqrt(-2 * np.log(u[0])), np.sqrt(-2 * np.log(u[2]))
    z[0::4], z[1::4] = rad0 * np.cos(2 * np.pi * u[1]), rad0 * np.sin(2 * np.pi * u[1])
    z[2::4], z[3::4] = rad1 * np.cos(2 * np.pi * u[3]), rad1 * np.sin(2 * np.pi * u[3])
    np.testing.assert_allclose(got, 2.0 + 0.5 * z, rtol=0, atol=2e-5)  # float32 log/sincos


def test_noise_statistics_and_determinism(cuda):
    import torch
    from cageo_gb300 import api
    t = torch.empty((2048, 2048), dtype=torch.float32, device=cuda)
    api.noise_philox(t, 42, 0, 1.0, 3.0)
    a = t.clone()
    assert abs(float(a.mean()) - 1.0) < 0.01 and abs(float(a.std()) - 3.0) < 0.01
    assert torch.isfinite(a).all()
    api.noise_philox(t, 42, 0, 1.0, 3.0)
    assert torch.equal(a, t)
    api.noise_philox(t, 42, 1, 1.0, 3.0)
    assert not torch.equal(a, t)
    # odd sizes: the tail group is written, nothing beyond it
    u = torch.full((3, 7), 99.0, device=cuda)
    api.noise_philox(u[:, :5].contiguous(), 1, 0)  # contiguity copy is written, original untouched
    assert float(u.max()) == 99.0
    v = torch.empty(21, device=cuda)
    api.noise_philox(v.view(3, 7), 1, 0)
    assert torch.isfinite(v).all()


def test_to_bytes_matches_reference_formula(cuda):
    import torch
    from cageo_gb300 import api
    rng = np.random.default_rng(4)
    counts = rng.integers(0, 37, size=(100, 130)).astype(np.float32)
    got = api.to_bytes(torch.from_numpy(counts).to(cuda)).cpu().numpy()
    lo, hi = np.float32(counts.min()), np.float32(counts.max())
    ref = np.rint(np.float32(255.0) * ((counts - lo) / hi)).astype(np.uint8)
    assert np.array_equal(got, ref)
    zero = api.to_bytes(torch.zeros((4, 4), device=cuda)).cpu().numpy()
    assert np.all(zero == 0)


def test_to_bytes_matches_reference_fixture(cuda):
    """The reference's own byte images (ToByteArrayAlgorithm on the CPU,
    tests/golden/jpeg/cases.npz), rounding ties included."""
    import os
    import torch
    from cageo_gb300 import api
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "jpeg", "cases.npz"))
    n = sum(1 for k in g.files if k.startswith("counts_"))
    assert n >= 4
    for i in range(n):
        got = api.to_bytes(torch.from_numpy(g["counts_%d" % i]).to(cuda)).cpu().numpy()
        assert np.array_equal(got, g["bytes_%d" % i]), str(g["cname_%d" % i])


def test_drainage_cli_jpeg(cuda, tmp_path):
    import torch
    from cageo_gb300 import _build, api
    from jpeg_decode import decode
    dem, streams = make_case(96, 72, seed=23)
    d = _write_inputs(tmp_path, dem, streams)
    base = [_build.DRAINAGE, "--dem-path", str(d), "-i", "4", "--seed", "5"]
    assert subprocess.run(base + ["-o", "c.bin"], cwd=tmp_path, capture_output=True).returncode == 0
    assert subprocess.run(base + ["-o", "c.jpg"], cwd=tmp_path, capture_output=True).returncode == 0
    counts = api.read_raster(str(tmp_path / "c.bin"), dem.shape)
    img = api.to_bytes(torch.from_numpy(counts).to(cuda)).cpu().numpy()
    # The CLI's file is the writer's file of the byte image (the writer's
    # bytes are pinned to the reference encoder by the CPU tests).
    api.write_jpeg(str(tmp_path / "w.jpg"), img)
    assert (tmp_path / "c.jpg").read_bytes() == (tmp_path / "w.jpg").read_bytes()
    back = decode(str(tmp_path / "c.jpg"))
    assert back.shape == img.shape
    assert np.mean(np.abs(back.astype(int) - img.astype(int))) < 12


def test_drainage_cli_batch(cuda, tmp_path):
    """--batch K: the same counts as one realization at a time; a batch the
    fill mode does not allow is refused."""
    from cageo_gb300 import _build, api
    dem, streams = make_case(90, 70, seed=25)
    d = _write_inputs(tmp_path, dem, streams)
    base = [_build.DRAINAGE, "--dem-path", str(d), "--seed", "9", "-i", "7"]
    one = subprocess.run(base + ["-o", "one.bin"], cwd=tmp_path, capture_output=True)
    four = subprocess.run(base + ["--batch", "4", "-o", "four.bin"], cwd=tmp_path,
                          capture_output=True)
    assert one.returncode == 0 and four.returncode == 0
    a = api.read_raster(str(tmp_path / "one.bin"), dem.shape)
    b = api.read_raster(str(tmp_path / "four.bin"), dem.shape)
    assert np.array_equal(a, b) and a.max() > 0
    bad = subprocess.run(base + ["--batch", "2", "--fill", "exact"], cwd=tmp_path,
                         capture_output=True, text=True)
    assert bad.returncode != 0 and "CPU-compatible" in bad.stderr


def test_drainage_cli_checkpoint_resume(cuda, tmp_path):
    from cageo_gb300 import _build, api
    dem, streams = make_case(80, 64, seed=24)
    d = _write_inputs(tmp_path, dem, streams)
    base = [_build.DRAINAGE, "--dem-path", str(d), "--seed", "8"]
    full = subprocess.run(base + ["-i", "4", "-o", "full.bin"], cwd=tmp_path, capture_output=True)
    assert full.returncode == 0
    part = subprocess.run(base + ["-i", "2", "--checkpoint", "ck.bin"], cwd=tmp_path,
                          capture_output=True)
    assert part.returncode == 0
    rest = subprocess.run(base + ["-i", "4", "--resume", "ck.bin", "-o", "resumed.bin"],
                          cwd=tmp_path, capture_output=True, text=True)
    assert rest.returncode == 0 and "Resuming at realization 2" in rest.stdout
    a = api.read_raster(str(tmp_path / "full.bin"), dem.shape)
    b = api.read_raster(str(tmp_path / "resumed.bin"), dem.shape)
    assert np.array_equal(a, b)
    # A checkpoint holding more realizations than --iterations is refused; one
    # holding exactly that many still writes the END output.
    over = subprocess.run(base + ["-i", "1", "--resume", "ck.bin", "-o", "over.bin"],
                          cwd=tmp_path, capture_output=True, text=True)
    assert over.returncode != 0 and "more than --iterations" in over.stdout
    assert not (tmp_path / "over.bin").exists()
    same = subprocess.run(base + ["-i", "2", "--resume", "ck.bin", "-o", "same.bin"],
                          cwd=tmp_path, capture_output=True, text=True)
    assert same.returncode == 0
    c = api.read_raster(str(tmp_path / "same.bin"), dem.shape)
    assert c.max() <= 2 and c.sum() > 0
    # Another practical range: the checkpoint belongs to another run.
    other = subprocess.run(base + ["-i", "4", "--practical-range", "80", "--resume", "ck.bin"],
                           cwd=tmp_path, capture_output=True, text=True)
    assert other.returncode != 0 and "practical range" in other.stderr
