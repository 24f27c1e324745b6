"""The JPEG writer (host code) writes the bytes the reference's jpge encoder
writes (src/main.cpp:258-271): against the committed fixtures made from
the reference (tests/golden/jpeg/cases.npz, by tests/golden/make_golden.py),
and, where the reference harness was built here, against jpge itself on
seeded images of many sizes.  A decoder checks that the files read back."""
import os

import numpy as np
import pytest

from jpeg_decode import decode, parse

CASES = os.path.join(os.path.dirname(__file__), "golden", "jpeg", "cases.npz")


def _psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return 99.0 if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


def _ours(tmp_path, img, quality=85):
    from cageo_gb300 import api
    p = tmp_path / "ours.jpg"
    api.write_jpeg(str(p), img, quality)
    return p.read_bytes()


def _golden():
    g = np.load(CASES)
    n = sum(1 for k in g.files if k.startswith("img_"))
    return g, n


def test_fixture_cases_present():
    g, n = _golden()
    assert n == 11 and sum(1 for k in g.files if k.startswith("counts_")) >= 4


@pytest.mark.parametrize("i", range(11))
def test_bytes_equal_reference_fixture(tmp_path, i):
    g, _ = _golden()
    img, want, q = g["img_%d" % i], g["jpg_%d" % i].tobytes(), int(g["quality_%d" % i])
    assert _ours(tmp_path, img, q) == want, str(g["name_%d" % i])


def test_count_images_equal_reference_fixture(tmp_path):
    """The JPEG of the reference's byte image of each fixture count grid."""
    g, _ = _golden()
    for i in range(sum(1 for k in g.files if k.startswith("counts_"))):
        assert _ours(tmp_path, g["bytes_%d" % i]) == g["cjpg_%d" % i].tobytes(), \
            str(g["cname_%d" % i])


def _reference():
    from oracle import Reference
    try:
        return Reference()
    except FileNotFoundError:
        pytest.skip("reference harness not built here (oracle/_ref)")


@pytest.mark.parametrize("seed", range(4))
def test_bytes_equal_jpge(tmp_path, seed):
    """Random sizes (1..300 per side), content and quality against the
    reference's encoder compiled from its sources."""
    R = _reference()
    rng = np.random.default_rng(100 + seed)
    for _ in range(6):
        W, H = (int(v) for v in rng.integers(1, 301, size=2))
        kind = rng.integers(0, 3)
        if kind == 0:
            img = rng.integers(0, 256, (H, W)).astype(np.uint8)
        elif kind == 1:
            y, x = np.mgrid[0:H, 0:W]
            img = (127 + 120 * np.sin(x / rng.uniform(2, 20)) *
                   np.cos(y / rng.uniform(2, 20))).astype(np.uint8)
        else:
            c = np.zeros((H, W), np.float32)
            c[rng.random((H, W)) < rng.uniform(0.02, 0.3)] = rng.integers(1, 100)
            img = R.to_bytes(c) if c.max() > 0 else np.zeros((H, W), np.uint8)
        q = int(rng.choice([0, 1, 25, 49, 50, 85, 99, 100]))
        want = R.jpeg(img, str(tmp_path / "ref.jpg"), q)
        assert _ours(tmp_path, img, q or 85) == want, (W, H, kind, q)


def test_layout_is_the_reference_encoders(tmp_path):
    """Three components (Y 2x2, Cb and Cr 1x1), two quantization tables."""
    img = np.full((20, 30), 77, np.uint8)
    p = tmp_path / "a.jpg"
    p.write_bytes(_ours(tmp_path, img))
    quant, tables, comps, scan, W, H, _ = parse(str(p))
    assert (W, H) == (30, 20)
    assert comps == [(1, 2, 2, 0), (2, 1, 1, 1), (3, 1, 1, 1)]
    assert scan == [(1, 0, 0), (2, 1, 1), (3, 1, 1)]
    assert sorted(quant) == [0, 1] and sorted(tables) == [0x00, 0x01, 0x10, 0x11]


@pytest.mark.parametrize("W,H", [(64, 48), (37, 21), (8, 8), (1, 1), (33, 17)])
def test_jpeg_roundtrip(tmp_path, W, H):
    y, x = np.mgrid[0:H, 0:W]
    img = (127 + 100 * np.sin(x / 7.0) * np.cos(y / 5.0)).astype(np.uint8)
    p = tmp_path / "a.jpg"
    p.write_bytes(_ours(tmp_path, img))
    raw = p.read_bytes()
    assert raw[:2] == b"\xff\xd8" and raw[-2:] == b"\xff\xd9" and b"JFIF" in raw[:20]
    back = decode(str(p))
    assert back.shape == img.shape
    assert _psnr(back, img) > 32


def test_jpeg_counts_like_image(tmp_path):
    from cageo_gb300 import api
    rng = np.random.default_rng(0)
    counts = np.zeros((40, 56), np.float32)
    counts[rng.random(counts.shape) < 0.1] = 20.0   # sparse border lines, like MC counts
    img = np.rint(np.float32(255.0) * ((counts - counts.min()) / counts.max())).astype(np.uint8)
    p = tmp_path / "c.jpg"
    p.write_bytes(_ours(tmp_path, img, 100))
    assert _psnr(decode(str(p)), img) > 25
    with pytest.raises(api.CageoError):
        api.write_jpeg(str(p), img, 0)
