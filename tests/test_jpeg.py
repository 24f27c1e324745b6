"""The JPEG writer (host code) produces a baseline JFIF that decodes back to
its input within quality-85 error."""
import numpy as np
import pytest

from jpeg_decode import decode


def _psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return 99.0 if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


@pytest.mark.parametrize("W,H", [(64, 48), (37, 21), (8, 8)])
def test_jpeg_roundtrip(tmp_path, W, H):
    from cageo_gb300 import api
    y, x = np.mgrid[0:H, 0:W]
    img = (127 + 100 * np.sin(x / 7.0) * np.cos(y / 5.0)).astype(np.uint8)
    p = tmp_path / "a.jpg"
    api.write_jpeg(str(p), img, 85)
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
    api.write_jpeg(str(p), img, 100)
    assert _psnr(decode(str(p)), img) > 25
    with pytest.raises(api.CageoError):
        api.write_jpeg(str(p), img, 0)
