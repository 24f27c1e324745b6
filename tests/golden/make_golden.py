"""Generate tests/golden/*.npz from the drainage reference's own CPU stage
code, compiled from the reference sources by `make -C oracle ref` into
oracle/_ref/libref.so (see oracle/ref_harness.cpp).

Each case stores seeded inputs (DEM, stream raster, noise, filter) and the
reference's output of every stage, run in the reference's order.
`jpeg/cases.npz` holds the JPEG output path: count grids with the
reference's byte images of them (ToByteArrayAlgorithm on the CPU), and byte
images with the files the reference's jpge encoder writes for them
(default parameters, one channel; a few other qualities).  Filter
taps are built by the library's FP64 builder and noise is seeded numpy
noise; both are injected (the reference builds them with FFTW/Eigen and
thrust RNG, which are not available).  Run from the repository root, with
CAGEO_REFERENCE naming the reference checkout (a directory holding src/):

    CAGEO_REFERENCE=<checkout> python tests/golden/make_golden.py [--jpeg-only]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

from oracle import Reference, build  # noqa: E402
from cageo_gb300 import api  # noqa: E402
from cases import make_case, gaussian_noise  # noqa: E402

CASES = [
    # name, W, H, seed, model, range_m, sigma, extra make_case kwargs, dem offset, nodata cells
    ("gauss_96x80", 96, 80, 11, 1, 60.0, 1.5, {}, 0.0, 0),
    ("expo_131x257", 131, 257, 12, 0, 30.0, 2.0, {}, 0.0, 0),
    ("plateau_120x90", 120, 90, 13, 1, 60.0, 0.5, {"plateaus": 0.3}, 0.0, 0),
    ("nodata_64x48", 64, 48, 14, 1, 40.0, 1.0, {"ids": "ones"}, 0.0, 25),
]


def jpeg_images():
    """(name, image, quality) cases: sizes below, at and across the 16x16
    coding unit, smooth, noisy, count-like and extreme content."""
    rng = np.random.default_rng(31)
    out = []
    for W, H in [(1, 1), (7, 5), (16, 16), (17, 33), (64, 48)]:
        y, x = np.mgrid[0:H, 0:W]
        out.append(("sine_%dx%d" % (W, H),
                    (127 + 100 * np.sin(x / 7.0) * np.cos(y / 5.0)).astype(np.uint8), 0))
    out.append(("noise_33x19", rng.integers(0, 256, (19, 33)).astype(np.uint8), 0))
    y, x = np.mgrid[0:40, 0:48]
    out.append(("checker_48x40", (((x + y) & 1) * 255).astype(np.uint8), 0))
    # Rows 0-3 of each block white, rows 4-7 black: the largest operand the
    # transform can see (32640).
    out.append(("bands_24x24", np.where((np.mgrid[0:24, 0:24][0] % 8) < 4, 255, 0)
                .astype(np.uint8), 0))
    y, x = np.mgrid[0:48, 0:64]
    sine = (127 + 100 * np.sin(x / 7.0) * np.cos(y / 5.0)).astype(np.uint8)
    for q in (10, 50, 100):
        out.append(("sine_64x48_q%d" % q, sine, q))
    return out


def count_grids():
    """(name, counts) cases for the byte image, rounding ties included."""
    rng = np.random.default_rng(32)
    c1 = rng.integers(0, 37, size=(50, 70)).astype(np.float32)
    c2 = rng.integers(5, 41, size=(30, 20)).astype(np.float32)   # min above 0
    c3 = np.tile(np.arange(11, dtype=np.float32), (3, 1))        # 25.5, 76.5, ... ties
    c4 = np.zeros((40, 56), np.float32)
    c4[rng.random(c4.shape) < 0.1] = 20.0                        # sparse border lines
    return [("ints_70x50", c1), ("offset_20x30", c2), ("ties_11x3", c3), ("sparse_56x40", c4)]


def make_jpeg(R):
    import tempfile
    arrays = {}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "x.jpg")
        for i, (name, img, q) in enumerate(jpeg_images()):
            data = R.jpeg(img, path, q)
            arrays["img_%d" % i] = img
            arrays["jpg_%d" % i] = np.frombuffer(data, np.uint8)
            arrays["quality_%d" % i] = np.int32(q or 85)
            arrays["name_%d" % i] = np.array(name)
        for i, (name, c) in enumerate(count_grids()):
            b = R.to_bytes(c)
            arrays["counts_%d" % i] = c
            arrays["bytes_%d" % i] = b
            arrays["cjpg_%d" % i] = np.frombuffer(R.jpeg(b, path), np.uint8)
            arrays["cname_%d" % i] = np.array(name)
    os.makedirs(os.path.join(HERE, "jpeg"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "jpeg", "cases.npz"), **arrays)
    print("jpeg/cases.npz written")


def main():
    build(ref=True)
    R = Reference()
    make_jpeg(R)
    if "--jpeg-only" in sys.argv[1:]:
        return
    for name, W, H, seed, model, rng_m, sigma, kw, offset, nodata in CASES:
        dem, streams = make_case(W, H, seed=seed, nodata_cells=nodata, **kw)
        dem = dem + np.float32(offset)
        r = api.filter_radius(rng_m, 10.0)
        taps = api.filter_build(model, rng_m, 10.0, r)
        noise = gaussian_noise(W, H, seed + 100, sigma)
        conv = R.convolve(noise, taps, r, model)
        real = R.realistic_dem(dem, conv)
        burned = R.stream_burn(real, streams)
        q, filled = R.pitfill(burned)
        dirs = R.flow_route(filled)
        labels = R.flow_trace(dirs, streams)
        mc = R.border_accumulate(labels, np.zeros((H, W), np.float32))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), dem=dem, streams=streams,
                            noise=noise, taps=taps, radius=r, model=model, conv=conv,
                            realistic=real, burned=burned, quantized=q, filled=filled,
                            dirs=dirs, labels=labels, border=mc)
        print(name, "written")


if __name__ == "__main__":
    main()
