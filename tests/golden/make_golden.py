"""Generate tests/golden/*.npz from the drainage reference's own CPU stage
code, compiled from the reference sources by `make -C oracle ref` into
oracle/_ref/libref.so (see oracle/ref_harness.cpp).

Each case stores seeded inputs (DEM, stream raster, noise, filter) and the
reference's output of every stage, run in the reference's order.  Filter
taps are built by the library's FP64 builder and noise is seeded numpy
noise; both are injected (the reference builds them with FFTW/Eigen and
thrust RNG, which are not available).  Run from the repository root, with
CAGEO_REFERENCE naming the reference checkout (a directory holding src/):

    CAGEO_REFERENCE=<checkout> python tests/golden/make_golden.py
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


def main():
    build(ref=True)
    R = Reference()
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
