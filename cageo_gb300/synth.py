"""Seeded synthetic inputs in the shapes the drainage benchmarks use.

The reference ships no sample rasters, so every test and benchmark runs on
inputs made here:

* ``fbm_dem``      -- spectral fractional-Brownian-motion terrain (white noise
  -> FFT -> amplitude ~ k^-(H+1) -> inverse FFT), scaled to a relief range;
* ``add_pits``     -- random conical pits of a given depth range;
* ``add_plateaus`` -- constant-elevation discs (flat lakes) covering a share
  of the area;
* ``make_streams`` -- a float32 stream raster (1.0 or a per-component id on
  streams, ``nodata`` elsewhere) from D8 flow accumulation on the
  priority-flood-routed DEM, as the reference reads it
  (``StreamData<float>``, a cell is a stream when ``streams >= 0``).
"""
import ctypes

import numpy as np

from . import _build


def fbm_dem(width, height, hurst=0.8, seed=0, lo=80.0, hi=180.0):
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((height, width))
    spec = np.fft.rfft2(noise)
    ky = np.fft.fftfreq(height)[:, None]
    kx = np.fft.rfftfreq(width)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    spec *= k ** (-(hurst + 1.0))
    spec[0, 0] = 0.0
    z = np.fft.irfft2(spec, s=(height, width))
    z -= z.min()
    z /= max(z.max(), 1e-30)
    return (lo + (hi - lo) * z).astype(np.float32)


def add_pits(dem, count, seed=0, depth=(0.5, 3.0), radius=(1, 4)):
    """Subtract `count` cones (depth U[depth], radius U{radius}) at interior centres."""
    dem = dem.copy()
    H, W = dem.shape
    rng = np.random.default_rng(seed + 7919)
    cy = rng.integers(1, H - 1, count)
    cx = rng.integers(1, W - 1, count)
    dep = rng.uniform(depth[0], depth[1], count).astype(np.float32)
    rad = rng.integers(radius[0], radius[1] + 1, count)
    for y, x, d, r in zip(cy, cx, dep, rad):
        y0, y1, x0, x1 = max(y - r, 0), min(y + r + 1, H), max(x - r, 0), min(x + r + 1, W)
        yy, xx = np.mgrid[y0:y1, x0:x1]
        dist = np.sqrt((yy - y) ** 2 + (xx - x) ** 2)
        cone = np.where(dist <= r, d * (1.0 - dist / (r + 1.0)), 0.0).astype(np.float32)
        dem[y0:y1, x0:x1] -= cone
    return dem


def add_plateaus(dem, share=0.2, seed=0, radius=(50, 400)):
    """Flatten discs (radius U[radius]) to their centre elevation until `share` of the area is flat."""
    dem = dem.copy()
    H, W = dem.shape
    rng = np.random.default_rng(seed + 104729)
    flat = np.zeros((H, W), bool)
    target = share * H * W
    covered = 0  # flat.sum(), kept up to date disc by disc
    guard = 0
    while covered < target and guard < 100000:
        guard += 1
        r = int(rng.integers(radius[0], radius[1] + 1))
        y = int(rng.integers(0, H))
        x = int(rng.integers(0, W))
        y0, y1, x0, x1 = max(y - r, 0), min(y + r + 1, H), max(x - r, 0), min(x + r + 1, W)
        yy, xx = np.mgrid[y0:y1, x0:x1]
        disc = (yy - y) ** 2 + (xx - x) ** 2 <= r * r
        dem[y0:y1, x0:x1][disc] = dem[y, x]
        window = flat[y0:y1, x0:x1]
        covered += int(np.count_nonzero(disc & ~window))
        window |= disc
    return dem


def make_streams(dem, threshold, nodata=-9999.0, ids="ones", return_accum=False):
    """Stream raster from D8 accumulation > threshold; ids = 'ones' or 'components'."""
    lib = _build.load_synth()
    d = np.ascontiguousarray(dem, np.float32)
    H, W = d.shape
    out = np.empty((H, W), np.float32)
    acc = np.empty((H, W), np.int32)
    rc = lib.cageo_synth_streams(
        d.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), W, H, int(threshold),
        1 if ids == "components" else 0, ctypes.c_float(nodata),
        out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
        acc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if rc == 2:
        raise MemoryError("stream synthesis ran out of host memory")
    if rc:
        raise ValueError("grid too small (or too large) for stream synthesis")
    return (out, acc) if return_accum else out


# Named workloads (sizes, generator settings and filter) used by tests and
# bench.py.  Relief and pit counts follow the benchmark descriptions.
WORKLOADS = {
    "plain-512": dict(width=512, height=512, hurst=0.8, seed=0, lo=80.0, hi=180.0, pits=200,
                      threshold=500, model="Gaussian", range_m=60.0, sigma=1.5, cell=10.0,
                      realizations=20),
    "plain-4096": dict(width=4096, height=4096, hurst=0.75, seed=1, lo=0.0, hi=300.0, pits=2000,
                       threshold=2000, model="Gaussian", range_m=60.0, sigma=1.5, cell=10.0,
                       realizations=100),
    "eval-8192": dict(width=8192, height=8192, hurst=0.8, seed=3, lo=0.0, hi=300.0, pits=20000,
                      threshold=2000, model="Gaussian", range_m=60.0, sigma=1.5, cell=10.0,
                      realizations=100),
    # Stress case: 16384^2 with 20 % of the area in flat lake plateaus
    # (constant-elevation discs of radius 50-400 cells), Gaussian 90 m.
    "stress-16384": dict(width=16384, height=16384, hurst=0.8, seed=5, lo=0.0, hi=300.0,
                         pits=80000, threshold=2000, model="Gaussian", range_m=90.0, sigma=1.5,
                         cell=10.0, realizations=1000, plateaus=0.2),
}


# The batched benchmark: a 2048^2 DEM and three uneven tiles (width x height).
BATCH_SHAPES = [(2048, 2048), (257, 1013), (1500, 733), (3001, 401)]


def batched_grids(seed=5, scale=1.0, ids="ones"):
    """(dem, streams) for each batch shape: fBm (Hurst 0.8, 0-300 m), pits, threshold 2000."""
    grids = []
    for k, (w, h) in enumerate(BATCH_SHAPES):
        w, h = max(int(w * scale), 16), max(int(h * scale), 16)
        dem = add_pits(fbm_dem(w, h, 0.8, seed + k, 0.0, 300.0), max(w * h // 2000, 1), seed + k)
        grids.append((dem, make_streams(dem, max(int(2000 * scale * scale), 20), ids=ids)))
    return grids


def workload(name, ids="ones", scale=None):
    """(dem, streams, params) for a named workload; `scale` shrinks width/height."""
    p = dict(WORKLOADS[name])
    if scale:
        p["width"] = max(int(p["width"] * scale), 16)
        p["height"] = max(int(p["height"] * scale), 16)
        p["pits"] = max(int(p["pits"] * scale * scale), 1)
    dem = fbm_dem(p["width"], p["height"], p["hurst"], p["seed"], p["lo"], p["hi"])
    dem = add_pits(dem, p["pits"], p["seed"])
    if p.get("plateaus"):
        dem = add_plateaus(dem, p["plateaus"], p["seed"], radius=(50, 400))
    streams = make_streams(dem, p["threshold"], ids=ids)
    return dem, streams, p
