"""Seeded test cases shared by the parity tests (inputs only; outputs come
from the oracle or the golden fixtures)."""
import numpy as np

from cageo_gb300 import synth


def make_case(W, H, seed=0, pits=None, threshold=None, ids="components", hurst=0.8,
              lo=80.0, hi=180.0, plateaus=0.0, nodata_cells=0):
    dem = synth.fbm_dem(W, H, hurst, seed, lo, hi)
    dem = synth.add_pits(dem, pits if pits is not None else max(W * H // 1300, 1), seed)
    if plateaus:
        dem = synth.add_plateaus(dem, plateaus, seed, radius=(3, max(4, min(W, H) // 6)))
    streams = synth.make_streams(dem, threshold or max(20, W * H // 500), ids=ids)
    if nodata_cells:
        rng = np.random.default_rng(seed + 5)
        idx = rng.choice(W * H, nodata_cells, replace=False)
        dem.reshape(-1)[idx] = -9999.0
    return dem, streams


def gaussian_noise(W, H, seed, sigma=1.5):
    return (np.random.default_rng(seed).standard_normal((H, W)) * sigma).astype(np.float32)


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


def philox_np(ctr, key):
    """Philox4x32-10 (Salmon et al. 2011) restated with numpy uint64 arithmetic."""
    c = [x.astype(np.uint64) for x in ctr]
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    mask = np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + np.uint64(0x9E3779B9)) & mask
        k1 = (k1 + np.uint64(0xBB67AE85)) & mask
    return c
