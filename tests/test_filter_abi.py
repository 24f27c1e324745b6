"""CPU tests of the native library's host-only parts: every symbol of
include/cageo.h is exported, and the FP64 filter builder matches a numpy
construction of the reference's recipe (FFT + SVD,
src/convolution/ConvolutionAlgorithm.cpp:18-172)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _numpy_filter(model, rng_m, cell, r):
    y, x = np.mgrid[-r:r + 1, -r:r + 1]
    if model == 0:
        d = np.sqrt((x * x + y * y).astype(np.float32))
        corr = np.exp(-d / np.float32((np.float32(rng_m) / np.float32(3.0)) / np.float32(cell)))
    else:
        s = np.float32(np.float32(rng_m) / np.float32(1.73205080757)) / np.float32(cell)
        corr = np.exp(-(x * x + y * y) / (float(s) ** 2))
    corr = corr.astype(np.float32).astype(np.float64)
    F = np.sqrt(np.abs(np.fft.fft2(corr)))
    k = np.real(np.fft.ifft2(F))
    k = np.fft.fftshift(k).astype(np.float32)
    if model == 0:
        return k.reshape(-1)
    u, s, _ = np.linalg.svd(k.astype(np.float64))
    return (u[:, 0] * np.sqrt(s[0])).astype(np.float32)


def test_header_symbols_exported():
    from cageo_gb300 import _build
    lib = ctypes.CDLL(_build.LIB)
    with open(os.path.join(ROOT, "include", "cageo.h")) as f:
        decl = f.read()
    names = set(re.findall(r"\b(cageo_[a-z0-9_]+)\s*\(", decl))
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("model,rng_m", [(1, 60.0), (1, 90.0), (1, 30.0), (0, 30.0), (0, 60.0),
                                         (0, 45.0), (0, 75.0), (0, 97.5), (0, 120.0),
                                         (1, 120.0), (1, 42.0)])
def test_filter_matches_numpy(model, rng_m):
    from cageo_gb300 import api
    r = api.filter_radius(rng_m, 10.0)
    assert r == int(np.ceil(np.float32(rng_m / 10.0) * np.float32(2.5)))
    got = api.filter_build(model, rng_m, 10.0, r)
    ref = _numpy_filter(model, rng_m, 10.0, r)
    if model == 1 and np.sign(got.sum()) != np.sign(ref.sum()):
        ref = -ref  # the singular vector's sign is arbitrary and cancels in use
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-7 * np.abs(ref).max())


def test_filter_rejects_bad_arguments():
    from cageo_gb300 import api
    with pytest.raises(api.CageoError):
        api.filter_build(5, 60.0, 10.0, 3)
