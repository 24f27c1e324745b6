"""The CUDA stages reproduce the reference's golden fixtures bit for bit."""
import glob
import os

import numpy as np
import pytest

from cases import bits

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_golden(cuda, path):
    import torch
    from cageo_gb300 import api
    g = np.load(path)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    r, model = int(g["radius"]), int(g["model"])
    conv = api.convolve(t(g["noise"]), model, g["taps"], r)
    assert np.array_equal(bits(conv.cpu().numpy()), bits(g["conv"]))
    api.realistic_dem(t(g["dem"]), conv)
    assert np.array_equal(bits(conv.cpu().numpy()), bits(g["realistic"]))
    st = t(g["streams"])
    api.stream_burn(conv, st)
    assert np.array_equal(bits(conv.cpu().numpy()), bits(g["burned"]))
    filled = api.pitfill(conv)
    assert np.array_equal(bits(conv.cpu().numpy()), bits(g["quantized"]))
    assert np.array_equal(bits(filled.cpu().numpy()), bits(g["filled"]))
    dirs = api.route_d8(filled)
    assert np.array_equal(dirs.cpu().numpy(), g["dirs"])
    labels = api.trace(dirs, st)
    assert np.array_equal(labels.cpu().numpy(), g["labels"])
    mc = torch.zeros_like(filled)
    api.border_accumulate(labels, mc)
    assert np.array_equal(mc.cpu().numpy(), g["border"])
