"""cageo_pitfill_static -- the pit fill for callers that cannot allocate
device memory (a host application that owns the GPU's memory and forbids
plug-ins to call cudaMalloc, or a loop that must not pay an allocation's
latency) -- gives the same result as cageo_pitfill, called through the C
ABI, on two calls in a row with different grids (the shared static scratch
keeps the previous call's contents, which must not leak into the next).

This file is collected last so that a run stopping at its first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from cases import bits, gaussian_noise, make_case

pytestmark = pytest.mark.gpu


def _burned_dem(api, cuda, W, H, seed):
    import torch
    dem, streams = make_case(W, H, seed=seed)
    field = torch.from_numpy(gaussian_noise(W, H, seed + 1)).to(cuda)
    api.realistic_dem(torch.from_numpy(dem).to(cuda), field)
    api.stream_burn(field, torch.from_numpy(streams).to(cuda))
    return field


def test_static_fill_matches_allocating_fill(cuda):
    import torch
    from cageo_gb300 import api
    lib = api.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for W, H, seed in [(512, 512, 31), (257, 131, 32)]:
        src = _burned_dem(api, cuda, W, H, seed)
        a, b = src.clone(), src.clone()
        fa, fb = torch.empty_like(src), torch.empty_like(src)
        st = lib.cageo_pitfill_static(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(fa.data_ptr()),
                                      W, H, -9999.0, api.FILL_CPU_COMPAT, stream)
        assert st == 0, lib.cageo_last_error_string().decode()
        st = lib.cageo_pitfill(ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(fb.data_ptr()), W, H,
                               -9999.0, api.FILL_CPU_COMPAT, None, 0, stream)
        assert st == 0, lib.cageo_last_error_string().decode()
        torch.cuda.synchronize()
        assert np.array_equal(bits(a.cpu().numpy()), bits(b.cpu().numpy())), "quantized DEM"
        assert np.array_equal(bits(fa.cpu().numpy()), bits(fb.cpu().numpy())), "filled DEM"


def test_static_fill_refuses_grids_beyond_its_scratch(cuda):
    import torch
    from cageo_gb300 import api
    lib = api.lib()
    assert lib.cageo_pitfill_static_max_bytes() == 64 << 20
    dummy = torch.zeros(4, device=cuda)
    st = lib.cageo_pitfill_static(ctypes.c_void_p(dummy.data_ptr()),
                                  ctypes.c_void_p(dummy.data_ptr() + 8), 4096, 4096, -9999.0,
                                  api.FILL_CPU_COMPAT, None)
    assert st == 1
    assert "static scratch" in lib.cageo_last_error_string().decode()
