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


def _fill_both(lib, api, cuda, src, mode, stream):
    """(static result, allocating result), each as (dem after the call, filled)."""
    import torch
    H, W = src.shape
    a, b = src.clone(), src.clone()
    fa, fb = torch.empty_like(src), torch.empty_like(src)
    st = lib.cageo_pitfill_static(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(fa.data_ptr()),
                                  W, H, -9999.0, mode, stream)
    assert st == 0, lib.cageo_last_error_string().decode()
    st = lib.cageo_pitfill(ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(fb.data_ptr()), W, H,
                           -9999.0, mode, None, 0, stream)
    assert st == 0, lib.cageo_last_error_string().decode()
    torch.cuda.synchronize()
    return (a.cpu().numpy(), fa.cpu().numpy()), (b.cpu().numpy(), fb.cpu().numpy())


@pytest.mark.parametrize("modes", [("compat", "compat"), ("compat", "exact"), ("exact", "compat")])
def test_static_fill_matches_allocating_fill(cuda, modes):
    """Two calls in a row on different grids, in either fill mode: the
    second runs on the scratch the first left behind."""
    import torch
    from cageo_gb300 import api
    lib = api.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    code = {"compat": api.FILL_CPU_COMPAT, "exact": api.FILL_EXACT}
    for (W, H, seed), mode in zip([(512, 512, 31), (257, 131, 32)], modes):
        src = _burned_dem(api, cuda, W, H, seed)
        (qa, fa), (qb, fb) = _fill_both(lib, api, cuda, src, code[mode], stream)
        assert np.array_equal(bits(qa), bits(qb)), "DEM after the fill (%s)" % mode
        assert np.array_equal(bits(fa), bits(fb)), "filled DEM (%s)" % mode


def test_static_fill_allocates_no_device_memory(cuda):
    """After its first call on a device (which looks up the scratch
    array's address), a call changes the device's free memory by nothing."""
    import torch
    from cageo_gb300 import api
    lib = api.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    src = _burned_dem(api, cuda, 384, 320, 41)
    dem, filled = src.clone(), torch.empty_like(src)
    args = (ctypes.c_void_p(dem.data_ptr()), ctypes.c_void_p(filled.data_ptr()), 384, 320,
            -9999.0, api.FILL_CPU_COMPAT, stream)
    assert lib.cageo_pitfill_static(*args) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for mode in (api.FILL_CPU_COMPAT, api.FILL_EXACT):
        dem.copy_(src)
        assert lib.cageo_pitfill_static(*args[:5], mode, stream) == 0, \
            lib.cageo_last_error_string().decode()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0


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
