"""Python binding of the C ABI in include/cageo.h (ctypes; no torch types cross it).

Each stage function mirrors one reference stage algorithm's ``execute``
(see include/cageo.h for the reference interface each replaces) on CUDA
tensors: grids are ``torch.float32`` tensors of shape (H, W) on the current
CUDA device, directions ``int8`` (H, W, 2) holding (dx, dy), labels
``int32`` (H, W).  Calls run on torch's current stream.  A non-zero status
raises :class:`CageoError` with the library's message; a missing library
raises ``FileNotFoundError`` -- there is no fallback implementation.
"""
import ctypes
import os

import numpy as np

from . import _build

FILTER_EXPONENTIAL = 0
FILTER_GAUSSIAN = 1
FILL_CPU_COMPAT = 0
FILL_EXACT = 1
ROUTE_CPU_COMPAT = 0
ROUTE_GPU_ORDER = 1
TRACE_CPU_COMPAT = 0
TRACE_DEAD_END_ERROR = 1
OUTSIDE = -9999
LAKE = -9998
ERROR = -9996


class CageoError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("cageo status %d: %s" % (status, message))
        self.status = status


class PipelineConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int),
                ("cell_size", ctypes.c_float), ("filter_model", ctypes.c_int),
                ("practical_range", ctypes.c_float), ("error_mean", ctypes.c_float),
                ("error_stddev", ctypes.c_float), ("bevel_radius", ctypes.c_int),
                ("nodata_dem", ctypes.c_float), ("nodata_stream", ctypes.c_float),
                ("seed", ctypes.c_uint64), ("use_graphs", ctypes.c_int),
                ("fill_mode", ctypes.c_int)]


class Tuning(ctypes.Structure):
    _fields_ = [("fill_rounds", ctypes.c_int), ("fill_warps", ctypes.c_int),
                ("conv_tile", ctypes.c_int)]

    def as_dict(self):
        return {"fill_rounds": self.fill_rounds, "fill_warps": self.fill_warps,
                "conv_tile": self.conv_tile}


# Output tile (columns, rows) of the fused front's separable convolution per
# cageo_tuning.conv_tile value.
CONV_TILES = ((64, 32), (128, 32), (64, 64), (96, 32))


def autotune_candidates():
    n = lib().cageo_autotune_candidates(None, 0)
    arr = (Tuning * n)()
    lib().cageo_autotune_candidates(ctypes.cast(arr, _vp), n)
    return [t.as_dict() for t in arr]


class RasterInfo(ctypes.Structure):
    _fields_ = [("ncols", ctypes.c_int), ("nrows", ctypes.c_int),
                ("xllcorner", ctypes.c_double), ("yllcorner", ctypes.c_double),
                ("cellsize", ctypes.c_float), ("nodata_value", ctypes.c_float),
                ("byteorder_msb", ctypes.c_int)]


_vp, _i, _f, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t
_SIGS = {
    "cageo_version": ([], ctypes.c_char_p),
    "cageo_last_error_string": ([], ctypes.c_char_p),
    "cageo_noise_philox": ([_vp, _i, _i, ctypes.c_uint64, ctypes.c_uint32, _f, _f, _vp], _i),
    "cageo_philox4x32_10": ([_vp, ctypes.c_int64, _vp, _vp, _vp], _i),
    "cageo_filter_radius": ([_f, _f], _i),
    "cageo_filter_build": ([_i, _f, _f, _i, _vp], _i),
    "cageo_convolve": ([_vp, _vp, _i, _i, _i, _vp, _i, _vp], _i),
    "cageo_realistic_dem": ([_vp, _vp, _i, _i, _f, _vp], _i),
    "cageo_stream_burn": ([_vp, _vp, _i, _i, _i, _f, _f, _vp], _i),
    "cageo_pitfill_workspace_size": ([_i, _i], _sz),
    "cageo_pitfill": ([_vp, _vp, _i, _i, _f, _i, _vp, _sz, _vp], _i),
    "cageo_pitfill_exact_warm": ([_vp, _vp, _vp, _i, _i, _f, _vp, _sz, _vp, _vp], _i),
    "cageo_pitfill_static_max_bytes": ([], _sz),
    "cageo_pitfill_static": ([_vp, _vp, _i, _i, _f, _i, _vp], _i),
    "cageo_route_workspace_size": ([_i, _i], _sz),
    "cageo_route_d8": ([_vp, _vp, _vp, _i, _i, _vp, _sz, _vp], _i),
    "cageo_route_d8_mode": ([_vp, _vp, _vp, _i, _i, _f, _i, _vp, _sz, _vp], _i),
    "cageo_trace_workspace_size": ([_i, _i], _sz),
    "cageo_trace": ([_vp, _vp, _vp, _i, _i, _vp, _sz, _vp], _i),
    "cageo_trace_mode": ([_vp, _vp, _vp, _i, _i, _i, _vp, _sz, _vp], _i),
    "cageo_border_accumulate": ([_vp, _vp, _i, _i, _vp], _i),
    "cageo_ws_param_count": ([], _i),
    "cageo_ws_features": ([_vp, _vp, _i, _i, _i, _f, _vp], _i),
    "cageo_ws_forward": ([_vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp], _i),
    "cageo_ws_backward": ([_vp] * 5 + [_i, _i, _i] + [_vp] * 5, _i),
    "cageo_ws_mse": ([_vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp], _i),
    "cageo_ws_adam": ([_vp, _vp, _vp, _vp, _i, _f, _f, _f, _f, _i, _vp], _i),
    "cageo_ws_infer": ([_vp, _vp, _vp, _vp, _i, _i, _f, _f, _vp], _i),
    "cageo_pipeline_create": ([ctypes.POINTER(_vp), ctypes.POINTER(PipelineConfig), _vp, _vp], _i),
    "cageo_pipeline_create_device": ([ctypes.POINTER(_vp), ctypes.POINTER(PipelineConfig), _vp,
                                      _vp], _i),
    "cageo_pipeline_run": ([_vp, ctypes.c_uint32, _i], _i),
    "cageo_pipeline_run_filter": ([_vp, ctypes.c_uint32, _i, _i, _f, _f, _f], _i),
    "cageo_pipeline_set_batch": ([_vp, _i], _i),
    "cageo_pipeline_counts": ([_vp, _vp], _i),
    "cageo_pipeline_counts_device": ([_vp, _vp], _i),
    "cageo_pipeline_last_stages": ([_vp, _vp, _vp, _vp], _i),
    "cageo_pipeline_reset_counts": ([_vp], _i),
    "cageo_pipeline_save": ([_vp, ctypes.c_char_p, ctypes.c_uint32], _i),
    "cageo_pipeline_load": ([_vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint32)], _i),
    "cageo_pipeline_stream": ([_vp], _vp),
    "cageo_pipeline_graph_kernels": ([_vp, _vp], _i),
    "cageo_pipeline_stats": ([_vp, _vp, _i], _i),
    "cageo_pipeline_profile": ([_vp, ctypes.c_uint32, _vp, _i], _i),
    "cageo_pipeline_destroy": ([_vp], None),
    "cageo_pipeline_set_warmstart": ([_vp, _vp, _i, _f], _i),
    "cageo_pipeline_autotune": ([_vp, ctypes.c_uint32, _i, _vp, _vp, _i], _i),
    "cageo_autotune_candidates": ([_vp, _i], _i),
    "cageo_pipeline_set_tuning": ([_vp, _vp], _i),
    "cageo_pipeline_get_tuning": ([_vp, _vp], _i),
    "cageo_pipeline_warmstart_stats": ([_vp, _vp, _i], _i),
    "cageo_to_bytes": ([_vp, _vp, _i, _i, _vp], _i),
    "cageo_write_jpeg": ([ctypes.c_char_p, _vp, _i, _i, _i], _i),
    "cageo_pipeline_counts_bytes": ([_vp, _vp], _i),
    "cageo_read_header": ([ctypes.c_char_p, ctypes.POINTER(RasterInfo)], _i),
    "cageo_write_header": ([ctypes.c_char_p, ctypes.POINTER(RasterInfo)], _i),
    "cageo_read_raster": ([ctypes.c_char_p, _vp, _sz], _i),
    "cageo_write_raster": ([ctypes.c_char_p, _vp, _sz], _i),
}

_lib = None


def lib():
    """The loaded libcageo with typed signatures (raises if it was not built)."""
    global _lib
    if _lib is None:
        L = _build.load()
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        raise CageoError(status, lib().cageo_last_error_string().decode())


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _grid(t, dtype, name):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
        raise TypeError("%s must be a contiguous CUDA %s tensor" % (name, dtype))
    return t


def version():
    return lib().cageo_version().decode()


# ---- A1 ---------------------------------------------------------------------
def noise_philox(field, seed, realization, mean=0.0, stddev=1.0):
    import torch
    _grid(field, torch.float32, "field")
    H, W = field.shape
    _check(lib().cageo_noise_philox(_ptr(field), W, H, seed, realization, mean, stddev, _stream()))
    return field


def philox4x32_10(counter, key, n=1, device=None):
    """Raw Philox4x32-10 words: (n, 4) uint32 numpy array; block i uses the
    counter (counter[0] + i, counter[1], counter[2], counter[3])."""
    import torch
    out = torch.empty(4 * n, dtype=torch.int32, device=device or "cuda")
    c = (ctypes.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in counter])
    k = (ctypes.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    _check(lib().cageo_philox4x32_10(_ptr(out), n, ctypes.cast(c, _vp), ctypes.cast(k, _vp),
                                     _stream()))
    return out.cpu().numpy().view(np.uint32).reshape(n, 4)


# ---- A2 ---------------------------------------------------------------------
def filter_radius(practical_range, cell_size):
    return lib().cageo_filter_radius(practical_range, cell_size)


def filter_build(model, practical_range, cell_size, radius=None):
    if radius is None:
        radius = filter_radius(practical_range, cell_size)
    n = 2 * radius + 1
    out = np.zeros(n if model == FILTER_GAUSSIAN else n * n, np.float32)
    _check(lib().cageo_filter_build(model, practical_range, cell_size, radius,
                                    out.ctypes.data_as(ctypes.c_void_p)))
    return out


# ---- A3..A9 -------------------------------------------------------------------
def convolve(field, model, taps, radius):
    import torch
    _grid(field, torch.float32, "field")
    H, W = field.shape
    t = torch.as_tensor(np.asarray(taps, np.float32)).to(field.device)
    out = torch.empty_like(field)
    _check(lib().cageo_convolve(_ptr(field), _ptr(out), W, H, model, _ptr(t), radius, _stream()))
    return out


def realistic_dem(dem, field, nodata_dem=-9999.0):
    import torch
    _grid(dem, torch.float32, "dem")
    _grid(field, torch.float32, "field")
    H, W = field.shape
    _check(lib().cageo_realistic_dem(_ptr(dem), _ptr(field), W, H, nodata_dem, _stream()))
    return field


def stream_burn(dem, streams, bevel_radius=2, nodata_dem=-9999.0, nodata_stream=-9999.0):
    import torch
    _grid(dem, torch.float32, "dem")
    _grid(streams, torch.float32, "streams")
    H, W = dem.shape
    _check(lib().cageo_stream_burn(_ptr(dem), _ptr(streams), W, H, bevel_radius, nodata_dem,
                                   nodata_stream, _stream()))
    return dem


def pitfill(dem, nodata_dem=-9999.0, workspace=None, mode=FILL_CPU_COMPAT):
    """Returns the filled grid.  CPU_COMPAT quantizes `dem` in place (as the
    reference's CPU path does); EXACT leaves it unchanged."""
    import torch
    _grid(dem, torch.float32, "dem")
    H, W = dem.shape
    filled = torch.empty_like(dem)
    ws, wsb = (None, 0) if workspace is None else (_ptr(workspace), workspace.numel())
    _check(lib().cageo_pitfill(_ptr(dem), _ptr(filled), W, H, nodata_dem, mode, ws, wsb,
                               _stream()))
    return filled


FILL_STATS = ("last_pass", "phases", "passes", "passes_b", "us", "us_b", "us_phases", "tiles",
              "rounds", "tiles_b", "rounds_b", "kcyc_load", "kcyc_sweep", "kcyc_store",
              "kcyc_idle", "kcyc_idle_b", "reset_cells")


def pitfill_exact_warm(dem, warm=None, nodata_dem=-9999.0, workspace=None):
    """Exact fill relaxed down from `warm` (None: +inf), verified and repaired
    by the fill itself (the result is the exact fill for any start).  Returns
    (filled, stats dict)."""
    import torch
    _grid(dem, torch.float32, "dem")
    if warm is not None:
        _grid(warm, torch.float32, "warm")
    H, W = dem.shape
    filled = torch.empty_like(dem)
    ws, wsb = (None, 0) if workspace is None else (_ptr(workspace), workspace.numel())
    st = (ctypes.c_int64 * len(FILL_STATS))()
    _check(lib().cageo_pitfill_exact_warm(_ptr(dem), _ptr(warm) if warm is not None else None,
                                          _ptr(filled), W, H, nodata_dem, ws, wsb,
                                          ctypes.cast(st, _vp), _stream()))
    return filled, dict(zip(FILL_STATS, list(st)))


def route_d8(filled, with_flatdist=False, mode=ROUTE_CPU_COMPAT, nodata_dem=-9999.0):
    import torch
    _grid(filled, torch.float32, "filled")
    H, W = filled.shape
    d = torch.empty((H, W, 2), dtype=torch.int8, device=filled.device)
    fd = torch.empty((H, W), dtype=torch.int32, device=filled.device) if with_flatdist else None
    _check(lib().cageo_route_d8_mode(_ptr(filled), _ptr(d), _ptr(fd) if fd is not None else None,
                                     W, H, nodata_dem, mode, None, 0, _stream()))
    return (d, fd) if with_flatdist else d


def trace(dirs, streams, mode=TRACE_CPU_COMPAT):
    import torch
    _grid(dirs, torch.int8, "dirs")
    _grid(streams, torch.float32, "streams")
    H, W = streams.shape
    lab = torch.empty((H, W), dtype=torch.int32, device=streams.device)
    _check(lib().cageo_trace_mode(_ptr(dirs), _ptr(streams), _ptr(lab), W, H, mode, None, 0,
                                  _stream()))
    return lab


def border_accumulate(labels, counts):
    import torch
    _grid(labels, torch.int32, "labels")
    _grid(counts, torch.float32, "counts")
    H, W = labels.shape
    _check(lib().cageo_border_accumulate(_ptr(labels), _ptr(counts), W, H, _stream()))
    return counts


# ---- learned warm start (no counterpart in the reference) -------------------------
def ws_features(v, nodata_dem=-9999.0):
    """v: (B, H, W) or (H, W) float32 CUDA -> features (B, 4, H, W)."""
    import torch
    _grid(v, torch.float32, "v")
    vb = v if v.dim() == 3 else v[None]
    B, H, W = vb.shape
    f = torch.empty((B, 4, H, W), dtype=torch.float32, device=v.device)
    _check(lib().cageo_ws_features(_ptr(vb), _ptr(f), W, H, B, nodata_dem, _stream()))
    return f


def ws_forward(params, feat):
    """Training forward pass: returns (a1, a2, out) with out (B, H, W)."""
    import torch
    B, _, H, W = feat.shape
    a1 = torch.empty((B, 32, H, W), dtype=torch.float32, device=feat.device)
    a2 = torch.empty_like(a1)
    out = torch.empty((B, H, W), dtype=torch.float32, device=feat.device)
    _check(lib().cageo_ws_forward(_ptr(params), _ptr(feat), W, H, B, _ptr(a1), _ptr(a2),
                                  _ptr(out), _stream()))
    return a1, a2, out


def ws_backward(params, feat, a1, a2, dout, grad, tmp1=None, tmp2=None, wflip=None):
    """Adds dL/dparams (given dL/dout) into `grad`."""
    import torch
    B, _, H, W = feat.shape
    tmp1 = torch.empty_like(a1) if tmp1 is None else tmp1
    tmp2 = torch.empty_like(a1) if tmp2 is None else tmp2
    wflip = torch.empty(9216, dtype=torch.float32, device=feat.device) if wflip is None else wflip
    _check(lib().cageo_ws_backward(_ptr(params), _ptr(feat), _ptr(a1), _ptr(a2), _ptr(dout), W, H,
                                   B, _ptr(grad), _ptr(tmp1), _ptr(tmp2), _ptr(wflip), _stream()))
    return grad


def ws_mse(y, target, dy, loss, margin=3):
    B, H, W = y.shape
    _check(lib().cageo_ws_mse(_ptr(y), _ptr(target), _ptr(dy), _ptr(loss), W, H, B, margin,
                              _stream()))


def ws_adam(params, grad, m, v, lr, step, beta1=0.9, beta2=0.999, eps=1e-8):
    _check(lib().cageo_ws_adam(_ptr(params), _ptr(grad), _ptr(m), _ptr(v), params.numel(), lr,
                               beta1, beta2, eps, step, _stream()))


def ws_infer(params, v, threshold=0.0, nodata_dem=-9999.0, want_warm=True, want_depth=False):
    """Fused inference on one grid: returns (warm or None, depth or None)."""
    import torch
    _grid(v, torch.float32, "v")
    H, W = v.shape
    warm = torch.empty_like(v) if want_warm else None
    depth = torch.empty_like(v) if want_depth else None
    _check(lib().cageo_ws_infer(_ptr(params), _ptr(v), _ptr(warm) if warm is not None else None,
                                _ptr(depth) if depth is not None else None, W, H, nodata_dem,
                                threshold, _stream()))
    return warm, depth


# ---- pipeline -------------------------------------------------------------------
class Pipeline:
    """The Monte Carlo loop (src/main.cpp:180-283) on device-resident grids.

    ``dem`` and ``streams`` are float32 (H, W) numpy arrays (host) or CUDA
    tensors (device).  ``run(first, count)`` accumulates border counts of
    realizations first..first+count-1; ``counts()`` returns them as float32.
    """

    def __init__(self, dem, streams, cell_size=10.0, filter_model=FILTER_GAUSSIAN,
                 practical_range=60.0, error_mean=0.0, error_stddev=1.0, bevel_radius=2,
                 nodata_dem=-9999.0, nodata_stream=-9999.0, seed=0, use_graphs=True,
                 fill_mode=FILL_CPU_COMPAT):
        H, W = dem.shape
        self.shape = (H, W)
        cfg = PipelineConfig(W, H, cell_size, filter_model, practical_range, error_mean,
                             error_stddev, bevel_radius, nodata_dem, nodata_stream, seed,
                             1 if use_graphs else 0, fill_mode)
        self._p = ctypes.c_void_p()
        if isinstance(dem, np.ndarray):
            d = np.ascontiguousarray(dem, np.float32)
            s = np.ascontiguousarray(streams, np.float32)
            _check(lib().cageo_pipeline_create(ctypes.byref(self._p), ctypes.byref(cfg),
                                               d.ctypes.data_as(_vp), s.ctypes.data_as(_vp)))
        else:
            _check(lib().cageo_pipeline_create_device(ctypes.byref(self._p), ctypes.byref(cfg),
                                                      _ptr(dem.contiguous()),
                                                      _ptr(streams.contiguous())))

    def run(self, first, count):
        _check(lib().cageo_pipeline_run(self._p, first, count))

    def set_batch(self, batch):
        """Realizations per batched step (1: one at a time); see
        cageo_pipeline_set_batch."""
        _check(lib().cageo_pipeline_set_batch(self._p, int(batch)))

    def run_filter(self, first, count, filter_model, practical_range, error_mean, error_stddev):
        """Run with this filter and error model (kept for later runs)."""
        _check(lib().cageo_pipeline_run_filter(self._p, first, count, filter_model,
                                               practical_range, error_mean, error_stddev))

    def counts(self, out=None):
        """Float counts: a new host numpy array, or into `out` (a CUDA tensor, or a
        contiguous host float32 torch tensor, e.g. pinned)."""
        if out is not None:
            if out.is_cuda:
                _check(lib().cageo_pipeline_counts_device(self._p, _ptr(out)))
            else:
                _check(lib().cageo_pipeline_counts(self._p, _ptr(out)))
            return out
        h = np.empty(self.shape, np.float32)
        _check(lib().cageo_pipeline_counts(self._p, h.ctypes.data_as(_vp)))
        return h

    def last_stages(self):
        H, W = self.shape
        f = np.empty((H, W), np.float32)
        d = np.empty((H, W, 2), np.int8)
        lab = np.empty((H, W), np.int32)
        _check(lib().cageo_pipeline_last_stages(self._p, f.ctypes.data_as(_vp),
                                                d.ctypes.data_as(_vp), lab.ctypes.data_as(_vp)))
        return f, d, lab

    def save(self, path, next_realization):
        _check(lib().cageo_pipeline_save(self._p, os.fsencode(path), next_realization))

    def load(self, path):
        """Restore counts from a checkpoint; returns the next realization number."""
        nxt = ctypes.c_uint32()
        _check(lib().cageo_pipeline_load(self._p, os.fsencode(path), ctypes.byref(nxt)))
        return nxt.value

    def reset_counts(self):
        _check(lib().cageo_pipeline_reset_counts(self._p))

    def stats(self):
        s = np.zeros(25, np.int64)
        _check(lib().cageo_pipeline_stats(self._p, s.ctypes.data_as(_vp), 25))
        keys = ("fill_passes", "fill_phases", "flat_layers", "trace_jumps", "burn_reruns",
                "flood_a_passes", "flood_b_passes", "flood_a_us", "flood_b_us", "phases_us",
                "flood_a_tiles", "flood_a_rounds", "flood_b_tiles", "flood_b_rounds",
                "flat_cells", "flat_bfs_us", "tile_kcycles_load", "tile_kcycles_sweep",
                "tile_kcycles_store", "flat_tiles", "flat_kcycles_load", "flat_kcycles_bfs",
                "flat_kcycles_store", "flood_a_kcycles_idle", "flood_b_kcycles_idle")
        return {k: int(v) for k, v in zip(keys, s)}

    STAGES = ("noise", "front", "fill", "route", "trace", "border")

    def autotune(self, first, trials=3):
        """Pick the tuning (the fill's sweep rounds per tile visit and warps
        per SM of its lower-bound flood, then the front's convolution tile)
        by timing every candidate; resets the counts.  Returns (chosen
        tuning, [(candidate, ms per realization)]); a convolution tile that
        does not apply has 0 ms."""
        cands = autotune_candidates()
        best = Tuning()
        ms = np.zeros(len(cands), np.float32)
        _check(lib().cageo_pipeline_autotune(self._p, first, trials, ctypes.byref(best),
                                             ms.ctypes.data_as(_vp), len(cands)))
        return best.as_dict(), [(c, float(v)) for c, v in zip(cands, ms)]

    def set_tuning(self, fill_rounds, fill_warps, conv_tile=None):
        """Set the tuning; conv_tile None keeps the current tile."""
        if conv_tile is None:
            conv_tile = self.tuning()["conv_tile"]
        _check(lib().cageo_pipeline_set_tuning(
            self._p, ctypes.byref(Tuning(fill_rounds, fill_warps, conv_tile))))

    def tuning(self):
        t = Tuning()
        _check(lib().cageo_pipeline_get_tuning(self._p, ctypes.byref(t)))
        return t.as_dict()

    def set_warmstart(self, params, threshold):
        """Learned warm start (exact mode); params None switches it off."""
        if params is None:
            _check(lib().cageo_pipeline_set_warmstart(self._p, None, 0, 0.0))
            return
        a = np.ascontiguousarray(params, np.float32)
        _check(lib().cageo_pipeline_set_warmstart(self._p, a.ctypes.data_as(_vp), a.size,
                                                  threshold))

    def warmstart_stats(self):
        s = np.zeros(9, np.int64)
        _check(lib().cageo_pipeline_warmstart_stats(self._p, s.ctypes.data_as(_vp), 9))
        keys = ("realizations", "repaired", "reset_cells", "warm_tiles", "warm_rounds",
                "repair_rounds", "warm_fill_us", "repair_fill_us", "repair_tiles")
        return {k: int(v) for k, v in zip(keys, s)}

    FILL_PARTS = ("fill_setup", "flood_a", "flood_b", "phases", "fill_final")

    def profile(self, realization, fill_parts=False):
        """Run one realization with per-stage CUDA event timing; returns
        {stage: ms} (with fill_parts, also the pit fill's parts)."""
        ms = np.zeros(11, np.float32)
        _check(lib().cageo_pipeline_profile(self._p, realization, ms.ctypes.data_as(_vp), 11))
        out = dict(zip(self.STAGES, (float(v) for v in ms[:6])))
        if fill_parts:
            out.update(zip(self.FILL_PARTS, (float(v) for v in ms[6:])))
        return out

    def graph_kernels(self):
        """Kernel launches in the captured per-realization CUDA graph."""
        n = ctypes.c_int64()
        _check(lib().cageo_pipeline_graph_kernels(self._p, ctypes.byref(n)))
        return n.value

    @property
    def stream(self):
        return lib().cageo_pipeline_stream(self._p)

    def close(self):
        if self._p:
            lib().cageo_pipeline_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def to_bytes(counts):
    """uint8 image rintf(255*((v-min)/max)) of a float CUDA grid (the reference's JPEG bytes)."""
    import torch
    _grid(counts, torch.float32, "counts")
    H, W = counts.shape
    out = torch.empty((H, W), dtype=torch.uint8, device=counts.device)
    _check(lib().cageo_to_bytes(_ptr(counts), _ptr(out), W, H, _stream()))
    return out


def write_jpeg(path, gray, quality=85):
    g = np.ascontiguousarray(gray, np.uint8)
    H, W = g.shape
    _check(lib().cageo_write_jpeg(os.fsencode(path), g.ctypes.data_as(_vp), W, H, quality))


# ---- A10 --------------------------------------------------------------------------
def read_header(path):
    info = RasterInfo()
    _check(lib().cageo_read_header(os.fsencode(path), ctypes.byref(info)))
    return info


def write_header(path, ncols, nrows, cellsize, nodata, xll=0.0, yll=0.0):
    info = RasterInfo(ncols, nrows, xll, yll, cellsize, nodata, 0)
    _check(lib().cageo_write_header(os.fsencode(path), ctypes.byref(info)))


def read_raster(path, shape):
    out = np.empty(shape, np.float32)
    _check(lib().cageo_read_raster(os.fsencode(path), out.ctypes.data_as(_vp), out.size))
    return out


def write_raster(path, data):
    d = np.ascontiguousarray(data, np.float32)
    _check(lib().cageo_write_raster(os.fsencode(path), d.ctypes.data_as(_vp), d.size))
