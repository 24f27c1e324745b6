"""ctypes front end of the test oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg, never by the ``cageo_gb300`` package.

``Oracle`` wraps ``_build/liboracle.so`` (the CPU restatement in
``cageo_oracle.cpp``).  ``Reference`` wraps ``_ref/libref.so`` (the drainage
reference's own CPU stage templates compiled from its sources by
``make ref``), which exists only where those sources were available.
Both expose the same numpy-level functions, so a test can run either.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int)
_i8p = ctypes.POINTER(ctypes.c_int8)


def _p(a, t):
    return a.ctypes.data_as(t)


REFERENCE_ENV = "CAGEO_REFERENCE"


def reference_checkout():
    """The reference checkout named by $CAGEO_REFERENCE (a directory holding
    src/), or None when it is unset or does not hold the sources."""
    ref = os.environ.get(REFERENCE_ENV, "")
    return ref if ref and os.path.isdir(os.path.join(ref, "src")) else None


def build(ref=False):
    """Compile the restatement (and, with ref=True, the reference harness
    from the checkout named by $CAGEO_REFERENCE)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        src = reference_checkout()
        if src is None:
            raise RuntimeError("set %s to a reference checkout (a directory holding src/)"
                               % REFERENCE_ENV)
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + src], check=True)


class _Base:
    prefix = ""
    path = ""

    def __init__(self):
        if not os.path.exists(self.path):
            raise FileNotFoundError(self.path)
        self.lib = ctypes.CDLL(self.path)

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # Each method mirrors one reference stage; arrays are C-contiguous numpy.
    def realistic_dem(self, dem, field, nodata_dem=-9999.0):
        f = np.ascontiguousarray(field, np.float32).copy()
        d = np.ascontiguousarray(dem, np.float32)
        H, W = d.shape
        if self.prefix == "orc_":
            self._fn("realistic_dem")(_p(d, _f32p), _p(f, _f32p), ctypes.c_int64(W * H),
                                      ctypes.c_float(nodata_dem))
        else:
            self._fn("realistic_dem")(_p(d, _f32p), _p(f, _f32p), W, H, ctypes.c_float(nodata_dem))
        return f

    def stream_burn(self, rdem, streams, bevel=2, nodata_dem=-9999.0, nodata_stream=-9999.0):
        d = np.ascontiguousarray(rdem, np.float32).copy()
        s = np.ascontiguousarray(streams, np.float32)
        H, W = d.shape
        self._fn("stream_burn")(_p(d, _f32p), _p(s, _f32p), W, H, bevel,
                                ctypes.c_float(nodata_dem), ctypes.c_float(nodata_stream))
        return d

    def pitfill(self, rdem, nodata=-9999.0):
        """Returns (quantized dem, filled)."""
        d = np.ascontiguousarray(rdem, np.float32).copy()
        H, W = d.shape
        f = np.empty_like(d)
        self._fn("pitfill")(_p(d, _f32p), _p(f, _f32p), W, H, ctypes.c_float(nodata))
        return d, f

    def flow_route(self, filled):
        """Returns dir as int8 (H, W, 2) holding (dx, dy)."""
        d = np.ascontiguousarray(filled, np.float32)
        H, W = d.shape
        dirs = np.zeros((H, W, 2), np.int8)
        fd = np.zeros((H, W), np.int32)
        self._fn("flow_route")(_p(d, _f32p), _p(dirs, _i8p), _p(fd, _i32p), W, H)
        return dirs

    def flow_trace(self, dirs, streams):
        dd = np.ascontiguousarray(dirs, np.int8)
        s = np.ascontiguousarray(streams, np.float32)
        H, W = s.shape
        lab = np.zeros((H, W), np.int32)
        self._fn("flow_trace")(_p(dd, _i8p), _p(s, _f32p), _p(lab, _i32p), W, H)
        return lab

    def border_accumulate(self, label, mc):
        lab = np.ascontiguousarray(label, np.int32)
        m = np.ascontiguousarray(mc, np.float32).copy()
        H, W = lab.shape
        self._fn("border_accumulate")(_p(lab, _i32p), _p(m, _f32p), W, H)
        return m


class Oracle(_Base):
    prefix = "orc_"
    path = os.path.join(HERE, "_build", "liboracle.so")

    def convolve(self, field, filt, r, model):
        """model 1 = Gaussian (2r+1 taps), 0 = exponential ((2r+1)^2)."""
        x = np.ascontiguousarray(field, np.float32)
        H, W = x.shape
        out = np.empty_like(x)
        fl = np.ascontiguousarray(filt, np.float32)
        fn = self._fn("convolve_separable" if model == 1 else "convolve_2d")
        rc = fn(_p(x, _f32p), _p(out, _f32p), W, H, _p(fl, _f32p), r)
        if rc:
            raise ValueError("convolution rejected its arguments")
        return out

    def realization(self, dem, streams, noise, filt, r, model, mc, bevel=2,
                    nodata_dem=-9999.0, nodata_stream=-9999.0):
        """One full realization with injected noise; returns (mc, filled, dirs, labels)."""
        d = np.ascontiguousarray(dem, np.float32)
        s = np.ascontiguousarray(streams, np.float32)
        f = np.ascontiguousarray(noise, np.float32).copy()
        H, W = d.shape
        m = np.ascontiguousarray(mc, np.float32).copy()
        fl = np.ascontiguousarray(filt, np.float32)
        filled = np.empty((H, W), np.float32)
        dirs = np.empty((H, W, 2), np.int8)
        lab = np.empty((H, W), np.int32)
        rc = self._fn("realization")(_p(d, _f32p), _p(s, _f32p), _p(f, _f32p), W, H, model,
                                     _p(fl, _f32p), r, bevel, ctypes.c_float(nodata_dem),
                                     ctypes.c_float(nodata_stream), _p(m, _f32p),
                                     _p(filled, _f32p), _p(dirs, _i8p), _p(lab, _i32p))
        if rc:
            raise ValueError("realization rejected its arguments")
        return m, filled, dirs, lab

    def trace_path_stats(self, dirs, streams):
        """(longest terminating path in moves, cells whose path never terminates)."""
        dd = np.ascontiguousarray(dirs, np.int8)
        s = np.ascontiguousarray(streams, np.float32)
        H, W = s.shape
        out = np.zeros(2, np.int64)
        self.lib.orc_trace_path_stats(_p(dd, _i8p), _p(s, _f32p), W, H,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        return int(out[0]), int(out[1])

    def threads(self):
        return self.lib.orc_num_threads()

    # ---- the reference's GPU path semantics (exact mode) ----
    def pitfill_exact(self, rdem, nodata=-9999.0):
        d = np.ascontiguousarray(rdem, np.float32)
        H, W = d.shape
        f = np.empty_like(d)
        self.lib.orc_pitfill_exact(_p(d, _f32p), _p(f, _f32p), W, H, ctypes.c_float(nodata))
        return f

    def flow_route_gpu(self, filled, nodata=-9999.0, with_flatdist=False):
        d = np.ascontiguousarray(filled, np.float32)
        H, W = d.shape
        dirs = np.zeros((H, W, 2), np.int8)
        fd = np.zeros((H, W), np.int32)
        self.lib.orc_flow_route_gpu(_p(d, _f32p), _p(dirs, _i8p), _p(fd, _i32p), W, H,
                                    ctypes.c_float(nodata))
        return (dirs, fd) if with_flatdist else dirs

    def flow_trace_gpu(self, dirs, streams):
        dd = np.ascontiguousarray(dirs, np.int8)
        s = np.ascontiguousarray(streams, np.float32)
        H, W = s.shape
        lab = np.zeros((H, W), np.int32)
        self.lib.orc_flow_trace_gpu(_p(dd, _i8p), _p(s, _f32p), _p(lab, _i32p), W, H)
        return lab

    def realization_exact(self, dem, streams, noise, filt, r, model, mc, bevel=2,
                          nodata_dem=-9999.0, nodata_stream=-9999.0):
        """Exact-mode realization (GPU path semantics); returns (mc, filled, dirs, labels)."""
        d = np.ascontiguousarray(dem, np.float32)
        s = np.ascontiguousarray(streams, np.float32)
        f = np.ascontiguousarray(noise, np.float32).copy()
        H, W = d.shape
        m = np.ascontiguousarray(mc, np.float32).copy()
        fl = np.ascontiguousarray(filt, np.float32)
        filled = np.empty((H, W), np.float32)
        dirs = np.empty((H, W, 2), np.int8)
        lab = np.empty((H, W), np.int32)
        rc = self.lib.orc_realization_exact(_p(d, _f32p), _p(s, _f32p), _p(f, _f32p), W, H, model,
                                            _p(fl, _f32p), r, bevel, ctypes.c_float(nodata_dem),
                                            ctypes.c_float(nodata_stream), _p(m, _f32p),
                                            _p(filled, _f32p), _p(dirs, _i8p), _p(lab, _i32p))
        if rc:
            raise ValueError("realization rejected its arguments")
        return m, filled, dirs, lab


class Reference(_Base):
    prefix = "ref_"
    path = os.path.join(HERE, "_ref", "libref.so")

    def to_bytes(self, mc):
        """The driver's JPEG byte image of a count grid (reference CPU code)."""
        m = np.ascontiguousarray(mc, np.float32)
        H, W = m.shape
        out = np.empty((H, W), np.uint8)
        self.lib.ref_to_bytes(_p(m, _f32p), out.ctypes.data_as(ctypes.c_void_p), W, H)
        return out

    def jpeg(self, img, path, quality=0):
        """The reference's JPEG file of a byte image (the jpge encoder with
        its default parameters, one channel; quality 0 keeps the default
        85); returns the file's bytes."""
        g = np.ascontiguousarray(img, np.uint8)
        H, W = g.shape
        if self.lib.ref_write_jpeg(os.fsencode(path), g.ctypes.data_as(ctypes.c_void_p), W, H,
                                   quality):
            raise IOError("jpge could not write " + str(path))
        with open(path, "rb") as f:
            return f.read()

    def convolve(self, field, filt, r, model):
        x = np.ascontiguousarray(field, np.float32)
        H, W = x.shape
        out = np.empty_like(x)
        fl = np.ascontiguousarray(filt, np.float32)
        self._fn("convolve")(_p(x, _f32p), _p(out, _f32p), W, H, _p(fl, _f32p), r, model)
        return out
