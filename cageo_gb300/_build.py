"""In-tree build of the native libraries (no setup.py, no cmake).

* ``libcageo.so``       -- the CUDA kernels and the C ABI (include/cageo.h),
  nvcc for sm_103a only;
* ``libcageo_synth.so`` -- host helper for synthetic inputs (g++);
* ``drainage``          -- the command-line driver (g++, links libcageo).

Outputs go to ``cageo_gb300/_build/``.  Loading a library that is missing
raises; nothing falls back to another implementation.
"""
import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["common.cu", "noise_conv.cu", "surface.cu", "pitfill.cu", "routing.cu",
              "trace_border.cu", "pipeline.cu", "pitfill_static.cu", "learned.cu"]
HOST_SOURCES = ["filter.cpp", "raster_io.cpp", "jpeg.cpp"]

LIB = os.path.join(OUT, "libcageo.so")
SYNTH = os.path.join(OUT, "libcageo_synth.so")
DRAINAGE = os.path.join(OUT, "drainage")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(verbose=False, extra_nvcc=()):
    os.makedirs(OUT, exist_ok=True)
    objs, jobs = [], []
    for src in CU_SOURCES:
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I", INCLUDE, "-I", CSRC, "-rdc=false", "-c", os.path.join(CSRC, src),
                     "-o", o, *(["-Xptxas", "-v"] if verbose else []), *extra_nvcc])
    for src in HOST_SOURCES:
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        jobs.append(["g++", "-O3", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE,
                     "-I", os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, src),
                     "-o", o])
    jobs.append(["g++", "-O3", "-fPIC", "-shared", "-std=c++17", "-o", SYNTH,
                 os.path.join(CSRC, "synth.cpp")])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        results = list(ex.map(_run, jobs))
    if verbose:
        for r in results:
            if r.stderr:
                print(r.stderr)
    _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, "-I", os.path.join(CUDA_HOME, "include"),
          "-o", DRAINAGE, os.path.join(CSRC, "drainage_main.cpp"), "-L", OUT, "-lcageo",
          "-Wl,-rpath,$ORIGIN", "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart",
          "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")])
    return LIB


_synth = None
_lib = None


def load_synth():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH):
            raise FileNotFoundError("%s missing: run cageo_gb300._build.build()" % SYNTH)
        _synth = ctypes.CDLL(SYNTH)
    return _synth


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FileNotFoundError("%s missing: run cageo_gb300._build.build()" % LIB)
        _lib = ctypes.CDLL(LIB)
    return _lib
