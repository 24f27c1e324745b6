"""GB300 (sm_103a) Monte Carlo drainage-basin pipeline.

The native library (cageo_gb300/_build/libcageo.so, C ABI in include/cageo.h)
holds every kernel; ``cageo_gb300.api`` binds it, ``cageo_gb300.synth`` makes
seeded synthetic inputs, ``cageo_gb300._build.build()`` compiles it in tree.
"""
from . import _build  # noqa: F401

__all__ = ["api", "synth"]
