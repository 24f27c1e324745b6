"""The drainage command line's refusals, all taken before any device work
(option parsing, output names, filter type, bevel radius, the two headers;
src/main.cpp:321-442 and :60-110 for the reference's messages), so they
run without a GPU."""
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture()
def inputs(tmp_path):
    from cageo_gb300 import api
    d = tmp_path / "DEM"
    d.mkdir()
    for name in ("dem10", "streams"):
        api.write_header(str(d / (name + ".hdr")), 8, 6, 10.0, -9999.0)
        api.write_raster(str(d / (name + ".bin")), np.ones((6, 8), np.float32))
    return d


def _run(args, cwd):
    from cageo_gb300 import _build
    assert os.path.exists(_build.DRAINAGE), "run cageo_gb300._build.build() first"
    return subprocess.run([_build.DRAINAGE, *args], cwd=cwd, capture_output=True, text=True,
                          timeout=60)


def test_help_lists_reference_options(tmp_path):
    r = _run(["--help"], tmp_path)
    assert r.returncode == 0
    for opt in ("--dem", "--stream", "--dem-path", "--stream-path", "--filter-type",
                "--practical-range", "--error-mean", "--error-standard-deviation",
                "--iterations", "--gpu", "--cpu", "--output-file", "--output-option"):
        assert opt in r.stdout, opt


@pytest.mark.parametrize("args, text", [
    (["--cpu"], "GPU only"),
    (["--bogus"], "unrecognised option"),
    (["--dem"], "missing value"),
    (["--fill", "fast"], "'cpu' or 'exact'"),
    (["--filter-type", "Spherical"], "Unknown filter type"),
    (["--bevel-radius", "6"], "outside 1..5"),
    (["--bevel-radius=0"], "outside 1..5"),
    (["-o", "counts.tif"], "Unknown output extension"),
    (["--output-option", "middle"], "Unknown output option"),
    (["-i", "-3"], "must not be negative"),
    (["--practical-range", "abc"], "practical range"),
    (["--practical-range=0"], "practical range"),
])
def test_refusals(inputs, args, text):
    r = _run(["--dem-path", str(inputs), "-i", "1", "--seed", "1", *args], inputs.parent)
    assert r.returncode == 1, (args, r.stdout, r.stderr)
    assert text in r.stdout + r.stderr, (args, r.stdout, r.stderr)


def test_cpu_false_is_not_refused_by_the_parser(inputs):
    """`--cpu=0` keeps the GPU; the run then stops at the missing stream
    header, i.e. after parsing."""
    os.remove(inputs / "streams.hdr")
    r = _run(["--dem-path", str(inputs), "--cpu=0", "--gpu=1"], inputs.parent)
    assert r.returncode == 1 and "stream header" in r.stderr


@pytest.mark.parametrize("field, value, text", [
    ("ncols", 9, "sizes of the DEM and stream data"),
    ("nrows", 7, "row counts"),
    ("cellsize", 5.0, "cell size"),
])
def test_header_mismatch(inputs, field, value, text):
    from cageo_gb300 import api
    hdr = {"ncols": 8, "nrows": 6, "cellsize": 10.0}
    hdr[field] = value
    api.write_header(str(inputs / "streams.hdr"), hdr["ncols"], hdr["nrows"], hdr["cellsize"],
                     -9999.0)
    r = _run(["--dem-path", str(inputs)], inputs.parent)
    assert r.returncode == 1 and text in r.stdout and "Exiting" in r.stdout


def test_missing_and_malformed_inputs(inputs):
    r = _run(["--dem-path", str(inputs), "--dem", "absent"], inputs.parent)
    assert r.returncode == 1 and "DEM header" in r.stderr
    (inputs / "dem10.hdr").write_text("ncols 8\nnrows 6\nslope 3\n")
    r = _run(["--dem-path", str(inputs)], inputs.parent)
    assert r.returncode == 1 and "slope" in r.stderr
    from cageo_gb300 import api
    api.write_header(str(inputs / "dem10.hdr"), 8, 6, 10.0, -9999.0)
    api.write_raster(str(inputs / "dem10.bin"), np.ones(47, np.float32))  # one value short
    r = _run(["--dem-path", str(inputs)], inputs.parent)
    assert r.returncode == 1 and "DEM raster" in r.stderr
