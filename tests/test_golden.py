"""The oracle's CPU restatement reproduces the reference's own CPU stage
code (golden fixtures made by tests/golden/make_golden.py from the
reference sources) bit for bit, stage by stage."""
import glob
import os

import numpy as np
import pytest

from cases import bits

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def test_fixtures_present():
    assert len(GOLDEN) >= 4


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_port_matches_reference(oracle, path):
    g = np.load(path)
    r, model = int(g["radius"]), int(g["model"])
    conv = oracle.convolve(g["noise"], g["taps"], r, model)
    assert np.array_equal(bits(conv), bits(g["conv"]))
    real = oracle.realistic_dem(g["dem"], conv)
    assert np.array_equal(bits(real), bits(g["realistic"]))
    burned = oracle.stream_burn(real, g["streams"])
    assert np.array_equal(bits(burned), bits(g["burned"]))
    q, filled = oracle.pitfill(burned)
    assert np.array_equal(bits(q), bits(g["quantized"]))
    assert np.array_equal(bits(filled), bits(g["filled"]))
    dirs = oracle.flow_route(filled)
    assert np.array_equal(dirs, g["dirs"])
    labels = oracle.flow_trace(dirs, g["streams"])
    assert np.array_equal(labels, g["labels"])
    mc = oracle.border_accumulate(labels, np.zeros_like(filled))
    assert np.array_equal(mc, g["border"])


def test_fixtures_exercise_the_hard_cases():
    """The fill's skip rule, flats, streams and both labels occur in the fixtures."""
    seen = dict(overfill=0, flat_layers=0, outside=0, lake=0)
    for path in GOLDEN:
        g = np.load(path)
        seen["overfill"] += int(np.sum(g["filled"] > g["quantized"]))
        seen["outside"] += int(np.sum(g["labels"] == -9999))
        seen["lake"] += int(np.sum(g["labels"] == -9998))
    assert seen["overfill"] > 0 and seen["outside"] > 0 and seen["lake"] > 0


def test_reference_harness_reproduces_fixtures():
    """Where the reference harness is built (it needs the reference sources),
    it regenerates the fixtures exactly."""
    from oracle import Reference
    if not os.path.exists(Reference.path):
        pytest.skip("reference harness not built here")
    R = Reference()
    g = np.load(GOLDEN[0])
    q, filled = R.pitfill(g["burned"])
    assert np.array_equal(bits(filled), bits(g["filled"]))
    assert np.array_equal(R.flow_route(filled), g["dirs"])


def _passable(v, minE):
    """The reference fill's round trip toElev(toIndex(v)) == v in float32
    (src/pitfilling/PitFillingAlgorithmCPUOpenMP.h:56-60, 178)."""
    v = np.asarray(v, np.float32)
    p = np.float32(1000.0) * (v - np.float32(minE))
    z = np.where(p > 0, np.where(p >= np.float32(4294967040.0), np.float32(4294967295.0),
                                 np.trunc(p)), 0).astype(np.uint64)
    back = z.astype(np.float32) / np.float32(1000.0) + np.float32(minE)
    return back == v


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_raised_levels_are_passable(path):
    """The invariant the GPU fill's walled flood relies on: a level the
    reference's fill carries to another cell comes from a cell that
    expands, so every cell raised above its own q holds a passable value,
    never a non-passable q.  (A non-passable cell at its own q was reached
    below it; the walled flood treats it as a wall.)"""
    g = np.load(path)
    q, filled = g["quantized"], g["filled"]
    nodata = q == np.float32(-9999.0)
    minE = np.float32(q.min())  # over every cell, NODATA included, as the reference's minmax
    raised = (filled > q) & ~nodata
    assert raised.sum() > 0
    assert np.all(_passable(filled[raised], minE))
    # Non-passable cells exist, so the check is not vacuous.
    assert np.sum(~_passable(q[~nodata], minE)) > 0


@pytest.mark.parametrize("W,H,seed,plateaus,lo", [(256, 200, 61, 0.0, 80.0),
                                                   (300, 257, 62, 0.2, 80.0),
                                                   (200, 180, 63, 0.0, 0.0)])
def test_raised_levels_are_passable_oracle(oracle, W, H, seed, plateaus, lo):
    """The same invariant on seeded grids through the pinned restatement,
    with lake plateaus and with relief starting at 0 (burned streams at 0)."""
    from cases import make_case, gaussian_noise
    from cageo_gb300 import api
    dem, streams = make_case(W, H, seed=seed, plateaus=plateaus, lo=lo)
    r = api.filter_radius(60.0, 10.0)
    taps = api.filter_build(1, 60.0, 10.0, r)
    conv = oracle.convolve(gaussian_noise(W, H, seed + 1, 1.5), taps, r, 1)
    burned = oracle.stream_burn(oracle.realistic_dem(dem, conv), streams)
    q, filled = oracle.pitfill(burned)
    raised = filled > q
    assert raised.sum() > 0
    assert np.all(_passable(filled[raised], q.min()))
