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
