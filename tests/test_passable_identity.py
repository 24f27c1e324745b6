"""The fill's division-free passability test for quantized values (pitfill.cu
passable_quantized): with minE = 0, every q = RN(k / 1000) below 4096 m is
passable -- toElev(toIndex(q)) == q in float arithmetic -- exactly when
p = RN(1000 q) satisfies p >= rint(p).  Checked here for every such q in
IEEE single precision (numpy float32 operations round to nearest)."""
import numpy as np


def test_passable_identity_all_quantized_values():
    k = np.arange(0, 4096000, dtype=np.int64)
    q = (k.astype(np.float32) / np.float32(1000)).astype(np.float32)
    p = (np.float32(1000) * q).astype(np.float32)
    fast = p >= np.rint(p)
    z = np.where(p > 0, np.trunc(p), 0).astype(np.int64)
    elev = (z.astype(np.float32) / np.float32(1000)).astype(np.float32) + np.float32(0)
    assert q.max() < 4096.0
    assert np.array_equal(fast, elev == q)
