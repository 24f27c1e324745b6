"""The oracle's trace-path statistics (used to show the reference walk's
100001-step cap never triggers on a workload) against a direct walk."""
import numpy as np


def _walk_lengths(dirs, streams):
    H, W = streams.shape
    longest, never = 0, 0
    for y in range(H):
        for x in range(W):
            if streams[y, x] >= 0:
                continue
            cx, cy, steps = x, y, 0
            while steps <= W * H:
                dx, dy = dirs[cy, cx]
                cx, cy, steps = cx + dx, cy + dy, steps + 1
                if not (0 <= cx < W and 0 <= cy < H) or streams[cy, cx] >= 0:
                    break
            else:
                never += 1
                continue
            longest = max(longest, steps)
    return longest, never


def test_path_stats_hand_made(oracle):
    dirs = np.zeros((1, 6, 2), np.int8)
    dirs[0, :, 0] = 1  # every cell points east: lengths 6, 5, ..., 1
    streams = np.full((1, 6), -9999.0, np.float32)
    assert oracle.trace_path_stats(dirs, streams) == (6, 0)
    streams[0, 3] = 1.0  # cells 0..2 stop at the stream: 3, 2, 1; cells 4, 5: 2, 1
    assert oracle.trace_path_stats(dirs, streams) == (3, 0)
    dirs[0, 5] = 0  # cell 5 has no direction: 4 and 5 never terminate
    assert oracle.trace_path_stats(dirs, streams) == (3, 2)


def test_path_stats_random_directions(oracle):
    rng = np.random.default_rng(3)
    for H, W in [(7, 9), (16, 5), (12, 12)]:
        dirs = rng.integers(-1, 2, size=(H, W, 2)).astype(np.int8)
        streams = np.where(rng.random((H, W)) < 0.08, 1.0, -9999.0).astype(np.float32)
        assert oracle.trace_path_stats(dirs, streams) == _walk_lengths(dirs, streams)
