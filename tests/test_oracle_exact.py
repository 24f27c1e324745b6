"""The exact-mode oracle (the reference GPU path's semantics) against
independent literal restatements of the reference kernels' update rules.

orc_pitfill_exact computes the fill by a priority flood; here the reference
kernel's own rule (src/pitfilling/PitFillingAlgorithmGPUCUDA.cu:201-231,
:275-380) is iterated as a synchronous sweep until nothing changes.  The GPU
flat rules (src/flowrouting/FlowRoutingAlgorithmGPUCUDAOriginal.cu:391-437)
are checked on hand-made grids."""
import numpy as np

from cases import bits, make_case


def jacobi_fill(dem, nodata):
    """The reference kernel's rule, iterated synchronously: an interior,
    non-NODATA neighbour n of a source c that is above c's value and not at
    its own elevation takes max(c, dem[n]); sources are border cells and
    cells equal to 0; other cells start at 99990000."""
    H, W = dem.shape
    nod = dem == nodata
    F = np.full((H, W), np.float32(99990000.0))
    src = np.zeros((H, W), bool)
    src[0, :] = src[-1, :] = src[:, 0] = src[:, -1] = True
    src |= dem == 0.0
    src &= ~nod
    F[src] = dem[src]
    F[nod] = dem[nod]
    interior = np.zeros((H, W), bool)
    interior[1:-1, 1:-1] = True
    target = interior & ~nod
    active = src.copy()
    big = np.float32(np.inf)
    for _ in range(4 * H * W):
        cand = np.full((H, W), big, np.float32)
        P = np.pad(np.where(active, F, big), 1, constant_values=big)
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if dx == 0 and dy == 0:
                    continue
                c = P[1 + dy:1 + dy + H, 1 + dx:1 + dx + W]  # value of the neighbour at (y+dy, x+dx)
                cand = np.minimum(cand, c)
        ok = target & (cand < F) & (F != dem)
        new = np.where(ok, np.maximum(cand, dem), F).astype(np.float32)
        changed = new != F
        if not changed.any():
            return F
        F = new
        active = changed
    raise AssertionError("no convergence")


def test_exact_fill_matches_kernel_rule(oracle):
    for (W, H, seed, nod) in [(40, 30, 1, 0), (64, 48, 2, 30), (33, 71, 3, 0), (50, 50, 4, 80)]:
        dem, _ = make_case(W, H, seed=seed, nodata_cells=nod)
        dem = dem.copy()
        dem[5, 5] = 0.0  # an interior stream cell is a source
        got = oracle.pitfill_exact(dem)
        ref = jacobi_fill(dem, np.float32(-9999.0))
        assert np.array_equal(bits(got), bits(ref)), (W, H, seed)


def test_exact_fill_enclosed_cells_keep_initial_value(oracle):
    dem = np.full((9, 9), 50.0, np.float32)
    dem[3:6, 3:6] = -9999.0
    dem[4, 4] = 10.0  # enclosed by NODATA: no path from an outlet
    got = oracle.pitfill_exact(dem)
    assert got[4, 4] == np.float32(99990000.0)
    assert got[3, 3] == np.float32(-9999.0)
    assert np.all(got[0] == 50.0)


def test_gpu_flat_order_first_match():
    """A flat row draining west and east: layer-1 cells choose the first
    qualifying neighbour in N, W, E, S, NW, NE, SW, SE order."""
    from oracle import Oracle, build
    import os
    if not os.path.exists(Oracle.path):
        build()
    o = Oracle()
    dem = np.full((5, 7), 20.0, np.float32)
    dem[2, 0:6] = 10.0   # a flat trough ending at a border cell on the west
    dirs, fd = o.flow_route_gpu(dem, with_flatdist=True)
    # (2,1) is flat: its W neighbour (2,0) is a border cell (flatDist -1) at 10 <= 10.
    assert fd[2, 1] == 1 and tuple(dirs[2, 1]) == (-1, 0)
    # Layers grow eastwards; each cell drains west (first match W before E).
    assert list(fd[2, 1:6]) == [1, 2, 3, 4, 5]
    assert all(tuple(dirs[2, x]) == (-1, 0) for x in range(2, 6))


def test_gpu_routing_skips_nodata():
    """GPU first pass: NODATA cells get flatDist -3 and are never a steepest
    neighbour (the CPU rules would drop into a -9999 cell)."""
    from oracle import Oracle
    o = Oracle()
    dem = np.full((5, 5), 30.0, np.float32)
    dem[2, 2] = 20.0
    dem[2, 3] = -9999.0
    dem[1, 2] = 15.0
    dirs, fd = o.flow_route_gpu(dem, with_flatdist=True)
    assert fd[2, 3] == -3 and tuple(dirs[2, 3]) == (0, 0)
    assert tuple(dirs[2, 2]) == (0, -1)  # to the 15 m cell, not the NODATA one
    cpu = o.flow_route(dem)
    assert tuple(cpu[2, 2]) == (1, 0)


def test_dead_end_trace_reports_error():
    from oracle import Oracle
    o = Oracle()
    dirs = np.zeros((4, 4, 2), np.int8)
    dirs[0, :, 1] = -1   # top row points out
    dirs[1, 1] = (0, 0)  # dead end
    dirs[2, 1] = (0, -1) # drains into the dead end
    dirs[1, 2] = (0, -1) # drains north to the top row
    streams = np.full((4, 4), -9999.0, np.float32)
    lab = o.flow_trace_gpu(dirs, streams)
    assert lab[1, 1] == -9996 and lab[2, 1] == -9996
    assert lab[1, 2] == -9999
