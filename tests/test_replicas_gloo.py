"""Multi-rank host logic of the replica path on CPU with gloo (world size 2):
disjoint, covering realization shares and the final count sum."""
import os
import socket

import numpy as np
import pytest

from cageo_gb300.replicas import realization_range, reduces_on_device


def test_realization_range_partitions():
    for world in (1, 2, 3, 8):
        for total in (0, 1, 7, 100):
            seen = []
            for r in range(world):
                s, c = realization_range(r, world, total, first=5)
                seen.extend(range(s, s + c))
            assert seen == list(range(5, 5 + total))
    with pytest.raises(ValueError):
        realization_range(2, 2, 10)


def test_backend_choice_of_reduction_device():
    """NCCL all-reduces device tensors only: the replica sum then reduces a
    CUDA copy of the counts; gloo reduces the host copy."""
    assert reduces_on_device("nccl") and reduces_on_device("NCCL")
    assert not reduces_on_device("gloo") and not reduces_on_device("mpi")


class _FakePipeline:
    """Counts of `count` realizations starting at `start`: realization k adds
    k + 1 to every cell (host memory only)."""
    shape = (4, 5)

    def __init__(self):
        self.total = 0.0

    def run(self, start, count):
        self.total += float(sum(k + 1 for k in range(start, start + count)))

    def counts(self, out=None):
        assert out is None, "gloo reduces the host copy"
        return np.full(self.shape, self.total, np.float32)


def _run_worker(rank, world, port, out):
    import torch.distributed as dist
    from cageo_gb300.replicas import run
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    out[rank] = run(_FakePipeline(), rank, world, 10).numpy().copy()
    dist.destroy_process_group()


def test_gloo_world2_replica_run():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_run_worker, args=(2, port, out), nprocs=2, join=True,
                           start_method="spawn")
        for r in range(2):
            assert np.all(out[r] == float(sum(k + 1 for k in range(10))))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from cageo_gb300.replicas import realization_range, sum_counts
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    start, count = realization_range(rank, world, 10)
    # Stand-in for a pipeline's counts: each realization k adds k+1 to every cell.
    counts = torch.full((4, 5), float(sum(k + 1 for k in range(start, start + count))))
    sum_counts(counts)
    out[rank] = counts.numpy().copy()
    dist.destroy_process_group()


def test_gloo_world2_count_sum():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        expect = float(sum(k + 1 for k in range(10)))
        for r in range(2):
            assert np.all(out[r] == expect)
