"""Replicas across GPUs: realizations are independent, so N processes (one
per GPU) run disjoint realization numbers and the per-cell border counts
are summed once at the end -- the only exchange the Monte Carlo loop has.
NCCL reduces device tensors only, so with it the counts are reduced on the
GPU; other backends (gloo) reduce a host copy."""


def realization_range(rank, world, total, first=0):
    """Contiguous share of realizations [first, first+total) for `rank`: (start, count)."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("bad rank/world/total")
    base, extra = divmod(total, world)
    start = first + rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def sum_counts(counts, group=None):
    """Sum a count grid (torch tensor, in place) over the ranks of `group`."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(counts, op=dist.ReduceOp.SUM, group=group)
    return counts


def reduces_on_device(backend):
    """Whether a backend's all-reduce takes device tensors (NCCL) rather
    than host tensors (gloo, mpi)."""
    return str(backend).lower() == "nccl"


def run(pipeline, rank, world, total, first=0, group=None):
    """Run this rank's share on `pipeline` and return the summed float counts
    (a host tensor)."""
    import torch
    import torch.distributed as dist
    start, count = realization_range(rank, world, total, first)
    if count:
        pipeline.run(start, count)
    on_device = (dist.is_available() and dist.is_initialized()
                 and reduces_on_device(dist.get_backend(group)))
    if on_device:
        counts = torch.empty(pipeline.shape, dtype=torch.float32, device="cuda")
        pipeline.counts(out=counts)
        return sum_counts(counts, group).cpu()
    counts = torch.from_numpy(pipeline.counts())
    return sum_counts(counts, group)
