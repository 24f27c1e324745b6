"""Batches of realizations over several DEMs with per-realization filters.

The reference runs one DEM and one filter per process (src/main.cpp:110-136);
a batch here is a list of jobs (dem index, realization number, filter model,
practical range, error mean, error standard deviation) over a set of DEMs,
each DEM keeping its own count grid.  Every job is one realization with
exactly the stage semantics of a single run, so each job's contribution
equals a one-realization run of the reference on that DEM with that filter.
"""
import numpy as np

from . import api


class Batch:
    def __init__(self, grids, cell_size=10.0, seed=0, nodata_dem=-9999.0, nodata_stream=-9999.0,
                 bevel_radius=2):
        """grids: list of (dem, streams) float32 arrays (any shapes)."""
        import torch
        self.device = torch.cuda.current_device()  # worker threads run on this device too
        self.pipes = [api.Pipeline(d, s, cell_size=cell_size, filter_model=api.FILTER_EXPONENTIAL,
                                   practical_range=30.0, seed=seed, nodata_dem=nodata_dem,
                                   nodata_stream=nodata_stream, bevel_radius=bevel_radius,
                                   use_graphs=False)
                      for d, s in grids]

    def run(self, jobs, concurrent=True):
        """jobs: iterable of (dem_index, realization, model, range_m, mean, sd).

        With `concurrent`, each DEM's jobs run in order on a host thread of
        their own: every pipeline has its own stream and synchronizes only
        that stream, and the library releases the interpreter while it
        works, so the DEMs' kernels overlap on the GPU.  Each DEM's counts
        are sums of its jobs' border masks, so they do not depend on how
        the DEMs interleave."""
        per = [[] for _ in self.pipes]
        for job in jobs:
            per[job[0]].append(job)

        def run_dem(k):
            import torch
            torch.cuda.set_device(self.device)
            for _, real, model, rng_m, mean, sd in per[k]:
                self.pipes[k].run_filter(int(real), 1, int(model), float(rng_m), float(mean),
                                         float(sd))

        if not concurrent:
            for k in range(len(self.pipes)):
                run_dem(k)
            return
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=len(self.pipes)) as ex:
            for f in [ex.submit(run_dem, k) for k in range(len(self.pipes)) if per[k]]:
                f.result()

    def counts(self):
        return [p.counts() for p in self.pipes]

    def close(self):
        for p in self.pipes:
            p.close()


def mixed_jobs(n_dems, count, seed=0, model=api.FILTER_EXPONENTIAL, range_m=(30.0, 120.0),
               sd=(1.0, 3.0)):
    """`count` jobs round-robin over the DEMs, range and sd drawn uniformly."""
    rng = np.random.default_rng(seed)
    return [(j % n_dems, j, model, float(rng.uniform(*range_m)), 0.0, float(rng.uniform(*sd)))
            for j in range(count)]
