"""Benchmark: Monte Carlo drainage-basin realizations/s at an 8192 x 8192 DEM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload ("eval-8192"): 8192^2 float32 DEM from seeded spectral fBm (Hurst
0.8, 0-300 m relief, 10 m cells) with 20000 pits of 0.5-3 m; stream raster
1.0 where D8 accumulation on the priority-flood-routed DEM exceeds 2000
cells, -9999 elsewhere; Gaussian filter, 60 m practical range, error sd
1.5 m.  Synthetic data stands in for the reference's missing sample DEM.

A step is one batched step: `batch` realizations (noise -> convolution ->
realistic DEM -> burning -> pit fill -> routing -> tracing -> border count)
over the whole DEM, their pit fills sharing one stacked grid; `batch` is
chosen by timing among --batch-candidates, and the same realizations run
one at a time are reported beside it (batch_steps.plain_value).  Every grid is 256 MiB, larger than the 129 MB L2, so no flush is
needed between steps.  `value` times K steps with the grids resident on
the device (CUDA events on the pipeline's stream); `e2e` times the same K
steps through the C ABI from pinned host buffers: upload of DEM and
streams, the K realizations, download of the counts (the bytes are spread
over the K steps).

--impl reference times the reference's CPU algorithm (the oracle's
restatement, which is pinned bit-exactly to the reference's own CPU stage
code by the golden fixtures) on the host cores, one whole-DEM realization
per timed step.

With --gpus N > 1 (torchrun, one process per GPU) every rank runs its own
realizations (replicas: the path has no exchange until the final count
sum, which is done once after timing) and the value is the total rate.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC realizations/sec at 8192^2 DEM, learned+batched vs plain GPU, exact basins"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0
# Algorithmic bytes per cell of each stage (unfused compulsory I/O).
STAGE_BYTES = {"noise": 4, "front": 40, "fill": 8, "route": 5, "trace": 6, "border": 12}
PIPE_BYTES = 75
# The dominant kernel is the pit fill's lower-bound flood (fill_flood_kernel
# with clean marks, 35% of a realization).  Its algorithmic bytes are those
# of one fill pass: read q (4 B) and write the filled value (4 B) per cell.
# Its DRAM bytes per launch come from an ncu capture of the 4096^2 workload
# (dram__bytes_read.sum + dram__bytes_write.sum of that launch divided by
# its 16.8 M cells), applied per cell to the benchmark grid.
FLOOD_A_BYTES_PER_CELL = 8
FLOOD_A_TRAFFIC_PER_CELL = 614.9e6 / (4096 * 4096)


_T0 = time.time()


def progress(what):
    """One line on stderr per phase of the run, with the elapsed seconds."""
    print("[bench %7.1f s] %s" % (time.time() - _T0, what), file=sys.stderr, flush=True)


def peak_hbm():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def workload(name="eval-8192"):
    from cageo_gb300 import synth
    dem, streams, p = synth.workload(name, ids="ones")
    return dem, streams, p


def cpu_rate(dem, streams, p, steps, first_real, window=None, gpu_noise=True):
    """Oracle realizations (the reference's CPU algorithm, pinned bit-exactly
    to its own CPU stage code) on the whole DEM, or on its top-left
    `window` x `window` cells.  Returns (realizations/s of what was timed,
    threads, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle, build
    if not os.path.exists(Oracle.path):
        build()
    o = Oracle()
    from cageo_gb300 import api
    H, W = dem.shape
    wy, wx = (H, W) if window is None else (min(window, H), min(window, W))
    d = np.ascontiguousarray(dem[:wy, :wx])
    s = np.ascontiguousarray(streams[:wy, :wx])
    r = api.filter_radius(p["range_m"], p["cell"])
    taps = api.filter_build(api.FILTER_GAUSSIAN, p["range_m"], p["cell"], r)
    mc = np.zeros_like(d)
    if gpu_noise:
        import torch
        nt = torch.empty((wy, wx), dtype=torch.float32, device="cuda")
    total = 0.0
    for k in range(steps):
        if gpu_noise:
            api.noise_philox(nt, 1, first_real + k, 0.0, p["sigma"])
            noise = nt.cpu().numpy()
        else:
            noise = (np.random.default_rng(first_real + k).standard_normal((wy, wx))
                     * p["sigma"]).astype(np.float32)
        t0 = time.perf_counter()
        mc, *_ = o.realization(d, s, noise, taps, r, 1, mc)
        total += time.perf_counter() - t0
    return steps / total, o.threads(), total


def sample_text(steps, dem):
    """What cpu_rate timed: `steps` realizations of the whole DEM."""
    H, W = dem.shape
    return "%d realizations of the whole %dx%d DEM" % (steps, W, H)


# Untimed warm-up realizations of the reference arm run on this window of
# the DEM (they start the OpenMP pool and page the code in); the timed steps
# are whole-DEM realizations.
REF_WARMUP_WINDOW = 1024


def run_reference(args, rank, world):
    if rank != 0:
        return
    dem, streams, p = workload(args.workload)
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    cpu_rate(dem, streams, p, max(args.warmup, 1), 10_000, window=REF_WARMUP_WINDOW,
             gpu_noise=False)
    t0 = time.perf_counter()
    rate, threads, sec = cpu_rate(dem, streams, p, args.steps, 0, gpu_noise=False)
    wall = time.perf_counter() - t0
    H, W = dem.shape
    sample = sample_text(args.steps, dem)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "realizations/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 / rate, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "width": W, "height": H, "filter": "Gaussian %g m" % p["range_m"],
                       "error_sd": p["sigma"], "pits": p["pits"], "stream_threshold": p["threshold"],
                       "parallelism": "cpu",
                       "warmup_steps": "%d realizations of a %dx%d window (untimed)" % (
                           max(args.warmup, 1), min(REF_WARMUP_WINDOW, W), min(REF_WARMUP_WINDOW, H))},
            "cpu_baseline": {"value": rate, "unit": "realizations/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": "realizations/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


def batched(jobs=256, seed=5):
    """The batched configuration: `jobs` realizations round-robin over a
    2048^2 DEM and three uneven tiles (257x1013, 1500x733, 3001x401), each
    with its own exponential filter (range U[30, 120] m, sd U[1, 3] m).
    Wall time around the whole batch (filters are built per job), with the
    DEMs' jobs on concurrent streams, and the same jobs one DEM after
    another (plain_same_jobs)."""
    import torch
    from cageo_gb300 import batch, synth
    grids = synth.batched_grids(seed=seed)
    js = batch.mixed_jobs(len(grids), jobs, seed=seed)
    out = {}
    for name, concurrent in (("value", True), ("plain_same_jobs", False)):
        b = batch.Batch(grids, seed=seed)
        b.run(js[:len(grids)], concurrent=concurrent)  # warm-up: one job per DEM
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run(js, concurrent=concurrent)
        torch.cuda.synchronize()
        out[name] = jobs / (time.perf_counter() - t0)
        b.close()
    cells = sum(g[0].size for g in grids) / len(grids)
    return {"jobs": jobs, "value": out["value"], "unit": "realizations/s",
            "plain_same_jobs": out["plain_same_jobs"],
            "concurrent_over_sequential": out["value"] / out["plain_same_jobs"],
            "mean_cells_per_realization": cells,
            "shapes": [list(g[0].shape[::-1]) for g in grids],
            "filter": "Exponential, range U[30,120] m, sd U[1,3] m per job",
            "note": "value: each DEM's jobs on its own stream and host thread; "
                    "plain_same_jobs: the same jobs one DEM after another"}


# Dry thresholds (metres) of the learned warm start: cells predicted
# shallower start at their elevation.  Lower is more conservative (fewer
# wet cells started dry, each of which the fill must restart).
WARM_THRESHOLDS = (0.005, 0.0, -0.02, -0.5)


def exact_mode(dem, streams, cfg, steps, warmup, base):
    """The reference GPU path's semantics (exact fill): plain realizations/s
    and with the learned warm start at each dry threshold (verified and
    repaired inside the fill, so its counts equal the plain ones),
    device-timed on the pipeline's stream; the best threshold is reported as
    `learned`, every one under `learned_by_threshold`."""
    import torch
    from cageo_gb300 import api, learned
    H, W = dem.shape
    params = learned.load_params()

    def timed_run(pe):
        ext = torch.cuda.ExternalStream(pe.stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(ext)
        pe.run(base + 30_000, steps)
        b.record(ext)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        return {"value": steps / (ms / 1000.0), "unit": "realizations/s", "ms_per_step": ms / steps}

    pe = api.Pipeline(dem, streams, fill_mode=api.FILL_EXACT, **cfg)
    pe.run(base, warmup)
    plain = timed_run(pe)
    st = pe.stats()
    plain.update(fill_rounds_last=st["flood_a_rounds"], fill_us_last=st["flood_a_us"],
                 counts_sum=float(pe.counts().sum()))
    pe.close()
    rows = []
    for thr in WARM_THRESHOLDS:
        pe = api.Pipeline(dem, streams, fill_mode=api.FILL_EXACT, **cfg)
        pe.set_warmstart(params, thr)
        pe.run(base, warmup)
        pe.set_warmstart(params, thr)  # counters from zero
        row = timed_run(pe)
        ws = pe.warmstart_stats()
        k = max(1, ws["realizations"])
        row.update(threshold_m=thr, realizations_with_restarts=ws["repaired"] / k,
                   restarted_cells_per_step=ws["reset_cells"] / k,
                   restarted_cell_share=ws["reset_cells"] / k / (H * W),
                   warm_fill_rounds_per_step=ws["warm_rounds"] / k,
                   repair_fill_rounds_per_step=ws["repair_rounds"] / k,
                   repair_tiles_per_step=ws["repair_tiles"] / k,
                   warm_fill_us_per_step=ws["warm_fill_us"] / k,
                   repair_fill_us_per_step=ws["repair_fill_us"] / k,
                   counts_sum=float(pe.counts().sum()))
        row["counts_equal_plain"] = row["counts_sum"] == plain["counts_sum"]
        rows.append(row)
        pe.close()
    best = max(rows, key=lambda r: r["value"])
    out = {"plain": plain, "learned": dict(best), "learned_by_threshold": rows,
           "learned_over_plain": best["value"] / plain["value"]}
    # The fused network inference alone (features + 3 layers + warm surface)
    # on a grid of the workload's size, device-timed on torch's stream.
    pt = torch.from_numpy(params).cuda()
    v = torch.from_numpy(np.ascontiguousarray(dem)).cuda()
    for _ in range(2):
        api.ws_infer(pt, v, best["threshold_m"])
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(3):
        api.ws_infer(pt, v, best["threshold_m"])
    b.record()
    torch.cuda.synchronize()
    out["learned"]["inference_ms"] = a.elapsed_time(b) / 3
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-exact", action="store_true", help="skip the exact-mode measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched measurement")
    ap.add_argument("--batch-candidates", default="1,4,8,16",
                    help="realizations per batched step to choose from (by timing)")
    ap.add_argument("--workload", default="eval-8192",
                    help="eval-8192 (the benchmark) or a smaller case for profiling (plain-4096)")
    args = ap.parse_args()
    args.batch_candidates = [int(b) for b in args.batch_candidates.split(",") if b]
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    from cageo_gb300 import api, _build
    if not os.path.exists(_build.LIB):
        _build.build()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    dem, streams, p = workload(args.workload)
    progress("workload %s ready" % args.workload)
    H, W = dem.shape
    N = H * W
    cfg = dict(cell_size=p["cell"], filter_model=api.FILTER_GAUSSIAN,
               practical_range=p["range_m"], error_stddev=p["sigma"], seed=1)
    pipe = api.Pipeline(dem, streams, **cfg)
    from cageo_gb300.replicas import realization_range
    # disjoint realization numbers per rank (replicas; weak scaling)
    base, _ = realization_range(rank, world, world * 1_000_000)
    ext = torch.cuda.ExternalStream(pipe.stream)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(first, count):
        """Device milliseconds of `count` realizations on the pipeline's stream."""
        torch.cuda.synchronize()
        start.record(ext)
        pipe.run(first, count)
        stop.record(ext)
        torch.cuda.synchronize()
        return start.elapsed_time(stop)

    # Autotuning of the fill's launch settings, then of the realizations per
    # batched step (each candidate: one step to capture its graph, then 3
    # timed steps), then warm-up (graph capture) and the stage profile.
    # None of it is timed.
    tuned, tune_ms = pipe.autotune(base + 900_000, trials=3)
    progress("autotuned: %s" % tuned)
    batch_ms = {}
    for b in args.batch_candidates:
        try:
            pipe.set_batch(b)
        except api.CageoError as e:  # a stack of b grids at 2^31 cells or more, or no memory
            progress("batch size %d refused: %s" % (b, e))
            continue
        pipe.run(base + 800_000, b)
        batch_ms[b] = timed(base + 800_000 + 100 * b, 3 * b) / (3 * b)
    batch = min(batch_ms, key=batch_ms.get)
    progress("batch sizes timed: %s" % batch_ms)
    free_b, total_b = torch.cuda.mem_get_info()
    pipe.set_batch(batch)
    pipe.run(base, args.warmup * batch)
    prof = pipe.profile(base + args.warmup * batch, fill_parts=True)
    stage_ms = {k: prof[k] for k in pipe.STAGES}
    fill_parts_ms = {k: prof[k] for k in pipe.FILL_PARTS}
    stats = pipe.stats()
    pipe.reset_counts()
    progress("warm-up and stage profile done")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # A step is one batched step: `batch` realizations.
    barrier()
    with ClockSampler(local) as clocks:
        start.record(ext)
        pipe.run(base + 10_000, args.steps * batch)
        stop.record(ext)
        barrier()
    ms = start.elapsed_time(stop)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.steps * batch / (ms / 1000.0)
    progress("timed region: %.1f ms" % ms)
    gpu_launches = args.steps * pipe.graph_kernels()
    # The same realizations one at a time (the plain pipeline), for the
    # batching gain; not part of the headline.
    pipe.set_batch(1)
    pipe.run(base + 40_000, args.warmup)
    plain_ms = timed(base + 50_000, args.steps * batch)
    plain_value = world * args.steps * batch / (plain_ms / 1000.0)
    progress("one at a time: %.1f ms" % plain_ms)

    # End to end through the C ABI from pinned host memory.
    dem_h = torch.from_numpy(dem).pin_memory()
    st_h = torch.from_numpy(streams).pin_memory()
    counts_h = torch.empty((H, W), dtype=torch.float32).pin_memory()
    barrier()
    t0 = time.perf_counter()
    pe = api.Pipeline(dem_h.numpy(), st_h.numpy(), **cfg)
    pe.set_tuning(tuned["fill_rounds"], tuned["fill_warps"], tuned["conv_tile"])
    pe.set_batch(batch)
    pe.run(base + 20_000, args.steps * batch)
    pe.counts(out=counts_h)
    if world > 1:
        c = counts_h.cuda()
        dist.all_reduce(c)
        counts_h.copy_(c.cpu())
    barrier()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    pe.close()
    e2e_value = world * args.steps * batch / e2e_s
    progress("end to end: %.2f s" % e2e_s)

    if rank != 0:
        pipe.close()
        if world > 1:
            dist.destroy_process_group()
        return

    hbm, peak_kind = peak_hbm()
    flood_ms = fill_parts_ms["flood_a"]
    achieved = FLOOD_A_BYTES_PER_CELL * N / (flood_ms / 1000.0) / 1e9
    fill_achieved = STAGE_BYTES["fill"] * N / (stage_ms["fill"] / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "realizations/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded fBm DEM + pits, D8-accumulation streams)",
        "config": {"workload": args.workload, "width": W, "height": H, "filter": "Gaussian %g m" % p["range_m"],
                   "error_sd": p["sigma"], "pits": p["pits"], "stream_threshold": p["threshold"],
                   "hurst": p["hurst"], "relief_m": [p["lo"], p["hi"]],
                   "realizations_per_step": batch, "l2": "inputs larger than L2 (256 MiB grids)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "cuda_graph": True,
                   "autotune": {"chosen": tuned,
                                "ms_per_realization": [dict(c, ms=round(v, 4))
                                                       for c, v in tune_ms]}},
        "cells_per_s": value * N,
        "e2e": {"value": e2e_value, "unit": "realizations/s",
                "h2d_bytes_per_step": int(2 * 4 * N / args.steps),
                "d2h_bytes_per_step": int(4 * N / args.steps),
                "note": "upload of DEM+streams and download of the counts, once per job, spread over the steps"},
        "gpu_launches": None,
        "stage_ms": stage_ms,
        "fill_stats": stats,
        "fill_parts_ms": fill_parts_ms,
        "roofline": {"bound": "hbm",
                     "kernel": "fill_flood_kernel (pit fill, lower-bound flood with clean marks)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": FLOOD_A_TRAFFIC_PER_CELL * N,
                     "traffic_note": "DRAM bytes of one launch: ncu at 4096^2, scaled by cells",
                     "launch_ms": flood_ms,
                     "algorithmic_bytes_per_cell": FLOOD_A_BYTES_PER_CELL,
                     "peak_kind": peak_kind},
        "fill_stage_roofline": {"achieved": fill_achieved, "peak": hbm,
                                "frac": fill_achieved / hbm, "ms": stage_ms["fill"],
                                "algorithmic_bytes_per_cell": STAGE_BYTES["fill"]},
        "pipeline_roofline": {"achieved": value / world * N * PIPE_BYTES / 1e9, "peak": hbm,
                              "frac": value / world * N * PIPE_BYTES / 1e9 / hbm,
                              "bytes_per_cell": PIPE_BYTES},
        "clocks": clocks.summary(),
    }
    # Kernel nodes of the captured batched-step graph, replayed once per step.
    line["gpu_launches"] = gpu_launches
    # Device memory in use with the benchmark pipeline set up for its
    # largest batch candidate (every allocation of the library included).
    line["hbm_used_gb"] = round((total_b - free_b) / 1e9, 2)
    line["batch_steps"] = {
        "realizations_per_step": batch,
        "ms_per_realization": {str(b): round(v, 4) for b, v in batch_ms.items()},
        "value": value, "plain_value": plain_value, "batched_over_plain": value / plain_value,
        "note": "plain: the same number of realizations one at a time (batch 1), same pipeline"}
    if not args.no_exact:
        line["exact_mode"] = exact_mode(dem, streams, cfg, args.steps, args.warmup, base)
        progress("exact mode done")
    if not args.no_batched:
        line["batched"] = batched()
        progress("uneven-tile batch done")
    if not args.no_cpu_baseline:
        rate, threads, sec = cpu_rate(dem, streams, p, args.cpu_steps, 50_000)
        line["cpu_baseline"] = {"value": rate, "unit": "realizations/s", "cores": threads,
                                "kind": "port", "seconds": sec,
                                "sample": sample_text(args.cpu_steps, dem)}
    print(json.dumps(line), flush=True)
    pipe.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
