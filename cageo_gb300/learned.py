"""Learned warm start of the exact fill: training on the GPU with this
library's own kernels, and its evaluation.  No counterpart in the reference.

Training pairs (perturbed DEM, fill depth) come from the plain exact fill:
a 1024 x 1024 fBm tile (Hurst 0.8, relief scaled from 300 m over 8192 cells
to the tile's extent, pits, streams at accumulation 2000) plus one Philox
noise realization (Gaussian filter, 60 m range, 1.5 m sd) gives the burned
realistic grid v; the exact fill F of v gives the depth F - v.  The network
(csrc/learned.cu) learns min(depth, cap) from the features of v: mean
squared error over random 128 x 128 crops with a 3-cell margin, Adam.  One
pair per step, each (tile, realization) used once.

Usage (on a GPU):
    python -m cageo_gb300.learned train --steps 2000 --out params.npy
    python -m cageo_gb300.learned evaluate --params params.npy
    python -m cageo_gb300.learned infer --size 2048 --repeat 3   # time the inference
"""
import argparse
import json
import os
import time

import numpy as np

from . import api, synth

DEFAULT_PARAMS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                              "warmstart_params.npy")
N_PARAMS = 10721


def init_params(seed=0):
    """He-scaled random weights, zero biases."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    p[0:1152] = rng.standard_normal(1152) * np.sqrt(2.0 / 36)
    p[1184:10400] = rng.standard_normal(9216) * np.sqrt(2.0 / 288)
    p[10432:10720] = rng.standard_normal(288) * np.sqrt(1.0 / 288)
    return p


def load_params(path=None):
    return np.load(path or DEFAULT_PARAMS).astype(np.float32)


def load_meta(path=None):
    """Training record saved beside the parameters (threshold, loss, ...)."""
    p = (path or DEFAULT_PARAMS)[:-4] + ".json"
    with open(p) as f:
        return json.load(f)


class PairSource:
    """(v, features, depth) pairs on the GPU from seeded fBm tiles."""

    def __init__(self, size=1024, tiles=40, seed=1000, hurst=0.8, sd=1.5, range_m=60.0,
                 cell=10.0, threshold=2000, cap=2.0):
        import torch
        relief = 300.0 * (size / 8192.0) ** hurst
        pits = max(int(20000 * (size / 8192.0) ** 2), 1)
        self.tiles = []
        for k in range(tiles):
            dem = synth.add_pits(synth.fbm_dem(size, size, hurst, seed + k, 0.0, relief), pits,
                                 seed + k)
            streams = synth.make_streams(dem, threshold)
            self.tiles.append((torch.from_numpy(dem).cuda(), torch.from_numpy(streams).cuda()))
        self.seed, self.sd, self.cap = seed, sd, cap
        self.r = api.filter_radius(range_m, cell)
        self.taps = api.filter_build(api.FILTER_GAUSSIAN, range_m, cell, self.r)
        self.shape = (size, size)

    def realization(self, k, j):
        """Burned realistic grid of tile k, noise realization j."""
        import torch
        dem, streams = self.tiles[k % len(self.tiles)]
        noise = torch.empty_like(dem)
        api.noise_philox(noise, self.seed + 17 * (k % len(self.tiles)), j, 0.0, self.sd)
        v = api.convolve(noise, api.FILTER_GAUSSIAN, self.taps, self.r)
        api.realistic_dem(dem, v)
        api.stream_burn(v, streams)
        return v

    def pair(self, k, j):
        v = self.realization(k, j)
        filled = api.pitfill(v, mode=api.FILL_EXACT)
        depth = (filled - v).clamp_(0.0, self.cap)
        return v, api.ws_features(v)[0], depth


def train(steps=2000, batch=16, crop=128, lr=2e-3, seed=0, source=None, log=print):
    """Train from random initial weights; returns (params, loss history)."""
    import torch
    src = source or PairSource()
    dev = torch.device("cuda")
    params = torch.from_numpy(init_params(seed)).to(dev)
    m1, m2, grad = (torch.zeros_like(params) for _ in range(3))
    fb = torch.empty((batch, 4, crop, crop), device=dev)
    tb = torch.empty((batch, crop, crop), device=dev)
    dy = torch.empty_like(tb)
    loss = torch.zeros(1, device=dev)
    tmp1 = torch.empty((batch, 32, crop, crop), device=dev)
    tmp2 = torch.empty_like(tmp1)
    wflip = torch.empty(9216, device=dev)
    rng = np.random.default_rng(seed)
    H, W = src.shape
    hist = []
    t0 = time.time()
    for step in range(1, steps + 1):
        k, j = (step - 1) % len(src.tiles), (step - 1) // len(src.tiles)
        _, feat, depth = src.pair(k, j)
        ys = rng.integers(0, H - crop + 1, batch)
        xs = rng.integers(0, W - crop + 1, batch)
        for b in range(batch):
            fb[b] = feat[:, ys[b]:ys[b] + crop, xs[b]:xs[b] + crop]
            tb[b] = depth[ys[b]:ys[b] + crop, xs[b]:xs[b] + crop]
        a1, a2, out = api.ws_forward(params, fb)
        loss.zero_()
        api.ws_mse(out, tb, dy, loss, margin=3)
        grad.zero_()
        api.ws_backward(params, fb, a1, a2, dy, grad, tmp1, tmp2, wflip)
        step_lr = lr * (0.05 ** (step / steps))  # exponential decay to 5 %
        api.ws_adam(params, grad, m1, m2, step_lr, step)
        if step % 50 == 0 or step == 1:
            hist.append((step, float(loss.item())))
            if log:
                log("step %d loss %.5f (%.1f s)" % (step, hist[-1][1], time.time() - t0))
    return params.cpu().numpy(), hist


def evaluate(params, source=None, pairs=8, first_realization=1000,
             thresholds=(0.005, 0.01, 0.02, 0.05, 0.1, 0.2)):
    """Held-out pairs (realizations the training never used): per threshold,
    the cells marked dry, the cells truly dry, the wet cells marked dry
    (each one forces a repair), and the exact fill's sweep work cold vs warm."""
    import torch
    src = source or PairSource()
    p = torch.from_numpy(np.asarray(params, np.float32)).cuda()
    rows = {t: dict(marked=0, dry=0, false_dry=0, pairs_clean=0) for t in thresholds}
    sweep = dict(cold_rounds=0, warm_rounds={t: 0 for t in thresholds}, cold_tiles=0)
    cells = 0
    for n in range(pairs):
        k, j = n % len(src.tiles), first_realization + n
        v = src.realization(k, j)
        filled = api.pitfill(v, mode=api.FILL_EXACT)
        wet = filled > v
        _, pred = api.ws_infer(p, v, want_warm=False, want_depth=True)
        _, sc = api.pitfill_exact_warm(v)
        sweep["cold_rounds"] += sc["rounds"]
        sweep["cold_tiles"] += sc["tiles"]
        cells += v.numel()
        for t in thresholds:
            mark = pred < t
            fd = int((mark & wet).sum())
            r = rows[t]
            r["marked"] += int(mark.sum())
            r["dry"] += int((~wet).sum())
            r["false_dry"] += fd
            r["pairs_clean"] += int(fd == 0)
            warm = torch.where(mark, v, torch.full_like(v, float("inf")))
            _, sw = api.pitfill_exact_warm(v, warm)
            sweep["warm_rounds"][t] += sw["rounds"]
    return dict(cells=cells, pairs=pairs, thresholds=rows, sweeps=sweep)


def time_inference(params=None, size=2048, repeat=3, threshold=0.005, seed=3):
    """Runs the fused inference `repeat` times on a seeded size x size fBm
    grid (after one untimed call); returns (ms per call, share of cells
    started at +inf)."""
    import torch
    dem = synth.fbm_dem(size, size, 0.8, seed, 0.0, 300.0 * (size / 8192.0) ** 0.8)
    v = torch.from_numpy(dem).cuda()
    p = torch.from_numpy(np.asarray(params if params is not None else load_params(),
                                    np.float32)).cuda()
    warm, _ = api.ws_infer(p, v, threshold)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(repeat):
        warm, _ = api.ws_infer(p, v, threshold)
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / repeat, float(warm.isinf().float().mean())


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("cmd", choices=["train", "evaluate", "infer"])
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--tiles", type=int, default=40)
    ap.add_argument("--cap", type=float, default=2.0)
    ap.add_argument("--out", default=DEFAULT_PARAMS)
    ap.add_argument("--params", default=DEFAULT_PARAMS)
    ap.add_argument("--pairs", type=int, default=8)
    a = ap.parse_args()
    if a.cmd == "infer":
        ms, wet = time_inference(load_params(a.params), a.size, a.repeat)
        print(json.dumps({"size": a.size, "ms_per_inference": ms, "wet_start_share": wet}))
        return
    src = PairSource(tiles=a.tiles, cap=a.cap)
    if a.cmd == "train":
        params, hist = train(a.steps, source=src)
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        np.save(a.out, params)
        ev = evaluate(params, src, pairs=a.pairs)
        with open(a.out[:-4] + ".json", "w") as f:
            json.dump(dict(steps=a.steps, tiles=a.tiles, cap=a.cap, loss=hist, evaluation=ev), f,
                      indent=1)
        print(json.dumps(ev, indent=1))
    else:
        print(json.dumps(evaluate(load_params(a.params), src, pairs=a.pairs), indent=1))


if __name__ == "__main__":
    main()
