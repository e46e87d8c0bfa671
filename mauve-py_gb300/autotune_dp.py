#!/usr/bin/env python3
"""Chooses the gap-DP kernel shape on this GPU and writes dp_tuning.json.

    python mauve-py_gb300/autotune_dp.py [--nprob 4000]

Knobs: rows per lane of the full-DP kernel (4 or 8: the tile is a strip of
128 or 256 rows swept column by column) and of the banded kernel (1, 2, 4
or 8); warps per problem of the full DP, i.e. the bucket edge between the
problems a whole CTA (8 warps) pipelines and those one warp solves (at
least S strips: S in 8, 12, 16, 24, 32, 48); and, for the record, the
batch launched as one CUDA graph or launch by launch.  The full DP is timed on a
sample of the gap-DP distribution (lengths log-uniform 10-20,000,
divergence U(0,30%)); the banded DP on gaps drawn like the recoded-genome
pair's, with the trained band-proposal network's bands when weights are
present (else the network-free band).  The choice with the best time wins;
the measured table is written next to it.  mvg.Context applies the file.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (HERE, os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

import bandnet  # noqa: E402
import mvg  # noqa: E402

WEIGHTS = os.path.join(HERE, "bandnet_weights.npz")


def run(args):
    import torch

    import synth
    from train_bandnet import DeviceBatch, timed_banded, timed_full
    dev = torch.device("cuda", 0)
    ctx = mvg.Context(0)
    res = {"full": {}, "banded": {}}
    full = DeviceBatch(*synth.gap_batch(seed=21, nprob=args.nprob), dev)
    for rows in (4, 8):
        ctx.set_dp_rows(rows, 4)
        timed_full(ctx, full)  # warm
        secs = min(timed_full(ctx, full)[0] for _ in range(2))
        res["full"][rows] = {"seconds": secs, "gcups": full.cells / secs / 1e9}
    best_full = max(res["full"], key=lambda r: res["full"][r]["gcups"])
    ctx.set_dp_rows(best_full, 4)
    res["coop_min_strips"] = {}
    for strips in (8, 12, 16, 24, 32, 48):
        ctx.set_dp_coop_strips(strips)
        timed_full(ctx, full)  # warm
        secs = min(timed_full(ctx, full)[0] for _ in range(2))
        res["coop_min_strips"][strips] = {"seconds": secs, "gcups": full.cells / secs / 1e9}
    best_coop = max(res["coop_min_strips"], key=lambda r: res["coop_min_strips"][r]["gcups"])
    ctx.set_dp_coop_strips(best_coop)
    res["graph"] = {}
    for on in (True, False):
        ctx.set_dp_graph(on)
        timed_full(ctx, full)  # warm
        secs = min(timed_full(ctx, full)[0] for _ in range(2))
        res["graph"]["on" if on else "off"] = {"seconds": secs, "gcups": full.cells / secs / 1e9}
    ctx.set_dp_graph(True)
    band = DeviceBatch(*synth.gap_batch_recoded(seed=22, nprob=args.nprob * 5), dev)
    if os.path.exists(args.weights):
        w = np.load(args.weights)
        net = bandnet.BandNet(ctx, params=w["params"])
        if "whole" in w.files:
            ctx.set_band_whole_fraction(float(w["whole"]))
        if "gate" in w.files:
            ctx.set_band_gate(int(w["gate"]))
        d, h = net.propose_dev(*band.ptrs(), band.n, float(w["alpha"]), float(w["beta"]))
        src = "network"
    else:
        d, h = bandnet.heuristic_band(band.la, band.lb)
        src = "network-free band"
    for rows in (1, 2, 4, 8):
        ctx.set_dp_rows(best_full, rows)
        timed_banded(ctx, band, d, h)  # warm
        secs, used, cells = min((timed_banded(ctx, band, d, h)[:3] for _ in range(2)), key=lambda t: t[0])
        res["banded"][rows] = {"seconds": secs, "effective_gcups": band.cells / secs / 1e9,
                               "accept_rate": float((used == 1).mean()), "cells": cells}
    best_band = max(res["banded"], key=lambda r: res["banded"][r]["effective_gcups"])
    out = {"full_rows_per_lane": int(best_full), "band_rows_per_lane": int(best_band),
           "coop_min_strips": int(best_coop),
           "measured": res, "band_source": src, "gpu": torch.cuda.get_device_name(0),
           "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    print(json.dumps(out, indent=1))
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nprob", type=int, default=4000)
    ap.add_argument("--out", default=os.path.join(HERE, "dp_tuning.json"))
    ap.add_argument("--weights", default=WEIGHTS)
    run(ap.parse_args())


if __name__ == "__main__":
    main()
