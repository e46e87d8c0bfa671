#!/usr/bin/env python3
"""Benchmark of the pairwise anchoring + gap-alignment path on one GB300.

Step (the `value` workload): the anchoring path on the recoded-genome pair
(B = 4.6 Mbp at GC 0.508 with 40 copies of a 1.3 kbp repeat and 4,300 ORFs;
A = B with 3% ORF codon-third substitutions, 0.05% elsewhere, 200 indels,
5 rearrangements): 2-bit packing, canonical coding-seed mers and radix sort
for both genomes, unique-seed join, hashing, and the bucket-ordered
extension / containment replay that yields the reference's match list.
value = (|A| + |B|) / step time, in Mbp/s, inputs resident in HBM.
e2e   = the same through the host-buffer C-ABI call (copies inside).

`value` covers the anchoring stages only: the metric's "Mbp/s aligned"
(FASTA to XMFA) would also take LCB selection with breakpoint elimination
and the backbone HMM, which are not built here; the line says so in
"value_scope".

Measured in the same run, each with its own check:
  gap_dp          the batched gap DP on the whole 200,000-pair batch (lengths
                  log-uniform 10-20,000, divergence U(0,30%), subs:indels 9:1,
                  indel mean 3), GCUPS, with a one-gap-per-launch baseline on
                  a stratified sample and 400 problems compared with the oracle
  learned_band    plain full DP vs the network's bands (identical output)
  gap_search      the batched gap anchor search on 20,000 gaps drawn like a
                  recursion round's (oracle-checked on a sample of gaps)
  outside_lcbs    the search outside LCBs on the recoded pair (300 regions
                  per genome), checked against the oracle's matcher
  refinement      both gapped-alignment passes over 120 stand-in LCBs
                  (oracle-checked on the refinement ranges of 10 LCBs)
  backbone_detection  the backbone HMM's homologous segments of 20 LCBs
                  (host code, host threads; planted islands checked)
  index_lut       buildIndex's LUT step

    python bench.py [--gpus N --steps K --warmup W] [--impl gb300|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "mauve-py_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Mbp/s aligned & gap-DP GCUPS: batched+learned-band vs plain GPU, bit-exact"
WORKLOAD = ("recoded-genome pair: B 4.6 Mbp GC 0.508, 40x1.3 kbp repeat, 4,300 ORFs; A = B + 3% ORF codon-3rd "
            "subs, 0.05% elsewhere, 200 indels (mean 4), 5 rearrangements 5-50 kbp; coding seed w=15 (0x16df6d)")
GAP_WORKLOAD = ("batched gap DP: the 200,000-pair batch, lengths log-uniform 10-20,000, "
                "divergence U(0,30%), subs:indels 9:1, indel mean 3")
GAP_NPROB = 200_000
VALUE_SCOPE = ("anchoring Mbp/s: pack, coding-seed keys and sort, unique-seed join, hashing and the "
               "extension/containment replay to the reference's match list, for both genomes; 'Mbp/s aligned' "
               "(FASTA to XMFA) is not measured: LCB selection with breakpoint elimination and the backbone HMM "
               "are not built here (the gap search, the search outside LCBs, both gapped-alignment passes and "
               "the LUT are, each measured in its own section)")
L2_FLUSH_BYTES = 256 << 20
OPS_PER_CELL = 10  # D: 2 add + max, I: 2 add + max, M: add + 2 max + add


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout=3.0):
        """Blocks until the first sample has arrived, so that a short timed
        region that starts now is bracketed by samples."""
        t0 = time.time()
        while self.proc is not None and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        n0, t0 = len(self.lines), time.time()
        while len(self.lines) == n0 and time.time() - t0 < 0.6:  # one sample after the region
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world, device):
    """The slowest rank's time (the job's time): an all-reduce MAX over the
    process group (NCCL on the GPUs; any backend works)."""
    if world == 1:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_pair_seed(rank):
    """Each rank aligns its own genome pair (replicas, weak scaling): the
    recoded pair's generator seed for a rank."""
    return 1 + rank


def seeds_for(a, b):
    import oracle as O
    w = O.default_seed_weight((len(a) + len(b)) // 2)
    return O.get_seed(w, 3), w


# ------------------------------------------------------------- CPU side

def cpu_anchoring(a, b, seed, steps):
    """The oracle's restatement of the reference pipeline, single thread."""
    import oracle as O
    ts, m = [], None
    for _ in range(steps):
        t0 = time.perf_counter()
        m = O.pairwise_matches(a, b, seed)
        ts.append(time.perf_counter() - t0)
    return ts, m


def cpu_gapdp_gcups(sa, oa, sb, ob, sample, threads):
    import oracle as O
    la = np.diff(oa.astype(np.int64))
    order = np.argsort(la)
    idx = np.sort(order[np.linspace(0, len(order) - 1, sample).astype(np.int64)])
    a_parts = [sa[oa[k]:oa[k + 1]] for k in idx]
    b_parts = [sb[ob[k]:ob[k + 1]] for k in idx]
    soa = np.concatenate([[0], np.cumsum([len(x) for x in a_parts])]).astype(np.uint64)
    sob = np.concatenate([[0], np.cumsum([len(x) for x in b_parts])]).astype(np.uint64)
    cells = float(np.sum(np.diff(soa.astype(np.int64)) * np.diff(sob.astype(np.int64))))
    t0 = time.perf_counter()
    O.nw_batch(np.concatenate(a_parts), soa, np.concatenate(b_parts), sob, with_paths=True, nthreads=threads)
    dt = time.perf_counter() - t0
    return cells / dt / 1e9, cells, dt


WEIGHTS = os.path.join(ROOT, "mauve-py_gb300", "bandnet_weights.npz")
LB_NPROB = 200_000
# DRAM bytes of the seed-path kernels per match-finding call on the recoded
# pair, from one ncu capture (profiles/anchoring_launch_list_recoded_pair.md);
# below the algorithmic bytes because the sort passes' outputs stay in L2
SEED_PATH_TRAFFIC = 0.36e9
# stages of the seed path (pack, seed keys, bucket or radix sort, unique-pair join)
SEED_STAGES = ("pack", "sml_sort", "seed_scatter", "seed_local", "unique_join")


def learned_band_section(ctx, args, dev, stream, rank):
    """Plain full DP vs the learned band (network proposal + banded DP with
    exactness check + full-DP fallback) on gaps drawn like the recoded-genome
    pair's; both timed with CUDA events over whole calls, outputs compared."""
    if not os.path.exists(WEIGHTS):
        return None
    import torch

    import bandnet
    import synth
    w = np.load(WEIGHTS)
    net = bandnet.BandNet(ctx, params=w["params"])
    alpha, beta = float(w["alpha"]), float(w["beta"])
    whole = float(w["whole"]) if "whole" in w.files else 0.5
    gate = int(w["gate"]) if "gate" in w.files else 0
    ctx.set_band_whole_fraction(whole)
    ctx.set_band_gate(gate)
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=1000 + rank, nprob=args.lb_nprob)
    n = len(oa) - 1
    la, lb = np.diff(oa), np.diff(ob)
    cells = float(np.sum(la * lb))
    path_off = np.zeros(n + 1, np.uint64)
    path_off[1:] = np.cumsum(la + lb)
    t = [torch.from_numpy(x).to(dev) for x in (sa, oa.astype(np.int64), sb, ob.astype(np.int64),
                                             path_off.view(np.int64))]
    ptrs = [x.data_ptr() for x in t[:4]]
    bufs = []
    for _ in range(2):
        bufs.append((torch.zeros(n, dtype=torch.int32, device=dev),
                     torch.zeros(int(path_off[-1]) + 16, dtype=torch.uint8, device=dev),
                     torch.zeros(n, dtype=torch.int64, device=dev)))

    def full(b):
        ctx.gap_align_batch_dev(*ptrs, n, b[0].data_ptr(), b[1].data_ptr(), t[4].data_ptr(), b[2].data_ptr())

    def learned(b):
        d, h = net.propose_dev(*ptrs, n, alpha, beta)
        return ctx.gap_align_banded_dev(*ptrs, n, d, h, b[0].data_ptr(), b[1].data_ptr(), t[4].data_ptr(),
                                        b[2].data_ptr())

    def timed(fn, b, reps):
        out, ms = None, []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            out = fn(b)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return min(ms), out

    full(bufs[0])
    learned(bufs[1])  # warm-up
    ms_full, _ = timed(full, bufs[0], 3)
    ms_band, (used, band_cells) = timed(learned, bufs[1], 3)
    identical = all(bool(torch.equal(x, y)) for x, y in zip(bufs[0], bufs[1]))
    return {
        "workload": "%d gaps drawn like the recoded-genome pair's (lengths log-uniform 20-5000; 90%% at 0.5-3%% "
                    "substitutions, 10%% divergent)" % n,
        "cells_full": cells, "plain_full_ms": round(ms_full, 3), "plain_full_gcups": round(cells / ms_full / 1e6, 2),
        "learned_ms": round(ms_band, 3), "learned_effective_gcups": round(cells / ms_band / 1e6, 2),
        "speedup_vs_plain": round(ms_full / ms_band, 3), "accept_rate": round(float((used == 1).mean()), 4),
        "fallback_rate": round(float((used != 1).mean()), 4),
        "fallback_split": {"rejected_by_check": round(float((used == 0).mean()), 4),
                           "not_tried": round(float((used == 2).mean()), 4)},
        "cells_computed": band_cells,
        "identical_to_full": identical, "weights": "mauve-py_gb300/bandnet_weights.npz",
        "margins": {"alpha": alpha, "beta": beta, "whole_fraction": whole, "divergence_gate": gate},
    }


def gap_sample(oa, k):
    """k problem indices spread evenly over the length order (stratified)."""
    la = np.diff(oa.astype(np.int64))
    order = np.argsort(la, kind="stable")
    return np.sort(order[np.linspace(0, len(order) - 1, k).astype(np.int64)])


def gapdp_checks(ctx, sa, oa, sb, ob, d_sc, d_paths, d_po, d_pl, dev, rank):
    """(1) 400 problems of the timed batch, spread over the length order,
    compared with the oracle (scores and paths); (2) the one-gap-per-launch
    baseline: the same library call made once per problem on a stratified
    sample of 1,000 problems (host planning, launches and synchronisation per
    problem, as a caller without batching would), GCUPS over the sample."""
    import torch

    import oracle as O
    out = {}
    if rank == 0:
        idx = gap_sample(oa, 400)
        sc = d_sc.cpu().numpy()
        pl = d_pl.cpu().numpy()
        po = d_po.cpu().numpy()
        a_parts = [sa[oa[k]:oa[k + 1]] for k in idx]
        b_parts = [sb[ob[k]:ob[k + 1]] for k in idx]
        soa = np.concatenate([[0], np.cumsum([len(x) for x in a_parts])]).astype(np.uint64)
        sob = np.concatenate([[0], np.cumsum([len(x) for x in b_parts])]).astype(np.uint64)
        osc, opl, opath, opo = O.nw_batch(np.concatenate(a_parts), soa, np.concatenate(b_parts), sob,
                                          with_paths=True, nthreads=os.cpu_count() or 1)
        same = bool(np.array_equal(sc[idx], osc))
        for j, k in enumerate(idx):
            if not same:
                break
            g = d_paths[int(po[k]):int(po[k]) + int(pl[k])].cpu().numpy()
            same = int(pl[k]) == int(opl[j]) and np.array_equal(g, opath[int(opo[j]):int(opo[j]) + int(opl[j])])
        out["identical_to_oracle"] = same
        out["oracle_sample"] = "400 problems spread over the length order (scores and paths)"
    idx = gap_sample(oa, 1000)
    cells, tot = 0.0, 0.0
    for j, k in enumerate(np.concatenate([idx[:1], idx])):  # the first call warms up
        la, lb = int(oa[k + 1] - oa[k]), int(ob[k + 1] - ob[k])
        a = torch.from_numpy(sa[oa[k]:oa[k + 1]]).to(dev)
        b = torch.from_numpy(sb[ob[k]:ob[k + 1]]).to(dev)
        o1 = torch.tensor([0, la], dtype=torch.int64, device=dev)
        o2 = torch.tensor([0, lb], dtype=torch.int64, device=dev)
        pos = torch.tensor([0, la + lb], dtype=torch.int64, device=dev)
        scr = torch.zeros(1, dtype=torch.int32, device=dev)
        pth = torch.zeros(la + lb + 16, dtype=torch.uint8, device=dev)
        plen = torch.zeros(1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.gap_align_batch_dev(a.data_ptr(), o1.data_ptr(), b.data_ptr(), o2.data_ptr(), 1, scr.data_ptr(),
                                pth.data_ptr(), pos.data_ptr(), plen.data_ptr())
        torch.cuda.synchronize()
        if j > 0:
            tot += time.perf_counter() - t0
            cells += la * lb
    out["one_gap_per_launch"] = {"gcups": round(cells / tot / 1e9, 3), "cells": cells, "seconds": round(tot, 4),
                                 "sample": "1,000 problems spread over the length order, one library call each "
                                           "(inputs on the device, host time per call included)"}
    return out


GS_NGAPS = 20_000


def gap_search_section(ctx, dev, rank):
    """The batched gap anchor search on 20,000 inter-anchor gaps drawn like
    a recursion round's (both sides log-uniform 200-20,000 bp, the second
    derived from the first at divergence U(0, 30%), subs:indels 9:1, indel
    mean 3), embedded in two genomes with 100-bp spacers, searched in one
    call; the anchors of 100 gaps compared with the oracle."""
    import torch

    import oracle as O
    import synth
    sa, oa, sb, ob = synth.gap_batch(seed=40 + rank, nprob=GS_NGAPS, lmin=200, lmax=20_000)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    spacer = 100
    la, lb = np.diff(oa.astype(np.int64)), np.diff(ob.astype(np.int64))
    sta = oa[:-1].astype(np.int64) + spacer * (np.arange(GS_NGAPS) + 1)
    stb = ob[:-1].astype(np.int64) + spacer * (np.arange(GS_NGAPS) + 1)
    rng = np.random.default_rng(7)
    ga = rng.choice(acgt, int(oa[-1]) + spacer * (GS_NGAPS + 1))
    gb = rng.choice(acgt, int(ob[-1]) + spacer * (GS_NGAPS + 1))
    for k in range(GS_NGAPS):
        ga[sta[k]:sta[k] + la[k]] = acgt[sa[oa[k]:oa[k + 1]]]
        gb[stb[k]:stb[k] + lb[k]] = acgt[sb[ob[k]:ob[k + 1]]]
    gaps = np.stack([sta, la, stb, lb], axis=1).astype(np.int64)
    bases = float(la.sum() + lb.sum())
    da, db = torch.from_numpy(ga).to(dev), torch.from_numpy(gb).to(dev)
    cap = 1 << 24
    ctx.gap_anchor_search_dev(da.data_ptr(), len(ga), db.data_ptr(), len(gb), gaps, cap)  # warm-up
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        anc, off = ctx.gap_anchor_search_dev(da.data_ptr(), len(ga), db.data_ptr(), len(gb), gaps, cap)
        ts.append(time.perf_counter() - t0)
    t = min(ts)
    # one more call with per-stage CUDA events (not timed above)
    ctx.set_profiling(True)
    ctx.gap_anchor_search_dev(da.data_ptr(), len(ga), db.data_ptr(), len(gb), gaps, cap)
    stage_ms = {k: round(v, 3) for k, v in ctx.stage_times().items()}
    ctx.set_profiling(False)
    same = True
    cpu_s, cpu_bases = 0.0, 0.0
    for k in np.linspace(0, GS_NGAPS - 1, 100).astype(np.int64):
        xa, na_, xb, nb_ = (int(v) for v in gaps[k])
        t0 = time.perf_counter()
        w, want = O.gap_anchor_search(ga[xa:xa + na_], gb[xb:xb + nb_])
        cpu_s += time.perf_counter() - t0
        cpu_bases += na_ + nb_
        want = np.zeros((0, 3), np.int64) if want is None else want.copy()
        for q, o in ((0, xa), (1, xb)):
            want[:, q] = np.where(want[:, q] > 0, want[:, q] + o, want[:, q] - o)
        same = same and np.array_equal(anc[off[k]:off[k + 1]], want)
    return {"workload": "%d gaps drawn like a recursion round's (200-20,000 bp log-uniform, divergence U(0,30%%)), "
                        "%.1f Mbp of gap sequence, one call" % (GS_NGAPS, bases / 1e6),
            "value": round(bases / 1e6 / t, 2), "unit": "Mbp/s searched", "ms": round(1e3 * t, 3),
            "gaps": GS_NGAPS, "anchors": int(len(anc)),
            "timing": "host wall clock around the call (the host-side overlap filter included)",
            "stage_ms": stage_ms,
            "identical_to_oracle_on_sample": bool(same), "oracle_sample": "100 gaps spread over the list",
            "cpu_baseline": {"value": round(cpu_bases / 1e6 / cpu_s, 3), "unit": "Mbp/s searched", "cores": 1,
                             "kind": "port", "sample": "the same 100 gaps through the oracle, one thread"}}


OL_NREG = 300


def outside_lcbs_section(ctx, dev, rank):
    """The search outside LCBs (SearchLCBGaps) on the recoded pair: 300
    regions per genome (lengths uniform 0-4,000 bp, as LCB flanks), the
    genomes resident on the device, one call; the result compared with the
    oracle's matcher on the two concatenations finished by the library's
    host steps (which equal the reference's own on the fixtures)."""
    import torch

    import mvg
    import oracle as O
    import synth
    a, b = synth.genome_pair_recoded(seed=1 + rank)
    rng = np.random.default_rng(90 + rank)

    def regions(n):
        cuts = np.sort(rng.choice(np.arange(1, n - 4000), OL_NREG, replace=False))
        out, end = [], 1
        for c in cuts:
            lo = max(int(c), end)
            hi = min(n + 1, lo + int(rng.integers(0, 4000)))
            out += [lo, hi]
            end = hi
        return np.array(out, np.int64)

    ra, rb = regions(len(a)), regions(len(b))
    bases = float(np.diff(ra.reshape(-1, 2)).sum() + np.diff(rb.reshape(-1, 2)).sum())
    da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    cap = 1 << 20
    ctx.search_lcb_gaps_dev(da.data_ptr(), len(a), db.data_ptr(), len(b), ra, rb, cap)  # warm-up
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        got, w = ctx.search_lcb_gaps_dev(da.data_ptr(), len(a), db.data_ptr(), len(b), ra, rb, cap)
        ts.append(time.perf_counter() - t0)
    t = min(ts)
    ca = np.concatenate([a[l - 1:r - 1] for l, r in ra.reshape(-1, 2)])
    cb = np.concatenate([b[l - 1:r - 1] for l, r in rb.reshape(-1, 2)])
    t0 = time.perf_counter()
    raw = O.pairwise_matches(ca, cb, mvg.get_seed(w, 0))
    want = mvg.lcb_gap_finish(raw, ra, rb)
    cpu_s = time.perf_counter() - t0
    return {"workload": "recoded pair, %d regions per genome outside stand-in LCBs (0-4,000 bp), %.2f Mbp "
                        "concatenated, seed weight %d, one call" % (OL_NREG, bases / 1e6, w),
            "value": round(bases / 1e6 / t, 2), "unit": "Mbp/s searched", "ms": round(1e3 * t, 3),
            "matches": int(len(got)),
            "timing": "host wall clock around the device-genome call (gather, GPU matcher, host transposition "
                      "and overlap elimination)",
            "identical_to_oracle": bool(np.array_equal(got, want)),
            "cpu_baseline": {"value": round(bases / 1e6 / cpu_s, 3), "unit": "Mbp/s searched", "cores": 1,
                             "kind": "port", "sample": "the same regions: the oracle's matcher on the "
                                                       "concatenations, then the host steps"}}


RF_NLCB = 120


def refinement_section(ctx, rank):
    """Both gapped-alignment passes a two-genome run makes over its LCBs
    (refineAlignment's anchored realignment of every window, then the final
    RefineFast pass) on 120 stand-in LCBs (a random sequence and a copy with
    2-25% substitutions and one-sided gap runs, about 12,000 columns each);
    every pass is one batched gap-DP call; 200 of the refinement pass's
    ranges compared with the oracle's NWSmall."""
    import mvg
    import oracle as O
    rng = np.random.default_rng(120 + rank)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    lcbs = []
    for _ in range(RF_NLCB):
        n = int(rng.integers(6000, 18000))
        div = float(rng.uniform(0.02, 0.25))
        ra = acgt[rng.integers(0, 4, n)]
        rb = ra.copy()
        sub = rng.random(n) < div
        rb[sub] = acgt[(np.searchsorted(acgt, rb[sub]) + rng.integers(1, 4, int(sub.sum()))) % 4]
        runs = rng.random(n) < 0.01
        for c in np.nonzero(runs)[0]:
            ln = int(rng.geometric(1 / 4.0))
            (ra if rng.random() < 0.5 else rb)[c:c + ln] = ord("-")
        both = (ra == ord("-")) & (rb == ord("-"))
        ra, rb = ra[~both], rb[~both]
        lcbs.append((ra, rb))
    cols = float(sum(len(x[0]) for x in lcbs))
    # the recursion's gap enumeration over the same LCBs (host; each LCB as
    # if at genome position 1 of genomes just long enough)
    t0 = time.perf_counter()
    for ra, rb in lcbs:
        na, nb = int((ra != ord("-")).sum()), int((rb != ord("-")).sum())
        mvg.recursion_gaps(ra, rb, 1, False, 1, False, na, nb)
    rec_s = time.perf_counter() - t0
    ctx.gapped_alignment(lcbs[:4])  # warm-up
    t0 = time.perf_counter()
    first = ctx.refine_alignment(lcbs)
    t1 = time.perf_counter()
    final = ctx.iterative_refine(first)
    t2 = time.perf_counter()
    # the refinement pass's ranges on a sample, against the oracle
    same, cpu_s, cpu_cells, checked = True, 0.0, 0, 0
    code = np.full(256, 0, np.uint8)
    code[np.frombuffer(b"ACGT", np.uint8)] = np.arange(4, dtype=np.uint8)
    for k in range(0, RF_NLCB, 12):
        fa, fb = np.frombuffer(first[k][0], np.uint8), np.frombuffer(first[k][1], np.uint8)
        outa, outb, at = [], [], 0
        for lo, hi in mvg.refine_fast_ranges(fa, fb).tolist():
            outa.append(fa[at:lo])
            outb.append(fb[at:lo])
            wa, wb = fa[lo:hi], fb[lo:hi]
            x, y = wa[wa != ord("-")], wb[wb != ord("-")]
            if len(x) and len(y):
                t3 = time.perf_counter()
                path, _ = O.nw_align(code[x], code[y])
                cpu_s += time.perf_counter() - t3
                cpu_cells += len(x) * len(y)
                i = j = 0
                xa, xb = [], []
                for e in path:
                    xa.append(x[i] if e in "MD" else ord("-"))
                    xb.append(y[j] if e in "MI" else ord("-"))
                    i += e in "MD"
                    j += e in "MI"
                wa, wb = np.array(xa, np.uint8), np.array(xb, np.uint8)
                checked += 1
            outa.append(wa)
            outb.append(wb)
            at = hi
        outa.append(fa[at:])
        outb.append(fb[at:])
        same = same and np.concatenate(outa).tobytes() == final[k][0] and np.concatenate(outb).tobytes() == final[k][1]
    return {"workload": "%d stand-in LCBs of two genomes, %.2f M columns (divergence 2-25%%, one-sided gap runs)"
                        % (RF_NLCB, cols / 1e6),
            "value": round(cols / 1e6 / (t2 - t0), 3), "unit": "M columns/s (both passes)",
            "gapped_alignment_ms": round(1e3 * (t1 - t0), 2), "refinement_ms": round(1e3 * (t2 - t1), 2),
            "timing": "host wall clock around each pass (window and range planning on the host, one batched "
                      "gap-DP call and the GPU row rebuild per pass)",
            "refinement_identical_to_oracle_on_sample": bool(same),
            "recursion_gaps": {"value": round(cols / 1e6 / rec_s, 2), "unit": "M columns/s",
                               "timing": "host wall clock, one mvg_recursion_gaps call per LCB through the Python "
                                         "binding (one thread)"},
            "oracle_sample": "every refinement range of 10 LCBs (%d problems)" % checked,
            "cpu_baseline": {"value": round(cpu_cells / cpu_s / 1e9, 4) if cpu_s else None, "unit": "GCUPS",
                             "cores": 1, "kind": "port", "sample": "the oracle's NWSmall on the same ranges"}}


BB_NLCB = 20


def backbone_section(rank):
    """Backbone detection's homology HMM over 20 LCBs of 200,000 columns (a
    sequence and a 5%-substituted copy with one unrelated 10,000-column
    island each): all LCBs in one call (host threads), then each LCB on its
    own (one thread, as the reference runs the step); the islands found
    checked against where they were planted."""
    import mvg
    rng = np.random.default_rng(180 + rank)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    lcbs = []
    for _ in range(BB_NLCB):
        a = acgt[rng.integers(0, 4, 200_000)]
        b = a.copy()
        sub = rng.random(len(b)) < 0.05
        b[sub] = acgt[rng.integers(0, 4, int(sub.sum()))]
        b[50_000:60_000] = acgt[rng.integers(0, 4, 10_000)]
        lcbs.append((a, b))
    p = mvg.hmm_backbone_params(0.5)
    mvg.homologous_segments(lcbs[:2], p)  # warm-up
    t0 = time.perf_counter()
    segs = mvg.homologous_segments(lcbs, p)
    t = time.perf_counter() - t0
    t0 = time.perf_counter()
    for lcb in lcbs[:4]:
        mvg.homologous_segments([lcb], p)
    t1 = (time.perf_counter() - t0) * BB_NLCB / 4
    cols = float(sum(len(x[0]) for x in lcbs))
    # two homologous stretches around each island, their edges within a few
    # hundred columns of the planted ones (chance matches extend them)
    found = all(len(sg) == 2 and abs(int(sg[0][1]) - 50_000) < 300 and abs(int(sg[1][0]) - 60_000) < 300
                for sg in segs)
    return {"workload": "%d LCBs x 200,000 columns (5%% substitutions, one 10 kbp unrelated island each), "
                        "progressiveMauve's default HMM parameters" % BB_NLCB,
            "value": round(cols / 1e6 / t, 2), "unit": "M columns/s (host threads)", "ms": round(1e3 * t, 2),
            "islands_found": bool(found),
            "single_thread": {"value": round(cols / 1e6 / t1, 2), "unit": "M columns/s",
                              "sample": "4 of the LCBs one at a time (one host thread, as the reference runs it)"}}


def collinear_lcbs_section(rank):
    """LCBs with greedy breakpoint elimination for collinear genomes (host,
    one thread, a sequential heap of moves as in the reference) on a
    synthetic two-genome match list: 300 blocks of 100-1,500 bp, shuffled
    and 30% inverted in genome B, ungapped 9-40 bp matches along each, and
    2,000 random matches; checked that the LCBs and the deleted list
    partition the input."""
    import mvg
    rng = np.random.default_rng(190 + rank)
    nblk = 300
    lens = rng.integers(100, 1500, nblk)
    inv = rng.random(nblk) < 0.3
    pos_a = np.concatenate([[1], 1 + np.cumsum(lens)[:-1]])
    pos_b, p = np.zeros(nblk, np.int64), 1
    for k in rng.permutation(nblk):
        pos_b[k] = p
        p += int(lens[k]) + 10
    m = []
    for k in range(nblk):
        x = 0
        while x < lens[k] - 20:
            L = min(int(rng.integers(9, 40)), int(lens[k] - x))
            m.append((pos_a[k] + x, -(pos_b[k] + lens[k] - x - L) if inv[k] else pos_b[k] + x, L))
            x += L + int(rng.integers(0, 30))
    for _ in range(2000):
        L = int(rng.integers(9, 30))
        m.append((int(rng.integers(1, pos_a[-1] + lens[-1] - L)), int(rng.integers(1, p)) * int(rng.choice([-1, 1])),
                  L))
    m = np.array(m, np.int64)[rng.permutation(len(m))]
    mvg.collinear_lcbs(m[:1000])  # warm-up
    t0 = time.perf_counter()
    lcbs, deleted = mvg.collinear_lcbs(m)
    t = time.perf_counter() - t0
    key = sorted(map(tuple, np.concatenate(lcbs + [deleted]).tolist()))
    return {"workload": "%d matches: %d blocks shuffled and 30%% inverted, 2,000 random matches" % (len(m), nblk),
            "value": round(len(m) / 1e3 / t, 1), "unit": "k matches/s (one host thread)", "ms": round(1e3 * t, 2),
            "lcbs": len(lcbs), "deleted": int(len(deleted)),
            "partition_ok": key == sorted(map(tuple, m.tolist()))}


def xmfa_section(ctx, dev, rank, flush):
    """The XMFA writer (WriteStandardAlignment for pairwise blocks) on a
    genome-sized alignment: 64 blocks, 4.6 Mbp per genome (2% substitutions,
    0.05% indels), every other block on the reverse strand of genome B.
    value: the rows resident on the device, the text assembled there and
    copied into pinned host memory, wall clock with the call's host planning;
    e2e: the host-rows call a user makes (rows copied in, text returned as
    bytes).  Checked by reading the text back with the buildIndex XMFA
    reader: every block's coordinates, strands and rows.  The rows are
    smaller than L2, so L2 is flushed before every timed call."""
    import torch

    import buildindex
    import synth
    gs, rs, off, rg, rr, _, _ = synth.lut_alignment_fast(41 + rank, n_ref=LUT_NREF, sub=0.02, indel=0.0005,
                                                          nblocks=64)
    nb = len(off) - 1
    rs = np.where(np.arange(nb) % 2 == 1, -rs, rs)
    starts = np.stack([gs, rs], 1).reshape(-1)
    lens = np.array([[int((x[int(off[b]):int(off[b + 1])] != ord("-")).sum()) for x in (rg, rr)] for b in range(nb)],
                    np.int64).reshape(-1)
    names = ("genome.fasta", "reference.fasta")
    d_a, d_b = torch.from_numpy(rg).to(dev), torch.from_numpy(rr).to(dev)
    need = ctx.xmfa_write_dev(*names, starts, lens, d_a.data_ptr(), d_b.data_ptr(), off)
    out = torch.empty(need, dtype=torch.uint8, pin_memory=True)

    def dev_step():
        return ctx.xmfa_write_dev(*names, starts, lens, d_a.data_ptr(), d_b.data_ptr(), off, out.data_ptr(), need)

    launches0 = ctx.kernel_launches()
    for _ in range(3):
        dev_step()
    launches = (ctx.kernel_launches() - launches0) / 3
    wall, e2e = [], []
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_step()
        wall.append(time.perf_counter() - t0)
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        text = ctx.xmfa_write(*names, starts, lens, rg, rr, off)
        e2e.append(time.perf_counter() - t0)
    same = out.numpy().tobytes() == text
    groups = buildindex.parse_xmfa_text(text.decode())
    ok = len(groups) == nb
    for b, grp in enumerate(groups if ok else []):
        for q, sub in enumerate(grp.alignments):
            s, n = int(starts[2 * b + q]), int(lens[2 * b + q])
            row = (rg, rr)[q][int(off[b]):int(off[b + 1])].tobytes().decode()
            ok = ok and sub.start_idx == abs(s) and sub.end_idx == abs(s) + n - 1 and sub.seq == row and \
                sub.strand == ("+" if s > 0 else "-")
    t, te = sorted(wall)[2], sorted(e2e)[1]
    return {"workload": "XMFA of %d blocks, %d columns, 4.6 Mbp per genome (%d bytes of text)" % (nb, len(rg), need),
            "value": round(need / 1e6 / t, 1), "unit": "MB/s of XMFA text", "ms": round(1e3 * t, 3),
            "e2e": {"value": round(need / 1e6 / te, 1), "unit": "MB/s of XMFA text", "ms": round(1e3 * te, 3),
                    "h2d_bytes_per_step": int(2 * len(rg)), "d2h_bytes_per_step": int(need)},
            "gpu_launches_per_step": launches, "device_and_host_paths_identical": bool(same),
            "reads_back": bool(ok)}


def mds42_section(ctx, dev, stream, flush):
    """Anchoring on the reference's own recoded E. coli fixture pair
    (tests/golden/mds42.npz, 3.98 Mbp each): device-resident throughput and
    whether the match list equals the reference's."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import load_mds42
    a, b, seed, want = load_mds42()
    da, db = torch.from_numpy(a.copy()).to(dev), torch.from_numpy(b.copy()).to(dev)
    out = torch.zeros(3 * (len(want) + 1024), dtype=torch.int64, device=dev)

    def step():
        return ctx.pairwise_matches_dev(da.data_ptr(), len(a), db.data_ptr(), len(b), seed, out.data_ptr(),
                                        len(want) + 1024)

    for _ in range(3):
        n = step()
    ms = []
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        n = step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    got = out[:3 * n].cpu().numpy().reshape(-1, 3)
    t = sorted(ms)[len(ms) // 2]
    return {"workload": "the reference's recoded E. coli fixture pair (mds42_recoded vs mds42_full, %.2f + %.2f Mbp), "
                        "coding seed w=15" % (len(a) / 1e6, len(b) / 1e6),
            "value": round((len(a) + len(b)) / 1e6 / (t / 1e3), 2), "unit": "Mbp/s", "ms": round(t, 3),
            "matches": int(n), "identical_to_reference": bool(n == len(want) and np.array_equal(got, want))}


LUT_NREF = 4_600_000


def lut_section(ctx, args, dev, stream, rank, flush):
    """buildIndex's LUT step on a genome-sized alignment: the LUT from the
    aligned blocks, fixZeroIdx, fillGaps(300), smoothEdges(20).  value:
    inputs resident on the device (CUDA events); e2e: the host C-ABI call
    with host buffers (copies inside the timed region, wall clock)."""
    import torch

    import indexutils as iu
    import synth
    gs, rs, off, rg, rr, genome, ref = synth.lut_alignment_fast(31 + rank, n_ref=LUT_NREF, sub=0.02, indel=0.0005,
                                                                nblocks=64)
    n, ncols = len(genome), len(rg)
    t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (gs, rs, off.view(np.int64), rg, rr, genome, ref)]
    d_lut = torch.empty(n, dtype=torch.int32, device=dev)
    ptrs = [x.data_ptr() for x in t]

    def dev_step():
        iu.buildIndexLutDev(*ptrs[:5], len(gs), ptrs[5], n, ptrs[6], len(ref), d_lut.data_ptr(), n, ctx=ctx)

    blocks = iu.Blocks(gs, rs, off, rg, rr)
    host_lut = None
    for _ in range(max(3, args.warmup)):
        dev_step()
        host_lut = iu.buildIndexFromGroups(blocks, n, genome, ref, ctx=ctx)
    reps = max(3, args.steps)
    ms = []
    launches0 = ctx.kernel_launches()
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dev_step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    launches = (ctx.kernel_launches() - launches0) / reps
    wall = []
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_lut = iu.buildIndexFromGroups(blocks, n, genome, ref, ctx=ctx)
        wall.append(time.perf_counter() - t0)
    dev_ms = sorted(ms)[len(ms) // 2]
    e2e_s = sorted(wall)[len(wall) // 2]
    same_paths = bool(np.array_equal(d_lut.cpu().numpy(), host_lut))
    # algorithmic bytes: both rows once, the LUT written once and read by each clean-up pass
    alg = 2.0 * ncols + 4.0 * n * 3
    return {
        "workload": "index LUT of a %.1f Mbp genome from %d aligned blocks (%d columns; 2%% substitutions, "
                    "0.05%% indels), fixZeroIdx + fillGaps(300) + smoothEdges(20)" % (n / 1e6, len(gs), ncols),
        "value": round(n / 1e6 / (dev_ms / 1e3), 2), "unit": "Mbp/s", "ms": round(dev_ms, 4),
        "e2e": {"value": round(n / 1e6 / e2e_s, 2), "unit": "Mbp/s", "ms": round(e2e_s * 1e3, 3),
                "h2d_bytes_per_step": int(2 * ncols + 16 * len(gs) + 8 + n + len(ref)),
                "d2h_bytes_per_step": int(4 * n)},
        "roofline": {"bound": "hbm", "achieved": round(alg / (dev_ms / 1e3) / 1e9, 2), "unit": "GB/s",
                     "algorithmic_bytes": alg, "note": "launch- and sync-bound at this size"},
        "gpu_launches_per_step": launches, "device_and_host_paths_identical": same_paths,
        "_host_lut": host_lut, "_inputs": (gs, rs, off, rg, rr, genome, ref),
    }


def cpu_lut(inputs):
    """The oracle's LUT path on one host thread (CPU baseline and check)."""
    import oracle as O
    gs, rs, off, rg, rr, genome, ref = inputs
    n = len(genome)
    lut = np.empty(n, np.int32)
    t0 = time.perf_counter()
    rc = O.lib().mo_lut_from_blocks(O._p(gs), O._p(rs), O._p(off), O._p(rg), O._p(rr), len(gs), O._p(lut), n)
    O.fix_zero_idx(lut, genome, ref)
    O.fill_gaps(lut, 300)
    O.smooth_edges(lut, 20)
    dt = time.perf_counter() - t0
    return rc, lut, dt


# ------------------------------------------------------------- arms

def run_reference(args, world, rank):
    if rank != 0:
        return 0
    import synth
    a, b = synth.genome_pair_recoded()
    seed, w = seeds_for(a, b)
    cpu_anchoring(a, b, seed, args.warmup)
    ts, m = cpu_anchoring(a, b, seed, args.steps)
    mbp = (len(a) + len(b)) / 1e6
    value = mbp * len(ts) / sum(ts)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mbp/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(ts) / len(ts), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/int64",
        "data": "synthetic (seeded numpy)",
        "config": {"workload": WORKLOAD, "matches": int(len(m))},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mbp/s", "cores": 1, "kind": "port",
                         "sample": "the full pair each step; CPU restatement of the reference (oracle/), "
                                   "single-threaded like the reference build"},
        "e2e": {"value": round(value, 4), "unit": "Mbp/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, world, rank, local):
    import torch

    import mvg
    import synth

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = mvg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    dev = torch.device("cuda", local)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def mor(x):
        return max_over_ranks(x, world, dev)

    line = {"metric": METRIC, "unit": "Mbp/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/int64",
            "data": "synthetic (seeded numpy)"}
    launches = 0

    if args.only in ("all", "anchor"):
        # ---- anchoring workload (weak scaling: each rank its own pair)
        if args.pair == "small":
            a, b = synth.genome_pair_small(seed=rank)
            workload = "plain-method pair: 1 Mbp i.i.d. GC 0.50, A = B + 0.5% subs, 50 indels, 2 x 10 kbp inversions"
        else:
            a, b = synth.genome_pair_recoded(seed=replica_pair_seed(rank))
            workload = WORKLOAD
        seed, w = seeds_for(a, b)
        na, nb = len(a), len(b)
        d_a = torch.from_numpy(a).to(dev)
        d_b = torch.from_numpy(b).to(dev)
        cap = 1 << 20
        d_out = torch.zeros(3 * cap, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()

        def step():
            return ctx.pairwise_matches_dev(d_a.data_ptr(), na, d_b.data_ptr(), nb, seed, d_out.data_ptr(), cap)

        for _ in range(args.warmup):
            nmatch = step()
        ctx.set_profiling(True)
        stage_tot = {}
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        sampler = ClockSampler(local)
        launches0 = ctx.kernel_launches()
        sampler.start()
        sampler.wait_first()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 255)  # evict L2 between steps (untimed)
            ev[k][0].record(stream)
            nmatch = step()
            ev[k][1].record(stream)
            for name, t in ctx.stage_times().items():
                stage_tot[name] = stage_tot.get(name, 0.0) + t
        torch.cuda.synchronize()
        launches += ctx.kernel_launches() - launches0
        tot_ms = mor(sum(e0.elapsed_time(e1) for e0, e1 in ev))
        if world > 1:
            torch.distributed.barrier()
        clocks_anchor = sampler.stop()
        ctx.set_profiling(False)
        value = world * args.steps * (na + nb) / 1e6 / (tot_ms / 1e3)

        # ---- e2e through the host-buffer C ABI (pinned inputs, copies inside)
        import ctypes
        pa = torch.from_numpy(a).pin_memory().numpy()
        pb = torch.from_numpy(b).pin_memory().numpy()
        host_out = torch.zeros(3 * cap, dtype=torch.int64).pin_memory().numpy()
        cnt = ctypes.c_uint64(0)
        L = mvg.load_library()

        def e2e_step():
            rc = L.mvg_pairwise_matches(ctx.handle, ctypes.c_void_p(pa.ctypes.data), na,
                                        ctypes.c_void_p(pb.ctypes.data), nb, seed,
                                        ctypes.c_void_p(host_out.ctypes.data), cap, ctypes.byref(cnt))
            mvg._check(rc)
            return int(cnt.value)

        for _ in range(max(1, args.warmup)):
            e2e_step()
        e2e_s = 0.0
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 255)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            n_e2e = e2e_step()
            e2e_s += time.perf_counter() - t0
        e2e_s = mor(e2e_s)
        assert n_e2e == nmatch
        e2e_value = world * args.steps * (na + nb) / 1e6 / e2e_s

        hbm_peak, peak_kind = peaks()
        P = (2 * w + 1 + 7) // 8
        per_base = 24.25 + 24 * P  # seed path bytes per base per genome
        seed_ms = sum(stage_tot.get(k, 0.0) for k in SEED_STAGES) / args.steps
        seed_bytes = per_base * (na + nb)
        stages = {k: round(v / args.steps, 4) for k, v in stage_tot.items()}
        step_ms = tot_ms / args.steps
        line.update({
            "value": round(value, 3), "value_scope": VALUE_SCOPE, "ms_per_step": round(step_ms, 4),
            "config": {"workload": workload, "bases": na + nb, "matches": int(nmatch), "seed_weight": w,
                       "l2": "flushed between timed steps (256 MiB device write, untimed)",
                       "parallelism": "replicas: one genome pair per GPU"},
            "roofline": {
                "bound": "hbm", "kernel": "seed path (pack + seed keys + LSD radix sort + unique join), both genomes",
                "achieved": round(seed_bytes / (seed_ms / 1e3) / 1e9, 2) if seed_ms else None,
                "peak": hbm_peak, "unit": "GB/s", "peak_kind": peak_kind,
                "frac": round(seed_bytes / (seed_ms / 1e3) / 1e9 / hbm_peak, 4) if seed_ms else None,
                "traffic": SEED_PATH_TRAFFIC if args.pair == "recoded" else None,
                "traffic_source": "ncu dram__bytes_read+write of the seed-path kernels per call "
                                  "(profiles/anchoring_launch_list_recoded_pair.md)",
                "algorithmic_bytes": seed_bytes, "bytes_per_base": per_base,
                "frac_whole_step": round(seed_bytes / (step_ms / 1e3) / 1e9 / hbm_peak, 4),
                "frac_whole_step_note": "the same per-base bytes over the whole anchoring step, including the "
                                        "latency-bound hashing, replay and emit stages",
                "stage_ms": stages, "dominant_stage": max(stages, key=stages.get) if stages else None},
            "e2e": {"value": round(e2e_value, 3), "unit": "Mbp/s", "h2d_bytes_per_step": na + nb,
                    "d2h_bytes_per_step": int(nmatch) * 24 + 12},
            "clocks": clocks_anchor,
        })

    if args.only in ("all", "anchor") and world == 1:
        line["reference_fixture_pair"] = mds42_section(ctx, dev, stream, flush)

    if args.only in ("all", "gapdp"):
        sa, oa, sb, ob = synth.gap_batch(seed=3 + rank, nprob=args.gap_nprob)
        oa = oa.astype(np.uint64)
        ob = ob.astype(np.uint64)
        n = len(oa) - 1
        cells = float(np.sum(np.diff(oa.astype(np.int64)) * np.diff(ob.astype(np.int64))))
        path_off = np.zeros(n + 1, np.uint64)
        path_off[1:] = np.cumsum(np.diff(oa.astype(np.int64)) + np.diff(ob.astype(np.int64)))
        d_sa = torch.from_numpy(sa).to(dev)
        d_sb = torch.from_numpy(sb).to(dev)
        d_oa = torch.from_numpy(oa.view(np.int64)).to(dev)
        d_ob = torch.from_numpy(ob.view(np.int64)).to(dev)
        d_po = torch.from_numpy(path_off.view(np.int64)).to(dev)
        d_sc = torch.zeros(n, dtype=torch.int32, device=dev)
        d_paths = torch.zeros(int(path_off[-1]) + 16, dtype=torch.uint8, device=dev)
        d_pl = torch.zeros(n, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()

        def dp_step():
            ctx.gap_align_batch_dev(d_sa.data_ptr(), d_oa.data_ptr(), d_sb.data_ptr(), d_ob.data_ptr(), n,
                                    d_sc.data_ptr(), d_paths.data_ptr(), d_po.data_ptr(), d_pl.data_ptr())

        dp_steps = max(1, min(args.steps, 2))
        for _ in range(1):  # the batch is ~5 s of GPU work: one warm-up pass
            dp_step()
        ctx.set_profiling(True)
        dp_stage = {}
        sampler = ClockSampler(local)
        launches0 = ctx.kernel_launches()
        sampler.start()
        dp_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(dp_steps)]
        for k in range(dp_steps):
            dp_ev[k][0].record(stream)
            dp_step()
            dp_ev[k][1].record(stream)
            for name, t in ctx.stage_times().items():
                dp_stage[name] = dp_stage.get(name, 0.0) + t
        torch.cuda.synchronize()
        launches += ctx.kernel_launches() - launches0
        clocks_dp = sampler.stop()
        ctx.set_profiling(False)
        dp_ms = mor(sum(e0.elapsed_time(e1) for e0, e1 in dp_ev) / dp_steps)
        gcups = world * cells / (dp_ms / 1e3) / 1e9
        int32_peak = ctx.probe_int32_peak()
        dp_kernel_ms = dp_stage.get("dp", 0.0) / dp_steps
        dp_achieved = cells * OPS_PER_CELL / (dp_kernel_ms / 1e3) if dp_kernel_ms else 0.0
        line["gap_dp"] = {
            "workload": GAP_WORKLOAD if args.gap_nprob == GAP_NPROB else "%d pairs from the same distribution"
                                                                          % args.gap_nprob,
            "gcups": round(gcups, 2), "cells": cells, "ms_per_batch": round(dp_ms, 3),
            "stage_ms": {k: round(v / dp_steps, 3) for k, v in dp_stage.items()},
            "roofline": {"bound": "int32-alu", "achieved": round(dp_achieved / 1e12, 3), "unit": "Tops/s",
                         "peak": round(int32_peak / 1e12, 3), "peak_kind": "measured (INT32 add/max probe)",
                         "frac": round(dp_achieved / int32_peak, 4) if int32_peak else None,
                         "ops_per_cell": OPS_PER_CELL},
            "clocks": clocks_dp,
        }
        line["gap_dp"].update(gapdp_checks(ctx, sa, oa, sb, ob, d_sc, d_paths, d_po, d_pl, dev, rank))
        if args.only == "gapdp":
            line.update({"value": round(gcups, 2), "unit": "GCUPS", "ms_per_step": round(dp_ms, 3)})
        lb_section = None if args.no_learned_band else learned_band_section(ctx, args, dev, stream, rank)
        if lb_section:
            line["gap_dp"]["learned_band"] = lb_section

    if args.only in ("all", "gapsearch"):
        line["gap_search"] = gap_search_section(ctx, dev, rank)
        if args.only == "gapsearch":
            gs = line["gap_search"]
            line.update({"value": gs["value"], "unit": gs["unit"], "ms_per_step": gs["ms"]})

    if args.only in ("all", "outside"):
        line["outside_lcbs"] = outside_lcbs_section(ctx, dev, rank)
        if args.only == "outside":
            ol = line["outside_lcbs"]
            line.update({"value": ol["value"], "unit": ol["unit"], "ms_per_step": ol["ms"]})
    if args.only in ("all", "refine"):
        line["refinement"] = refinement_section(ctx, rank)
        if args.only == "refine":
            rf = line["refinement"]
            line.update({"value": rf["value"], "unit": rf["unit"]})

    if args.only in ("all", "backbone"):
        line["backbone_detection"] = backbone_section(rank)
        if args.only == "backbone":
            bb = line["backbone_detection"]
            line.update({"value": bb["value"], "unit": bb["unit"], "ms_per_step": bb["ms"]})

    if args.only in ("all", "xmfa"):
        line["xmfa_writer"] = xmfa_section(ctx, dev, rank, flush)
        if args.only == "xmfa":
            xw = line["xmfa_writer"]
            line.update({"value": xw["value"], "unit": xw["unit"], "ms_per_step": xw["ms"]})

    if args.only in ("all", "lcbs"):
        line["collinear_lcbs"] = collinear_lcbs_section(rank)
        if args.only == "lcbs":
            cl = line["collinear_lcbs"]
            line.update({"value": cl["value"], "unit": cl["unit"], "ms_per_step": cl["ms"]})

    lut_sec = None
    if args.only in ("all", "lut"):
        lut_sec = lut_section(ctx, args, dev, stream, rank, flush)
        launches += int(lut_sec["gpu_launches_per_step"])
        line["index_lut"] = {k: v for k, v in lut_sec.items() if not k.startswith("_")}
        if args.only == "lut":
            line.update({"value": lut_sec["value"], "unit": "Mbp/s", "ms_per_step": lut_sec["ms"]})

    line["gpu_launches"] = int(launches)
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        ctx.close()
        return 0
    if world == 1 and not args.skip_cpu_baseline:
        import multiprocessing
        if args.only in ("all", "anchor"):
            ts, _ = cpu_anchoring(a, b, seed, 1)
            line["cpu_baseline"] = {"value": round((na + nb) / 1e6 / ts[0], 4), "unit": "Mbp/s", "cores": 1,
                                    "kind": "port",
                                    "sample": "the full pair once (oracle restatement, one thread)"}
        if lut_sec is not None:
            rc, cl, dt = cpu_lut(lut_sec["_inputs"])
            line["index_lut"]["cpu_baseline"] = {
                "value": round(len(cl) / 1e6 / dt, 2), "unit": "Mbp/s", "cores": 1, "kind": "port",
                "sample": "the same alignment once (oracle restatement of buildindex.py:112-137, one thread)"}
            line["index_lut"]["identical_to_oracle"] = bool(rc == 0 and np.array_equal(cl, lut_sec["_host_lut"]))
        if args.only in ("all", "gapdp"):
            threads = multiprocessing.cpu_count()
            cg, ccells, cdt = cpu_gapdp_gcups(sa, oa, sb, ob, 400, threads)
            line["gap_dp"]["cpu_baseline"] = {"gcups": round(cg, 4), "cores": threads, "kind": "port",
                                              "sample": "400 pairs spread over the length distribution, %.3g cells"
                                                        % ccells}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu-baseline", action="store_true")
    ap.add_argument("--only", choices=["all", "anchor", "gapdp", "gapsearch", "outside", "refine", "backbone", "lcbs",
                                         "xmfa", "lut"],
                    default="all",
                    help="run one half only (small cases for profiler captures)")
    ap.add_argument("--pair", choices=["recoded", "small"], default="recoded",
                    help="genome pair: recoded 4.6 Mbp (default) or the 1 Mbp plain-method pair")
    ap.add_argument("--gap-nprob", type=int, default=GAP_NPROB)
    ap.add_argument("--no-learned-band", action="store_true", help="skip the learned-band section (profiling)")
    ap.add_argument("--lb-nprob", type=int, default=LB_NPROB, help="gaps in the learned-band section")
    args = ap.parse_args()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        return run_reference(args, world, rank)
    import build as pkg_build
    pkg_build.build()
    return run_gb300(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
