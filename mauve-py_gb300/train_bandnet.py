#!/usr/bin/env python3
"""Trains the band-proposal network on the GPU and evaluates it.

    python mauve-py_gb300/train_bandnet.py [--train 1000000 --eval 200000]
                                           [--out mauve-py_gb300/bandnet_weights.npz]

1. Draws training and held-out gaps like the recoded-genome pair's
   (tests/synth.py gap_batch_recoded).
2. Labels them with the exact full DP (mvg_gapdp_envelope_dev): optimal
   score and path envelope -> band offset and the half-width the exactness
   check needs.
3. Trains with the library's own forward/backward/Adam kernels.
4. Calibrates the half-width margin (alpha, beta), the whole-matrix share
   and the divergence gate by timing the exact banded DP with its fallbacks
   on a separate draw of calibration gaps.
5. Evaluates on the held-out gaps: plain full DP vs learned band vs the band
   without the network, all with identical output (checked), and writes the
   weights, calibration and metrics.
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


class DeviceBatch:
    """Gap batch resident on the GPU (torch tensors for memory, raw pointers for the C ABI)."""

    def __init__(self, sa, oa, sb, ob, dev):
        import torch
        self.n = len(oa) - 1
        self.la = np.diff(oa).astype(np.int64)
        self.lb = np.diff(ob).astype(np.int64)
        self.oa, self.ob = oa.astype(np.uint64), ob.astype(np.uint64)
        self.sa = torch.from_numpy(sa).to(dev)
        self.sb = torch.from_numpy(sb).to(dev)
        self.doa = torch.from_numpy(self.oa.view(np.int64)).to(dev)
        self.dob = torch.from_numpy(self.ob.view(np.int64)).to(dev)
        self.cells = float(np.sum(self.la * self.lb))

    def ptrs(self):
        return self.sa.data_ptr(), self.doa.data_ptr(), self.sb.data_ptr(), self.dob.data_ptr()


def subset(sa, oa, sb, ob, idx):
    a = [sa[oa[k]:oa[k + 1]] for k in idx]
    b = [sb[ob[k]:ob[k + 1]] for k in idx]
    noa = np.concatenate([[0], np.cumsum([len(x) for x in a])]).astype(np.int64)
    nob = np.concatenate([[0], np.cumsum([len(x) for x in b])]).astype(np.int64)
    return np.concatenate(a), noa, np.concatenate(b), nob


def label(ctx, batch, chunk=100_000):
    scores = np.zeros(batch.n, np.int32)
    env = np.zeros((batch.n, 2), np.int32)
    for s in range(0, batch.n, chunk):
        e = min(batch.n, s + chunk)
        sub = DeviceBatch(*subset_host(batch, s, e), batch.sa.device)
        sc, en = bandnet.full_dp_labels_dev(ctx, *sub.ptrs(), sub.n, torch_device=batch.sa.device)
        scores[s:e] = sc
        env[s:e] = en
    return scores, env


def label_band_rejections(ctx, batch, delta, half, chunk=100_000):
    """Bool per gap: the banded DP with its label band fails the check."""
    import torch
    rej = np.zeros(batch.n, bool)
    for s in range(0, batch.n, chunk):
        e = min(batch.n, s + chunk)
        sub = DeviceBatch(*subset_host(batch, s, e), batch.sa.device)
        path_off = np.zeros(sub.n + 1, np.uint64)
        path_off[1:] = np.cumsum(sub.la + sub.lb)
        d_po = torch.from_numpy(path_off.view(np.int64)).to(batch.sa.device)
        d_paths = torch.zeros(int(path_off[-1]) + 16, dtype=torch.uint8, device=batch.sa.device)
        d_pl = torch.zeros(sub.n, dtype=torch.int64, device=batch.sa.device)
        d_sc = torch.zeros(sub.n, dtype=torch.int32, device=batch.sa.device)
        status, _ = ctx.gap_align_banded_dev(*sub.ptrs(), sub.n, delta[s:e], half[s:e], d_sc.data_ptr(),
                                             d_paths.data_ptr(), d_po.data_ptr(), d_pl.data_ptr())
        rej[s:e] = status == 0
    return rej


def subset_host(batch, s, e):
    sa = batch.sa[int(batch.oa[s]):int(batch.oa[e])].cpu().numpy()
    sb = batch.sb[int(batch.ob[s]):int(batch.ob[e])].cpu().numpy()
    oa = (batch.oa[s:e + 1] - batch.oa[s]).astype(np.int64)
    ob = (batch.ob[s:e + 1] - batch.ob[s]).astype(np.int64)
    return sa, oa, sb, ob


def subset_host_idx(batch, idx):
    sa = batch.sa.cpu().numpy()
    sb = batch.sb.cpu().numpy()
    return subset(sa, batch.oa.astype(np.int64), sb, batch.ob.astype(np.int64), idx)


def status_rates(status):
    """Shares of banded results kept (1), rejected by the check (0) and not
    tried (2); fallback = everything that ran the full DP."""
    return {"accept_rate": float((status == 1).mean()), "rejected_rate": float((status == 0).mean()),
            "not_tried_rate": float((status == 2).mean()), "fallback_rate": float((status != 1).mean())}


def timed_banded(ctx, batch, delta, half):
    """(seconds, used-band flags, cells) of the banded DP with fallback, paths on device."""
    import torch
    n = batch.n
    path_off = np.zeros(n + 1, np.uint64)
    path_off[1:] = np.cumsum(batch.la + batch.lb)
    d_po = torch.from_numpy(path_off.view(np.int64)).to(batch.sa.device)
    d_paths = torch.zeros(int(path_off[-1]) + 16, dtype=torch.uint8, device=batch.sa.device)
    d_pl = torch.zeros(n, dtype=torch.int64, device=batch.sa.device)
    d_sc = torch.zeros(n, dtype=torch.int32, device=batch.sa.device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    used, cells = ctx.gap_align_banded_dev(*batch.ptrs(), n, delta, half, d_sc.data_ptr(), d_paths.data_ptr(),
                                           d_po.data_ptr(), d_pl.data_ptr())
    torch.cuda.synchronize()
    return time.perf_counter() - t0, used, cells, d_sc, d_paths, d_pl, path_off


def timed_full(ctx, batch):
    import torch
    n = batch.n
    path_off = np.zeros(n + 1, np.uint64)
    path_off[1:] = np.cumsum(batch.la + batch.lb)
    d_po = torch.from_numpy(path_off.view(np.int64)).to(batch.sa.device)
    d_paths = torch.zeros(int(path_off[-1]) + 16, dtype=torch.uint8, device=batch.sa.device)
    d_pl = torch.zeros(n, dtype=torch.int64, device=batch.sa.device)
    d_sc = torch.zeros(n, dtype=torch.int32, device=batch.sa.device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.gap_align_batch_dev(*batch.ptrs(), n, d_sc.data_ptr(), d_paths.data_ptr(), d_po.data_ptr(), d_pl.data_ptr())
    torch.cuda.synchronize()
    return time.perf_counter() - t0, d_sc, d_paths, d_pl


def band_cells(la, lb, delta, half, srows):
    """Host copy of the band geometry's cell count (same formula as band.h)."""
    tot = 0
    for a, b, d, h in zip(la, lb, delta, half):
        ns = (a + srows - 1) // srows
        for k in range(ns):
            lo = 1 if k == 0 else min(max((k * srows + 1) * b // a + d - h, 1), b)
            last = min((k + 1) * srows, a)
            hi = b if k == ns - 1 else min(max(last * b // a + d + h + 1, 1), b)
            tot += (min(srows, a - k * srows)) * (hi - lo + 1)
    return tot


def train(args):
    import torch
    import synth
    dev = torch.device("cuda", 0)
    ctx = mvg.Context(0)
    t_all = time.time()
    n_tr, n_ev = args.train, args.eval
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=args.seed, nprob=n_tr + n_ev)
    tot_a, tot_b = bandnet.best_totals(sa, oa), bandnet.best_totals(sb, ob)
    tr = DeviceBatch(*subset(sa, oa, sb, ob, np.arange(n_tr)), dev)
    ev = DeviceBatch(*subset(sa, oa, sb, ob, np.arange(n_tr, n_tr + n_ev)), dev)
    del sa, sb
    print("data", tr.n, ev.n, "%.1fs" % (time.time() - t_all), flush=True)
    if args.calibrate_only:
        return calibrate_and_evaluate(args, ctx, dev, bandnet.BandNet(ctx, params=np.load(args.calibrate_only)["params"]),
                                      tr, ev, tot_a, tot_b, n_tr, [], 0, 0, 0.0, t_all)
    t0 = time.time()
    sc_tr, env_tr = label(ctx, tr)
    print("labels %.1fs (%.3g cells)" % (time.time() - t0, tr.cells), flush=True)
    T, d_lab_tr, h_lab_tr = bandnet.labels_from_full_dp(tr.la, tr.lb, sc_tr, env_tr, margin=args.margin,
                                                         totals=(tot_a[:n_tr], tot_b[:n_tr]))
    # gaps whose label band the exactness check still rejects are labelled
    # "whole matrix": proposing their band would only add a rerun
    t0 = time.time()
    rej = label_band_rejections(ctx, tr, d_lab_tr, h_lab_tr)
    T[rej, 1] = np.log1p(np.maximum(tr.la[rej], tr.lb[rej])).astype(np.float32)
    print("label bands rejected by the check: %d of %d (%.1fs)" % (int(rej.sum()), tr.n, time.time() - t0),
          flush=True)
    if not np.isfinite(T).all():
        raise RuntimeError("non-finite training targets")
    print("targets: |offset| max %.2f, log-half range %.2f..%.2f" % (np.abs(T[:, 0]).max(), T[:, 1].min(),
                                                                      T[:, 1].max()), flush=True)
    X = torch.zeros((tr.n, bandnet.N_IN), dtype=torch.bfloat16, device=dev)
    net = bandnet.BandNet(ctx, seed=args.seed)
    net.features_dev(*tr.ptrs(), tr.n, X.data_ptr())
    Tg = torch.from_numpy(T).to(dev)
    fit_idx = np.random.default_rng(args.seed).permutation(tr.n)
    fit_idx_t = torch.from_numpy(fit_idx).to(dev)
    # minibatches drawn with probability ~ cells^w: the gaps that carry the
    # DP's cells weigh more in the fit (w = 0: uniform)
    wts = torch.from_numpy((tr.la[fit_idx].astype(np.float64) * tr.lb[fit_idx]) ** args.cell_weight).to(dev)
    t0 = time.time()
    losses = []
    step = 0
    skipped = 0
    for ep in range(args.epochs):
        if args.cell_weight > 0:
            order = fit_idx_t[torch.multinomial(wts, len(fit_idx_t), replacement=True)]
        else:
            order = fit_idx_t[torch.randperm(len(fit_idx_t), device=dev)]
        lr = args.lr * (args.lr_decay ** ep)
        for s in range(0, len(order), args.batch):
            idx = order[s:s + args.batch]
            xb = X.index_select(0, idx).contiguous()
            tb = Tg.index_select(0, idx).contiguous()
            loss = net.train_step_dev(xb.data_ptr(), tb.data_ptr(), len(idx), lr)
            step += 1
            if not np.isfinite(loss):
                skipped += 1
                if skipped == 1:
                    out = torch.zeros((len(idx), 2), dtype=torch.float32, device=dev)
                    net.forward_dev(xb.data_ptr(), len(idx), out.data_ptr())
                    print("first non-finite minibatch at step %d: n %d, X finite %s, T finite %s, |T| max %.3g, "
                          "output finite %s, |output| max %.3g, params finite %s" % (
                              step, len(idx), bool(torch.isfinite(xb.float()).all()), bool(torch.isfinite(tb).all()),
                              float(tb.abs().max()), bool(torch.isfinite(out).all()),
                              float(out.abs().nan_to_num(0).max()), bool(np.isfinite(net.get_params()).all())),
                          flush=True)
            if step % 50 == 0:
                losses.append((step, loss))
        print("epoch %d loss %.4f (non-finite minibatches so far: %d)" % (
            ep, losses[-1][1] if losses else float("nan"), skipped), flush=True)
    train_s = time.time() - t0
    return calibrate_and_evaluate(args, ctx, dev, net, tr, ev, tot_a, tot_b, n_tr, losses, step, skipped, train_s, t_all)


def calibrate_and_evaluate(args, ctx, dev, net, tr, ev, tot_a, tot_b, n_tr, losses, step, skipped, train_s, t_all):
    import torch
    # calibrate alpha / beta on a separate draw of calibration gaps, as many
    # as a production batch, by timing the exact banded DP (with its
    # fallbacks) for each candidate margin (the faster of two runs)
    import synth
    vb = DeviceBatch(*synth.gap_batch_recoded(seed=args.seed + 7, nprob=args.calib), dev)
    best = None
    for gate in (0, 18, 20, 22, 24):
        ctx.set_band_gate(gate)
        for whole in (0.25, 0.3, 0.35, 0.45):
            ctx.set_band_whole_fraction(whole)
            for alpha in (1.15, 1.45, 1.6, 1.8, 2.0, 2.3):
                for beta in (0.0, 8.0, 16.0, 32.0):
                    d, h = net.propose_dev(*vb.ptrs(), vb.n, alpha, beta)
                    runs = [timed_banded(ctx, vb, d, h)[:3] for _ in range(2)]
                    secs, used, cells = min(runs, key=lambda r: r[0])
                    if best is None or secs < best[0]:
                        best = (secs, alpha, beta, whole, gate, float((used == 1).mean()), cells)
    _, alpha, beta, whole, gate, acc_v, _ = best
    ctx.set_band_whole_fraction(whole)
    ctx.set_band_gate(gate)
    print("calibrated alpha %.2f beta %.1f whole %.2f gate %d (validation accept %.3f)" % (alpha, beta, whole, gate,
                                                                                           acc_v), flush=True)
    params = net.get_params()
    # held-out evaluation: full vs learned band vs band without the network
    res = {"train_gaps": tr.n, "eval_gaps": ev.n, "train_seconds": train_s, "steps": step,
           "loss_curve": losses[-20:], "nonfinite_minibatches": skipped, "alpha": alpha, "beta": beta,
           "whole_fraction": whole, "divergence_gate": gate}
    tf, sc_f, p_f, pl_f = timed_full(ctx, ev)
    tf, sc_f, p_f, pl_f = timed_full(ctx, ev)  # second run: warm
    t_prop0 = time.perf_counter()
    dl, hl = net.propose_dev(*ev.ptrs(), ev.n, alpha, beta)
    torch.cuda.synchronize()
    t_prop = time.perf_counter() - t_prop0
    tl, used_l, cells_l, sc_l, p_l, pl_l, _ = timed_banded(ctx, ev, dl, hl)
    dh, hh = bandnet.heuristic_band(ev.la, ev.lb)
    th, used_h, cells_h, sc_h, p_h, pl_h, _ = timed_banded(ctx, ev, dh, hh)
    same_l = bool(torch.equal(sc_f, sc_l) and torch.equal(pl_f, pl_l) and torch.equal(p_f, p_l))
    same_h = bool(torch.equal(sc_f, sc_h) and torch.equal(pl_f, pl_h) and torch.equal(p_f, p_h))
    res.update({
        "eval_cells_full": ev.cells,
        "full": {"seconds": tf, "gcups": ev.cells / tf / 1e9},
        "learned": {"seconds": tl + t_prop, "dp_seconds": tl, "propose_seconds": t_prop,
                    "effective_gcups": ev.cells / (tl + t_prop) / 1e9, **status_rates(used_l), "cells": cells_l,
                    "identical_to_full": same_l},
        "no_network": {"seconds": th, "effective_gcups": ev.cells / th / 1e9, **status_rates(used_h),
                       "cells": cells_h, "identical_to_full": same_h},
    })
    res["speedup_learned_vs_full"] = tf / (tl + t_prop)
    res["speedup_no_network_vs_full"] = tf / th
    # where the banded time goes: the accepted gaps' banded DP alone, and the
    # full-DP cells of the gaps that fell back; plus the ceiling set by the
    # label bands (the full DP's own envelope + margin) on the same gaps
    gcups_full = ev.cells / tf / 1e9
    for key, (d, h, used) in (("learned", (dl, hl, used_l)), ("no_network", (dh, hh, used_h))):
        acc = np.nonzero(used == 1)[0]
        fb = np.nonzero(used != 1)[0]
        if len(acc) == 0:
            continue
        sub = DeviceBatch(*subset_host_idx(ev, acc), dev)
        ta, _, cells_a, *_ = timed_banded(ctx, sub, d[acc], h[acc])
        fb_cells = float(np.sum(ev.la[fb].astype(np.float64) * ev.lb[fb]))
        res[key].update({"accepted_band_seconds": ta, "accepted_band_cells": cells_a,
                         "accepted_band_gcups": cells_a / ta / 1e9 if ta > 0 else None,
                         "accepted_full_cells": float(np.sum(ev.la[acc].astype(np.float64) * ev.lb[acc])),
                         "fallback_full_cells": fb_cells,
                         "fallback_seconds_at_full_gcups": fb_cells / gcups_full / 1e9})
        del sub
    env = bandnet.full_dp_labels_dev(ctx, *ev.ptrs(), ev.n, torch_device=dev)
    _, d_lab, h_lab = bandnet.labels_from_full_dp(ev.la, ev.lb, *env, margin=args.margin,
                                                  totals=(tot_a[n_tr:], tot_b[n_tr:]))
    t_lab, used_lab, cells_lab, *_ = timed_banded(ctx, ev, d_lab, h_lab)
    res["label_band"] = {"seconds": t_lab, **status_rates(used_lab), "cells": cells_lab,
                         "speedup_vs_full": tf / t_lab}
    print(json.dumps(res, indent=1), flush=True)
    np.savez(args.out, params=params, alpha=np.float32(alpha), beta=np.float32(beta), whole=np.float32(whole),
             gate=np.int32(gate))
    with open(os.path.splitext(args.out)[0] + "_eval.json", "w") as f:
        json.dump(res, f, indent=1)
    print("total %.1fs" % (time.time() - t_all))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=1_000_000)
    ap.add_argument("--eval", type=int, default=200_000)
    ap.add_argument("--calib", type=int, default=200_000, help="gaps timed to calibrate the margins")
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--lr-decay", type=float, default=0.75, help="learning-rate factor per epoch")
    ap.add_argument("--margin", type=int, default=24, help="columns added to each label half-width")
    ap.add_argument("--cell-weight", type=float, default=0.5,
                    help="minibatch sampling probability ~ (LA*LB)^w")
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--out", default=os.path.join(HERE, "bandnet_weights.npz"))
    ap.add_argument("--calibrate-only", default="",
                    help="weights file whose network is kept: only recalibrate the margins and evaluate")
    train(ap.parse_args())


if __name__ == "__main__":
    main()
