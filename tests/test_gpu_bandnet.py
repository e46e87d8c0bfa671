"""GPU tests of the banded gap DP and the band-proposal network."""
import numpy as np
import pytest

import bandnet
import bandnet_ref as REF
import mvg
import oracle as O
import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


def _dev(arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _batch_ptrs(sa, oa, sb, ob):
    t = _dev([sa, oa.astype(np.int64), sb, ob.astype(np.int64)])
    return t, [x.data_ptr() for x in t]


@pytest.mark.parametrize("rows,band_rows", [(4, 1), (4, 2), (8, 4), (8, 8)])
def test_banded_output_identical_to_full(ctx, rows, band_rows):
    ctx.set_dp_rows(rows, band_rows)
    try:
        rng = np.random.default_rng(rows)
        sa, oa, sb, ob = synth.gap_batch_recoded(seed=11, nprob=300, lmin=1, lmax=1500)
        n = len(oa) - 1
        la, lb = np.diff(oa), np.diff(ob)
        s_full, p_full = ctx.gap_align_batch(sa, oa, sb, ob)
        for delta, half in [bandnet.heuristic_band(la, lb),
                            (rng.integers(-40, 40, n).astype(np.int32), rng.integers(0, 60, n).astype(np.int32)),
                            (np.zeros(n, np.int32), np.zeros(n, np.int32))]:
            s, p, used, cells = ctx.gap_align_banded(sa, oa, sb, ob, delta, half)
            np.testing.assert_array_equal(s, s_full)
            assert p == p_full
        oscores, _, _, _ = O.nw_batch(sa, oa, sb, ob, with_paths=False)
        np.testing.assert_array_equal(s_full, oscores)
    finally:
        ctx.set_dp_rows(8, 4)


def test_band_with_label_width_is_accepted_on_close_gaps(ctx):
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=12, nprob=400, lmin=50, lmax=3000, unrelated=0.0)
    la, lb = np.diff(oa), np.diff(ob)
    t, ptrs = _batch_ptrs(sa, oa, sb, ob)
    scores, env = bandnet.full_dp_labels_dev(ctx, *ptrs, len(la), torch_device=t[0].device)
    totals = (bandnet.best_totals(sa, oa), bandnet.best_totals(sb, ob))
    _, delta, half = bandnet.labels_from_full_dp(la, lb, scores, env, margin=16, totals=totals)
    s, p, used, cells = ctx.gap_align_banded(sa, oa, sb, ob, delta, half, with_paths=False)
    np.testing.assert_array_equal(s, scores)
    tried = used != 2
    assert tried.sum() > 100
    # the label width must pass the exactness check
    assert (used[tried] == 1).mean() > 0.9
    assert cells < 0.5 * float(np.sum(la * lb))


def test_envelope_matches_oracle_paths(ctx):
    sa, oa, sb, ob = synth.gap_batch(seed=13, nprob=50, lmin=1, lmax=800)
    t, ptrs = _batch_ptrs(sa, oa, sb, ob)
    scores, env = bandnet.full_dp_labels_dev(ctx, *ptrs, 50, torch_device=t[0].device)
    for k in range(50):
        a, b = sa[oa[k]:oa[k + 1]], sb[ob[k]:ob[k + 1]]
        path, sc = O.nw_align(a, b)
        assert sc == scores[k]
        i = j = 0
        devs = []
        for e in path:
            i += e != "I"
            j += e != "D"
            if i >= 1:
                devs.append(j - (i * len(b)) // len(a))
        assert (min(devs), max(devs)) == tuple(env[k]), k


def test_features_match_reference(ctx):
    import torch
    sa, oa, sb, ob = synth.gap_batch(seed=14, nprob=40, lmin=1, lmax=400)
    t, ptrs = _batch_ptrs(sa, oa, sb, ob)
    X = torch.zeros((40, bandnet.N_IN), dtype=torch.bfloat16, device=t[0].device)
    net = bandnet.BandNet(ctx)
    net.features_dev(*ptrs, 40, X.data_ptr())
    ref = REF.features(sa, oa, sb, ob)
    np.testing.assert_allclose(X.float().cpu().numpy(), ref, rtol=1e-2, atol=1e-3)


def test_mlp_gradients_match_cpu_oracle(ctx):
    """Loss and every parameter block's gradient against the float64 CPU
    reference (same bf16 roundings); tolerance 2e-2 relative in norm."""
    import torch
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=15, nprob=96, lmin=20, lmax=600)
    t, ptrs = _batch_ptrs(sa, oa, sb, ob)
    net = bandnet.BandNet(ctx, seed=3)
    n = 96
    X = torch.zeros((n, bandnet.N_IN), dtype=torch.bfloat16, device=t[0].device)
    net.features_dev(*ptrs, n, X.data_ptr())
    rng = np.random.default_rng(0)
    T = rng.normal(0, 1, (n, 2)).astype(np.float32)
    g, loss = net.grad_dev(X.data_ptr(), torch.from_numpy(T).cuda().data_ptr(), n)
    Xh = X.float().cpu().numpy().astype(np.float64)
    rloss, rg = REF.loss_and_grads(net.get_params(), Xh, T.astype(np.float64))
    assert abs(loss - rloss) <= 2e-2 * abs(rloss) + 1e-6
    sizes = [256 * 528, 256, 256 * 256, 256, 256 * 256, 256, 2 * 256, 2]
    off = 0
    for s in sizes:
        a, b = g[off:off + s], rg[off:off + s]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-7, (off, s)
        off += s
    # forward agrees too
    out = torch.zeros((n, 2), dtype=torch.float32, device=t[0].device)
    net.forward_dev(X.data_ptr(), n, out.data_ptr())
    np.testing.assert_allclose(out.cpu().numpy(), REF.forward(net.get_params(), Xh), rtol=2e-2, atol=2e-2)


def test_training_reduces_loss(ctx):
    import torch
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=16, nprob=3000, lmin=20, lmax=2000)
    la, lb = np.diff(oa), np.diff(ob)
    t, ptrs = _batch_ptrs(sa, oa, sb, ob)
    scores, env = bandnet.full_dp_labels_dev(ctx, *ptrs, len(la), torch_device=t[0].device)
    T, _, _ = bandnet.labels_from_full_dp(la, lb, scores, env)
    n = len(la)
    X = torch.zeros((n, bandnet.N_IN), dtype=torch.bfloat16, device=t[0].device)
    net = bandnet.BandNet(ctx, seed=1)
    net.features_dev(*ptrs, n, X.data_ptr())
    Tg = torch.from_numpy(T).cuda()
    first = net.train_step_dev(X.data_ptr(), Tg.data_ptr(), n, 1e-3)
    for _ in range(150):
        last = net.train_step_dev(X.data_ptr(), Tg.data_ptr(), n, 1e-3)
    assert last < 0.5 * first


def gate_share_ref(sa, oa, sb, ob, min_match):
    """numpy mirror of the proposal's divergence gate (k_band_gate)."""
    out = np.ones(len(oa) - 1)
    for p in range(len(oa) - 1):
        A = sa[oa[p]:oa[p + 1]].astype(np.int64) & 3
        B = sb[ob[p]:ob[p + 1]].astype(np.int64) & 3
        la, lb = len(A), len(B)
        nwin = 0 if la < 32 else min(8, la // 32)
        if nwin == 0:
            continue
        good = 0
        for k in range(nwin):
            i0 = 0 if nwin == 1 else k * (la - 32) // (nwin - 1)
            i = np.arange(i0, i0 + 32)
            j = i * lb // la
            best = 0
            for o in range(-8, 9):
                jj = j + o
                ok = (jj >= 0) & (jj < lb)
                m = np.zeros(32, bool)
                m[ok] = B[jj[ok]] == A[i[ok]]
                best = max(best, int(m.sum()))
            good += best >= min_match
        out[p] = good / nwin
    return out


def test_divergence_gate_matches_reference_and_sends_divergent_gaps_whole(ctx):
    import os
    weights = os.path.join(os.path.dirname(bandnet.__file__), "bandnet_weights.npz")
    w = np.load(weights)
    net = bandnet.BandNet(ctx, params=w["params"])
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=41, nprob=400, lmin=10, lmax=3000, unrelated=0.5)
    t, ptrs = _batch_ptrs(sa, oa, sb, ob)
    n = len(oa) - 1
    ctx.set_band_gate(0)
    _, h_off = net.propose_dev(*ptrs, n, 1.0, 0.0)
    ctx.set_band_gate(26)
    try:
        _, h_on = net.propose_dev(*ptrs, n, 1.0, 0.0)
    finally:
        ctx.set_band_gate(0)
    share = gate_share_ref(sa, oa, sb, ob, 26)
    gated = share < 0.5
    np.testing.assert_array_equal(h_on[gated], 1000000)
    np.testing.assert_array_equal(h_on[~gated], h_off[~gated])
    # the gate picks out the divergent gaps: score deficit per base far above
    # that of the closely related ones
    scores, _ = ctx.gap_align_batch(sa, oa, sb, ob, with_paths=False)
    la, lb = np.diff(oa), np.diff(ob)
    best = np.minimum(bandnet.best_totals(sa, oa), bandnet.best_totals(sb, ob))
    rate = (best - scores) / np.minimum(la, lb)
    big = la >= 256
    assert gated[big & (rate > 40)].mean() > 0.9
    assert gated[big & (rate < 10)].mean() < 0.05


def test_trained_network_beats_the_band_without_it(ctx):
    """What the trained network gains over the method without it: on 60,000
    gaps drawn like the recoded-genome pair's (a seed no training or
    calibration draw used), the network's bands and the heuristic band
    (bandnet.heuristic_band: centred, |LA - LB| + 10% + 32) both give output
    identical to the full DP, and the network's run computes at least 20%
    fewer DP cells (banded cells plus the full-DP reruns) and takes less
    time than the heuristic's."""
    import os
    import time

    import torch
    wpath = os.path.join(os.path.dirname(mvg.__file__), "bandnet_weights.npz")
    w = np.load(wpath)
    net = bandnet.BandNet(ctx, params=w["params"])
    alpha, beta = float(w["alpha"]), float(w["beta"])
    ctx.set_band_whole_fraction(float(w["whole"]))
    ctx.set_band_gate(int(w["gate"]))
    try:
        sa, oa, sb, ob = synth.gap_batch_recoded(seed=2026, nprob=60_000)
        n = len(oa) - 1
        la, lb = np.diff(oa), np.diff(ob)
        path_off = np.zeros(n + 1, np.uint64)
        path_off[1:] = np.cumsum(la + lb)
        t, ptrs = _batch_ptrs(sa, oa, sb, ob)
        d_poff = torch.from_numpy(path_off.view(np.int64)).cuda()

        def outputs():
            return (torch.zeros(n, dtype=torch.int32, device="cuda"),
                    torch.zeros(int(path_off[-1]) + 16, dtype=torch.uint8, device="cuda"),
                    torch.zeros(n, dtype=torch.int64, device="cuda"))

        full = outputs()
        ctx.gap_align_batch_dev(*ptrs, n, full[0].data_ptr(), full[1].data_ptr(), d_poff.data_ptr(),
                                full[2].data_ptr())

        def run(propose):
            best = None
            for _ in range(3):
                out = outputs()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                d, h = propose()
                used, cells = ctx.gap_align_banded_dev(*ptrs, n, d, h, out[0].data_ptr(), out[1].data_ptr(),
                                                       d_poff.data_ptr(), out[2].data_ptr())
                torch.cuda.synchronize()
                dt = time.perf_counter() - t0
                assert all(bool(torch.equal(x, y)) for x, y in zip(out, full))
                best = (dt, used, cells) if best is None or dt < best[0] else best
            return best

        t_net, used_net, cells_net = run(lambda: net.propose_dev(*ptrs, n, alpha, beta))
        t_heu, used_heu, cells_heu = run(lambda: bandnet.heuristic_band(la, lb))
    finally:
        ctx.set_band_whole_fraction(0.5)
        ctx.set_band_gate(0)
    msg = "network %.1f ms, %.3g cells, kept %.3f; heuristic %.1f ms, %.3g cells, kept %.3f" % (
        1e3 * t_net, cells_net, (used_net == 1).mean(), 1e3 * t_heu, cells_heu, (used_heu == 1).mean())
    assert cells_net < 0.8 * cells_heu, msg
    assert t_net < t_heu, msg
