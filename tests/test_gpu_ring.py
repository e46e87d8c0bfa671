"""GPU tests of the ring-scheduled banded gap DP (csrc/gapdp_ring.cuh).

Every banded result must equal the oracle's NWSmall (scores and paths) and
so the full DP's, whichever
group height the schedule picks; the tests build bands that land in each
height class and at the edges of the schedule's validity."""
import numpy as np
import pytest

import bandnet
import mvg
import oracle as O
import synth

pytestmark = pytest.mark.gpu

RING_ROWS = (4, 6, 8, 12, 16, 24, 32)


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


def ring_lo(LA, LB, delta, half, R, g):
    return (g * R + 1) * LB // LA + delta - half


def ring_rows(LA, LB, delta, half):
    """The group height the host picks (band.h ring_eligible), 0 if none."""
    half = max(half, 0)
    for R in RING_ROWS:
        G = (LA + R - 1) // R
        W = 2 * half + 2 + ((R - 1) * LB + LA - 1) // LA
        lo0, lol = ring_lo(LA, LB, delta, half, R, 0), ring_lo(LA, LB, delta, half, R, G - 1)
        if half > (1 << 20) or abs(delta) > (1 << 24):
            continue
        if lo0 > 1 or lo0 + W - 1 < 1 or lol > LB or lol + W - 1 < LB:
            continue
        if (R * LB + LA - 1) // LA > W - 1:
            continue
        if G > 32 and W > 32 + 32 * R * LB // LA:
            continue
        return R
    return 0


def whole_band(LA, LB, half, frac=0.5):
    return 2.0 * half + 2.0 + np.ceil(LB / LA) >= frac * LB


def batch_from_pairs(pairs):
    sa = np.concatenate([a for a, _ in pairs]).astype(np.uint8)
    sb = np.concatenate([b for _, b in pairs]).astype(np.uint8)
    oa = np.zeros(len(pairs) + 1, np.uint64)
    ob = np.zeros(len(pairs) + 1, np.uint64)
    oa[1:] = np.cumsum([len(a) for a, _ in pairs])
    ob[1:] = np.cumsum([len(b) for _, b in pairs])
    return sa, oa, sb, ob


def related_pair(rng, la, sub=0.02, indels=2):
    a = rng.integers(0, 4, la).astype(np.uint8)
    b = a.copy()
    m = rng.random(la) < sub
    b[m] = (b[m] + rng.integers(1, 4, int(m.sum()))) % 4
    for _ in range(indels):
        if len(b) < 4:
            break
        k = int(rng.integers(1, len(b) - 1))
        if rng.random() < 0.5:
            b = np.concatenate([b[:k], b[k + int(rng.integers(1, 5)):]])
        else:
            b = np.concatenate([b[:k], rng.integers(0, 4, int(rng.integers(1, 5))).astype(np.uint8), b[k:]])
    if len(b) == 0:
        b = rng.integers(0, 4, 1).astype(np.uint8)
    return a, b


def check_identical(ctx, sa, oa, sb, ob, delta, half):
    """Banded output equals the oracle's NWSmall scores and paths (and so the
    full DP's, checked as well)."""
    s_full, p_full = ctx.gap_align_batch(sa, oa, sb, ob)
    s, p, used, cells = ctx.gap_align_banded(sa, oa, sb, ob, np.asarray(delta, np.int32), np.asarray(half, np.int32))
    oscores, oplen, opaths, opoff = O.nw_batch(sa, oa, sb, ob)
    np.testing.assert_array_equal(s, oscores)
    raw = opaths.tobytes()
    for k in range(len(oa) - 1):
        assert p[k] == raw[int(opoff[k]):int(opoff[k]) + int(oplen[k])].decode(), k
    np.testing.assert_array_equal(s_full, oscores)
    assert p == p_full
    return used, cells, s_full


@pytest.mark.parametrize("R", RING_ROWS)
def test_each_group_height_matches_full_dp(ctx, R):
    """Bands sized so the schedule picks group height R; accepted ones must
    exist and every output equals the full DP's."""
    rng = np.random.default_rng(100 + R)
    pairs, deltas, halves = [], [], []
    # the largest half-width a height takes on a diagonal band is about
    # (31 R + 31) / 2; aim between the previous height's and this one's
    target_half = {4: 40, 6: 95, 8: 125, 12: 170, 16: 235, 24: 330, 32: 450}[R]
    while len(pairs) < 48:
        la = int(rng.integers(2 * target_half + 200, 6000))
        # divergence low enough for the band's exactness bound to pass:
        # each substitution costs about 210 against the best-base sum,
        # a band of half-width h absorbs about 155 h
        sub = float(rng.uniform(0.0005, 0.5 * 155 * target_half / (210 * la)))
        a, b = related_pair(rng, la, sub=sub, indels=int(rng.integers(0, 3)))
        half = int(target_half + rng.integers(-5, 6))
        delta = int(rng.integers(-8, 9))
        if ring_rows(len(a), len(b), delta, half) != R or whole_band(len(a), len(b), half):
            continue
        pairs.append((a, b))
        deltas.append(delta)
        halves.append(half)
    sa, oa, sb, ob = batch_from_pairs(pairs)
    used, cells, _ = check_identical(ctx, sa, oa, sb, ob, deltas, halves)
    assert (used == 1).sum() >= 24, used
    la, lb = np.diff(oa.astype(np.int64)), np.diff(ob.astype(np.int64))
    assert 0 < cells < float(np.sum(la * lb))


def test_ring_and_strip_kernels_agree_on_mixed_batch(ctx):
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=31, nprob=600, lmin=1, lmax=3000)
    la, lb = np.diff(oa), np.diff(ob)
    rng = np.random.default_rng(5)
    n = len(la)
    for delta, half in [bandnet.heuristic_band(la, lb),
                        (rng.integers(-60, 60, n).astype(np.int32), rng.integers(0, 400, n).astype(np.int32)),
                        (np.zeros(n, np.int32), np.zeros(n, np.int32))]:
        used_ring, _, _ = check_identical(ctx, sa, oa, sb, ob, delta, half)
        ctx.set_band_ring(False)
        try:
            used_strip, _, _ = check_identical(ctx, sa, oa, sb, ob, delta, half)
        finally:
            ctx.set_band_ring(True)
        assert set(np.unique(used_ring)) <= {0, 1, 2}
        assert set(np.unique(used_strip)) <= {0, 1, 2}


def test_ring_many_problems_per_warp(ctx):
    """Far more banded problems than warps, so every warp takes several in
    turn: scores, paths and the accepted bands equal the full DP's."""
    rng = np.random.default_rng(77)
    pairs, deltas, halves = [], [], []
    for _ in range(24000):
        la = int(rng.integers(20, 400))
        a, b = related_pair(rng, la, sub=float(rng.uniform(0.0, 0.03)), indels=int(rng.integers(0, 3)))
        pairs.append((a, b))
        deltas.append(int(rng.integers(-3, 4)))
        halves.append(int(rng.integers(4, 60)))
    sa, oa, sb, ob = batch_from_pairs(pairs)
    used, cells, _ = check_identical(ctx, sa, oa, sb, ob, deltas, halves)
    assert (used == 1).sum() > 5000
