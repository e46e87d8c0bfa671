"""GPU tests of the batched gap anchor search (csrc/gapsearch.cu):
pairwiseAnchorSearch for many gaps in one call, through the C ABI, against
the reference's own anchors (tests/golden/gapsearch.npz) and the oracle."""
import numpy as np
import pytest

import mvg
import oracle as O
import synth
from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


def embed(rng, pairs, spacer=(0, 300)):
    """Concatenates the gap pairs into two genomes with random spacers;
    returns (genome A, genome B, gap rows (start A, len A, start B, len B))."""
    parts_a, parts_b, rows = [], [], []
    pa = pb = 0
    for a, b in pairs:
        sa = synth.random_bases(rng, int(rng.integers(*spacer)))
        sb = synth.random_bases(rng, int(rng.integers(*spacer)))
        parts_a += [sa, a]
        parts_b += [sb, b]
        pa += len(sa)
        pb += len(sb)
        rows.append((pa, len(a), pb, len(b)))
        pa += len(a)
        pb += len(b)
    return np.concatenate(parts_a), np.concatenate(parts_b), np.array(rows, np.int64)


def shift(anchors, ra, rb):
    out = anchors.copy()
    for q, off in ((0, ra), (1, rb)):
        out[:, q] = np.where(out[:, q] > 0, out[:, q] + off, out[:, q] - off)
    return out


def test_gap_search_reference_fixtures(ctx):
    """44 gaps of 9 bp to 50 kbp in one call: every gap's anchors equal the
    reference's pairwiseAnchorSearch output (EliminateOverlaps_v2 and
    LengthFilter applied), in order, shifted to genome coordinates."""
    g = load_golden("gapsearch.npz")
    n = int(g["count"])
    rng = np.random.default_rng(1)
    ga, gb, rows = embed(rng, [(g["a%d" % k], g["b%d" % k]) for k in range(n)])
    anchors, off = ctx.gap_anchor_search(ga, gb, rows)
    assert len(off) == n + 1 and off[-1] == len(anchors)
    for k in range(n):
        want = shift(g["anc%d" % k], rows[k, 0], rows[k, 2])
        np.testing.assert_array_equal(anchors[off[k]:off[k + 1]], want, err_msg="gap %d" % k)


@pytest.mark.parametrize("seed", [0, 1])
def test_gap_search_random_gaps_vs_oracle(ctx, seed):
    """1,500 gaps drawn like a recursion round's (200 bp - 20 kbp, 0-25%
    substitutions, indels, inversions, repeats, unrelated gaps), searched
    in one call: equal to the oracle's search of each gap."""
    rng = np.random.default_rng(300 + seed)
    pairs = []
    for _ in range(1500):
        n = int(np.exp(rng.uniform(np.log(200), np.log(20_000))))
        b = synth.random_bases(rng, n, float(rng.uniform(0.35, 0.65)))
        if rng.random() < 0.2:
            b = synth.insert_repeats(rng, b, int(rng.integers(20, max(21, n // 5))), int(rng.integers(2, 6)))
        if rng.random() < 0.1:
            a = synth.random_bases(rng, int(n * rng.uniform(0.5, 1.5)) + 1)
        else:
            a = synth.mutate(rng, b, float(rng.uniform(0, 0.25)), int(rng.integers(0, 1 + n // 500)), 3.0,
                             int(rng.integers(0, 2)) if n > 3000 else 0, (100, max(101, n // 8)))
        pairs.append((a, b))
    ga, gb, rows = embed(rng, pairs)
    anchors, off = ctx.gap_anchor_search(ga, gb, rows)
    for k, (a, b) in enumerate(pairs):
        w, anc = O.gap_anchor_search(a, b)
        want = np.zeros((0, 3), np.int64) if anc is None else shift(anc, rows[k, 0], rows[k, 2])
        np.testing.assert_array_equal(anchors[off[k]:off[k + 1]], want, err_msg="gap %d" % k)


def test_gap_search_edge_gaps(ctx):
    """Empty and one-sided gaps, gaps too short for a seed weight of 5,
    gaps touching the genome ends, a repeated gap, and the device entry
    point: all equal to the oracle; a gap outside its genome is refused."""
    rng = np.random.default_rng(9)
    b = synth.random_bases(rng, 60_000)
    a = synth.mutate(rng, b, 0.05, 30, 3.0, 1, (500, 3000))
    rows = np.array([(0, 0, 0, 0), (0, 5000, 0, 0), (0, 0, 100, 4000), (10, 12, 10, 14), (0, 3000, 0, 3100),
                     (len(a) - 2500, 2500, len(b) - 2400, 2400), (20_000, 8000, 19_800, 8100),
                     (20_000, 8000, 19_800, 8100), (30_000, 1, 30_000, 1)], np.int64)
    anchors, off = ctx.gap_anchor_search(a, b, rows)
    for k, (xa, la, xb, lb) in enumerate(rows):
        w, anc = O.gap_anchor_search(a[xa:xa + la], b[xb:xb + lb])
        want = np.zeros((0, 3), np.int64) if anc is None else shift(anc, xa, xb)
        np.testing.assert_array_equal(anchors[off[k]:off[k + 1]], want, err_msg="gap %d" % k)
    import torch
    da, db = torch.from_numpy(a.copy()).cuda(), torch.from_numpy(b.copy()).cuda()
    dev_anchors, dev_off = ctx.gap_anchor_search_dev(da.data_ptr(), len(a), db.data_ptr(), len(b), rows,
                                                     len(anchors) + 8)
    np.testing.assert_array_equal(dev_anchors, anchors)
    np.testing.assert_array_equal(dev_off, off)
    with pytest.raises(IndexError):
        ctx.gap_anchor_search(a, b, np.array([(len(a) - 10, 20, 0, 100)], np.int64))
    assert ctx.gap_anchor_search(a, b, np.zeros((0, 4), np.int64))[0].shape == (0, 3)


def test_recursion_gaps_feed_the_gap_search(ctx):
    """One recursion round end to end: the gaps an LCB's alignment leaves
    (mvg_recursion_gaps, recurseOnPairs' rule: both genomes more than 200
    characters between two columns where both are aligned) are searched in
    one call, and every gap's anchors equal the oracle's pairwiseAnchorSearch
    on the same cut sequences, for a forward and a reverse-strand LCB."""
    import recursion_oracle as RO
    rng = np.random.default_rng(2024)
    a = synth.random_bases(rng, 60_000)
    b = synth.mutate(rng, a, 0.05, 40, 3.0, 0, (1, 2))
    for rev_b in (False, True):
        # an LCB whose rows alternate aligned stretches with one-sided runs
        ra, rb = [], []
        na = nb = 0
        while na < 40_000 and nb < 40_000:
            k = int(rng.integers(20, 200))
            ra.append(b"A" * k)
            rb.append(b"C" * k)
            na += k
            nb += k
            ga, gb = int(rng.integers(0, 900)), int(rng.integers(0, 900))
            ra.append(b"G" * ga + b"-" * gb)
            rb.append(b"-" * ga + b"T" * gb)
            na += ga
            nb += gb
        row_a = np.frombuffer(b"".join(ra), np.uint8)
        row_b = np.frombuffer(b"".join(rb), np.uint8)
        gaps, _ = mvg.recursion_gaps(row_a, row_b, 1001, False, 1501, rev_b, len(a), len(b))
        og, _ = RO.recursion_gaps(row_a, row_b, 1001, False, 1501, rev_b, len(a), len(b))
        assert [tuple(x) for x in gaps.tolist()] == og
        assert len(gaps) > 10
        anchors, off = ctx.gap_anchor_search(a, b, gaps)
        for k, (sa, la, sb, lb) in enumerate(gaps.tolist()):
            w, want = O.gap_anchor_search(a[sa:sa + la], b[sb:sb + lb])
            want = np.zeros((0, 3), np.int64) if want is None else shift(want, sa, sb)
            np.testing.assert_array_equal(anchors[off[k]:off[k + 1]], want, err_msg="gap %d" % k)


def test_recursion_round_equals_the_reference_recurse_on_pairs(ctx):
    """The reference's own recurseOnPairs on 22 LCBs
    (tests/golden/recursion.npz): every LCB's gaps (mvg_recursion_gaps) of a
    genome pair searched in ONE batched call, as a recursion round does, give
    each LCB the reference's anchors in its order."""
    from test_recursion import _golden_lcb
    g = load_golden("recursion.npz")
    by_pair = {}
    for k in range(int(g["count"])):
        by_pair.setdefault(int(g["pair%d" % k]), []).append(k)
    total = 0
    for p, ks in by_pair.items():
        rows_gaps, spans = [], []
        for k in ks:
            (ra, rb), a, b, (la, rva, lb, rvb), min_gap = _golden_lcb(g, k)
            gaps, _ = mvg.recursion_gaps(ra, rb, la, rva, lb, rvb, len(a), len(b), min_gap=min_gap)
            spans.append((k, len(rows_gaps), len(rows_gaps) + len(gaps)))
            rows_gaps += gaps.tolist()
        anchors, off = ctx.gap_anchor_search(g["a%d" % p], g["b%d" % p], np.array(rows_gaps, np.int64).reshape(-1, 4))
        for k, g0, g1 in spans:
            np.testing.assert_array_equal(anchors[off[g0]:off[g1]], g["c%d_anchors" % k], err_msg=str(k))
            total += int(off[g1] - off[g0])
    assert total > 1000
