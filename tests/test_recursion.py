"""Recursive anchor search gap finding (mvg_recursion_gaps) and the
gapped-alignment pass's windows (mvg_refine_windows) against the oracle's
restatements of recurseOnPairs / getInterveningCoordinates and of
refineAlignment / removeLargeGapsPP / IsDenseEnough.  Host code only: no
GPU."""
import numpy as np
import pytest

import mvg
import recursion_oracle as RO


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as pkg_build
    pkg_build.build()


def _rows(spec):
    return np.frombuffer(spec[0].encode(), np.uint8), np.frombuffer(spec[1].encode(), np.uint8)


def test_one_forward_gap_by_hand():
    """Two aligned columns, 5 characters of A only, 5 of B only, two aligned
    columns: the cut starts at the left anchor's own base and is one base
    shorter than the stretch between the anchors (the reference's
    arithmetic), in both genomes."""
    a, b = _rows(("AC" + "GGGGG" + "-----" + "TT", "AC" + "-----" + "CCCCC" + "TT"))
    gaps, flanks = mvg.recursion_gaps(a, b, 101, False, 201, False, 10_000, 10_000, min_gap=3)
    np.testing.assert_array_equal(gaps, [[101, 5, 201, 5]])
    assert not flanks.any()
    og, of = RO.recursion_gaps(a, b, 101, False, 201, False, 10_000, 10_000, min_gap=3)
    assert og == [tuple(x) for x in gaps.tolist()]


def test_gap_at_or_below_min_is_not_searched():
    a, b = _rows(("AC" + "GGG" + "---" + "TT", "AC" + "---" + "CCC" + "TT"))
    gaps, _ = mvg.recursion_gaps(a, b, 1, False, 1, False, 100, 100, min_gap=4)
    assert gaps.shape == (0, 4)


def _random_lcb(rng, ncols, p_gap_a, p_gap_b, runs):
    """Gapped rows with gap runs, so that long one-sided stretches occur."""
    a = np.full(ncols, ord("A"), np.uint8)
    b = np.full(ncols, ord("C"), np.uint8)
    c = 0
    while c < ncols:
        ln = int(rng.integers(1, runs))
        kind = rng.random()
        if kind < p_gap_a:
            a[c:c + ln] = ord("-")
        elif kind < p_gap_a + p_gap_b:
            b[c:c + ln] = ord("-")
        c += ln
    # no all-gap column
    both_gap = (a == ord("-")) & (b == ord("-"))
    a[both_gap] = ord("G")
    return a, b


@pytest.mark.parametrize("rev_a,rev_b", [(False, False), (False, True), (True, False), (True, True)])
def test_random_lcbs_match_the_oracle(rev_a, rev_b):
    """Gaps and flanks equal the oracle's on 200 random LCBs per orientation
    pair: gap runs of up to 60 columns, minimum gap 8 and 30, LCBs starting
    anywhere in the genome (including position 1, where the reference's
    right-anchor test compares counts with coordinates)."""
    rng = np.random.default_rng(7 + 2 * rev_a + rev_b)
    for it in range(200):
        ncols = int(rng.integers(0, 1500))
        a, b = _random_lcb(rng, ncols, 0.35, 0.35, 60)
        na, nb = int((a != ord("-")).sum()), int((b != ord("-")).sum())
        la = 1 if it % 5 == 0 else int(rng.integers(1, 5000))
        lb = 1 if it % 7 == 0 else int(rng.integers(1, 5000))
        ga = la + na + int(rng.integers(0, 3))
        gb = lb + nb + int(rng.integers(0, 3))
        for min_gap in (8, 30):
            gaps, flanks = mvg.recursion_gaps(a, b, la, rev_a, lb, rev_b, ga, gb, min_gap=min_gap)
            og, of = RO.recursion_gaps(a, b, la, rev_a, lb, rev_b, ga, gb, min_gap=min_gap)
            assert [tuple(x) for x in gaps.tolist()] == og, (it, min_gap)
            for q in range(2):
                want = list(of[q]) + [(0, 0)] * (2 - len(of[q]))
                assert [tuple(x) for x in flanks[q].tolist()] == want, (it, q)


def test_flanks_and_no_aligned_column():
    """Unaligned ends become flanks (merged when they touch); an LCB with no
    column where both genomes are aligned has one flank per genome and the
    whole LCB as its only gap when long enough."""
    a, b = _rows(("GGG" + "AC" + "TT", "---" + "AC" + "--"))
    _, flanks = mvg.recursion_gaps(a, b, 11, False, 21, False, 100, 100, min_gap=1)
    _, of = RO.recursion_gaps(a, b, 11, False, 21, False, 100, 100, min_gap=1)
    np.testing.assert_array_equal(flanks[0], [[11, 14], [16, 18]])
    assert [tuple(x) for x in flanks[0].tolist()] == list(of[0])
    a, b = _rows(("GGGGG-----", "-----CCCCC"))
    gaps, flanks = mvg.recursion_gaps(a, b, 5, False, 7, False, 100, 100, min_gap=2)
    og, of = RO.recursion_gaps(a, b, 5, False, 7, False, 100, 100, min_gap=2)
    assert [tuple(x) for x in gaps.tolist()] == og and len(og) == 1


def test_rejects_lcb_past_the_genome():
    a, b = _rows(("ACGT", "ACGT"))
    with pytest.raises(Exception):
        mvg.recursion_gaps(a, b, 10, False, 1, False, 12, 100)


def test_refine_windows_match_the_oracle():
    """refineAlignment's windows (long one-genome stretches cut out as gap
    windows with 300 columns kept on either side, windows halved while too
    long for their density) equal the oracle's restatement on random LCBs
    at several window limits, and tile the LCB."""
    rng = np.random.default_rng(1015)
    for it in range(60):
        parts_a, parts_b = [], []
        for s in range(int(rng.integers(1, 6))):
            n = int(rng.integers(50, 3000))
            a, b = _random_lcb(rng, n, 0.2, 0.2, 40)
            parts_a.append(a)
            parts_b.append(b)
            run = int(rng.choice([10, 800, 5001, 5300, 7000]))
            one = np.full(run, ord("A"), np.uint8)
            gap = np.full(run, ord("-"), np.uint8)
            parts_a.append(one if s % 2 else gap)
            parts_b.append(gap if s % 2 else one)
        ra, rb = np.concatenate(parts_a), np.concatenate(parts_b)
        for maxw in (400.0, 2500.0, 20000.0):
            got = [tuple(x) for x in mvg.refine_windows(ra, rb, maxw).tolist()]
            want = [(a, b, int(g)) for a, b, g in RO.refine_windows(ra, rb, maxw)]
            assert got == want, (it, maxw)
            assert got[0][0] == 0 and got[-1][1] == len(ra)
            assert all(x[1] == y[0] for x, y in zip(got[:-1], got[1:]))


def _golden_lcb(g, k):
    """Rows of golden LCB k (bases as 'A', gaps as '-'), its genomes and its
    parameters."""
    n = int(g["c%d_ncols" % k])
    rows = [np.where(np.unpackbits(g["c%d_mask_%s" % (k, q)])[:n] == 1, ord("A"), ord("-")).astype(np.uint8)
            for q in "ab"]
    p = int(g["pair%d" % k])
    left_a, left_b, rev_a, rev_b, min_gap = [int(x) for x in g["c%d_left" % k]]
    return rows, g["a%d" % p], g["b%d" % p], (left_a, bool(rev_a), left_b, bool(rev_b)), min_gap


def test_recursion_equals_the_reference_recurse_on_pairs():
    """22 LCBs (tests/golden/recursion.npz, the reference's own
    recurseOnPairs): the regions outside each LCB equal the reference's
    iv_regions, and the gaps, searched one by one with the oracle's
    pairwiseAnchorSearch and shifted to genome coordinates, give the
    reference's anchors in its order (all strand pairs, minimum gaps 200 and
    60, LCBs at a genome's first and last base, one without an aligned
    column)."""
    import oracle as O
    from conftest import load_golden
    g = load_golden("recursion.npz")
    total = 0
    for k in range(int(g["count"])):
        (ra, rb), a, b, (la, rva, lb, rvb), min_gap = _golden_lcb(g, k)
        gaps, flanks = mvg.recursion_gaps(ra, rb, la, rva, lb, rvb, len(a), len(b), min_gap=min_gap)
        for q, key in ((0, "ra"), (1, "rb")):
            got = [int(v) for lo, hi in flanks[q] if lo < hi for v in (lo, hi)]
            assert got == [int(v) for v in g["c%d_%s" % (k, key)]], (k, q)
        anchors = []
        for s0, l0, s1, l1 in gaps.tolist():
            _, anc = O.gap_anchor_search(a[s0:s0 + l0], b[s1:s1 + l1])
            for x, y, L in ([] if anc is None else anc.tolist()):
                anchors.append((x + s0 if x > 0 else x - s0, y + s1 if y > 0 else y - s1, L))
        want = g["c%d_anchors" % k]
        assert anchors == [tuple(r) for r in want.tolist()], k
        total += len(want)
    assert total > 1000


def _nw_rows(a, b):
    """Rows of the oracle's NWSmall alignment of two base arrays (either
    case), letters kept."""
    import oracle as O
    acgt = np.frombuffer(b"ACGT", np.uint8)
    path, _ = O.nw_align(np.searchsorted(acgt, a & 0xDF).astype(np.uint8),
                         np.searchsorted(acgt, b & 0xDF).astype(np.uint8))
    ra, rb, i, j = [], [], 0, 0
    for e in path:
        ra.append(a[i] if e in "MD" else ord("-"))
        rb.append(b[j] if e in "MI" else ord("-"))
        i += e in "MD"
        j += e in "MI"
    return np.array(ra, np.uint8), np.array(rb, np.uint8)


def _refine_on_cpu(ra, rb, maxw):
    out_a, out_b, at = [], [], 0
    for lo, hi in mvg.refine_fast_ranges(ra, rb, maxw).tolist():
        out_a.append(ra[at:lo])
        out_b.append(rb[at:lo])
        wa, wb = ra[lo:hi], rb[lo:hi]
        a, b = wa[wa != ord("-")], wb[wb != ord("-")]
        x, y = _nw_rows(a, b) if len(a) and len(b) else (wa, wb)
        out_a.append(x)
        out_b.append(y)
        at = hi
    out_a.append(ra[at:])
    out_b.append(rb[at:])
    return np.concatenate(out_a), np.concatenate(out_b)


def test_refinement_ranges_rebuild_the_reference_refinement():
    """The final iterative-refinement pass (refineAlignment with profile_aln
    = false) of 11 LCBs (tests/golden/refine.npz, the reference's own
    output), rebuilt on the CPU from mvg_refine_fast_ranges and the oracle's
    NWSmall per range: equal to the reference alone and after the
    gapped-alignment pass, including three LCBs made worse beforehand."""
    from conftest import load_golden
    g = load_golden("refine.npz")
    changed = 0
    for k in range(int(g["count"])):
        maxw = float(g["w%d" % k])
        ia, ib = _refine_on_cpu(g["a%d" % k], g["b%d" % k], maxw)
        np.testing.assert_array_equal(ia, g["ia%d" % k], err_msg=str(k))
        np.testing.assert_array_equal(ib, g["ib%d" % k], err_msg=str(k))
        fa, fb = _refine_on_cpu(g["oa%d" % k], g["ob%d" % k], maxw)
        np.testing.assert_array_equal(fa, g["fa%d" % k], err_msg=str(k))
        np.testing.assert_array_equal(fb, g["fb%d" % k], err_msg=str(k))
        changed += len(g["a%d" % k]) != len(ia) or bool((g["a%d" % k] != ia).any())
    assert changed >= 3
