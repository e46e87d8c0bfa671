"""The search outside LCBs, host steps (mvg_transpose_matches,
mvg_eliminate_overlaps, mvg_lcb_gap_finish) against the reference's own
transposeMatches / EliminateOverlaps / SearchLCBGaps output
(tests/golden/lcbgaps.npz).  No GPU."""
import numpy as np
import pytest

import mvg
from conftest import load_golden


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as pkg_build
    pkg_build.build()


def _post(g, key, k):
    off = g["post_%s_off" % key]
    return g["post_" + key][off[k]:off[k + 1]].astype(np.int64)


def test_host_steps_equal_the_reference_on_random_match_lists():
    """80 random match lists (reverse B starts, repeated A starts, exact
    duplicates, matches over region seams, zero-length and touching
    regions): transposeMatches for each genome, EliminateOverlaps and the
    finishing sequence equal the reference's, in order."""
    g = load_golden("lcbgaps.npz")
    n = len(g["post_m_off"]) - 1
    splits = 0
    for k in range(n):
        m = _post(g, "m", k).reshape(-1, 3)
        ra, rb = _post(g, "ra", k), _post(g, "rb", k)
        t0 = mvg.transpose_matches(m, 0, ra)
        np.testing.assert_array_equal(t0, _post(g, "t0", k).reshape(-1, 3), err_msg=str(k))
        np.testing.assert_array_equal(mvg.transpose_matches(m, 1, rb), _post(g, "t1", k).reshape(-1, 3))
        np.testing.assert_array_equal(mvg.eliminate_overlaps(m), _post(g, "eo", k).reshape(-1, 3))
        np.testing.assert_array_equal(mvg.lcb_gap_finish(m, ra, rb), _post(g, "fin", k).reshape(-1, 3))
        splits += len(t0) - len(m)
    assert splits > 100


def test_finish_equals_search_lcb_gaps_on_searched_genomes():
    """The reference's raw match list of each pair of region concatenations,
    finished on the host, equals the reference's SearchLCBGaps output for
    those genomes and regions (lowercase, N and IUPAC codes in one pair; one
    genome without regions; a pair too short to find anything)."""
    g = load_golden("lcbgaps.npz")
    for k in range(int(g["search_count"])):
        got = mvg.lcb_gap_finish(g["s%d_raw" % k], g["s%d_ra" % k], g["s%d_rb" % k])
        np.testing.assert_array_equal(got, g["s%d_fin" % k], err_msg=str(k))
    assert sum(len(g["s%d_fin" % k]) for k in range(int(g["search_count"]))) > 200


def test_transpose_maps_and_splits_by_hand():
    """A match over the seam of regions [11, 21) and [31, 41) (10 bases
    each): concatenation start 6, length 10 -> A 16..20 and, split off, A
    31..35.  B is reverse (B 3..12), so A's first half pairs with B's right
    half: the kept piece's B start moves to -8, the split-off piece keeps -3
    (the values the reference's transposeMatches gives)."""
    m = np.array([[6, -3, 10]], np.int64)
    out = mvg.transpose_matches(m, 0, [11, 21, 31, 41])
    np.testing.assert_array_equal(out, [[16, -8, 5], [31, -3, 5]])


def test_regions_are_collected_and_sorted_per_genome():
    f1 = np.array([[[50, 60], [0, 0]], [[7, 9], [20, 30]]], np.int64)
    f2 = np.array([[[10, 20], [80, 90]], [[0, 0], [0, 0]]], np.int64)
    ra, rb = mvg.lcb_gap_regions([f1, f2])
    np.testing.assert_array_equal(ra, [10, 20, 50, 60, 80, 90])
    np.testing.assert_array_equal(rb, [7, 9, 20, 30])


def test_bad_arguments_are_rejected():
    with pytest.raises(Exception):
        mvg.transpose_matches([[1, 1, 5]], 0, [10, 20, 30])  # odd boundary count
    with pytest.raises(Exception):
        mvg.transpose_matches([[1, 1, 5]], 2, [10, 20])  # no third genome
    with pytest.raises(Exception):
        mvg.lcb_gap_finish([[1, 1, 5]], [20, 10], [1, 5])  # region ends before it starts
    with pytest.raises(Exception):
        mvg.eliminate_overlaps([[1, 1, -5]])
