"""Pins the CPU oracle to the golden fixtures made by the reference's own
C++ code (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle as O
from conftest import load_golden


def test_seed_table_and_default_weights():
    g = load_golden("seeds.npz")
    for wi, w in enumerate(range(3, 32)):
        for r in range(6):
            assert O.get_seed(w, r) == int(g["table"][wi, r]), (w, r)
    for n, w in zip(g["lens"], g["weights"]):
        assert O.default_seed_weight(int(n)) == int(w), n
    # coding seed for the 1-4.6 Mbp genomes, solid 17-mer for 12 Mbp
    assert O.get_seed(O.default_seed_weight(4_600_000), 3) == 0x16DF6D
    assert O.get_seed(O.default_seed_weight(12_000_000), 3) == (1 << 17) - 1


def test_sml_fill_and_sort_match_reference():
    g = load_golden("sml.npz")
    for k in range(int(g["count"])):
        seq, seed = g["seq%d" % k], int(g["seed%d" % k])
        np.testing.assert_array_equal(O.seed_mers(seq, seed), g["fill%d" % k])
        pos, mer = O.sml_build(seq, seed)
        rpos, rmer = g["pos%d" % k], g["mer%d" % k]
        np.testing.assert_array_equal(mer, rmer)  # same sorted key sequence
        # same (mer, pos) multiset; tie order inside equal mers is unspecified in the reference
        ref = np.lexsort((rpos, rmer))
        np.testing.assert_array_equal(pos, rpos[ref])


def test_pairwise_match_lists_match_reference():
    g = load_golden("matches.npz")
    for k in range(int(g["count"])):
        m = O.pairwise_matches(g["a%d" % k], g["b%d" % k], int(g["seed%d" % k]))
        np.testing.assert_array_equal(m, g["m%d" % k], err_msg="case %d" % k)


def test_gap_search_memhash_equals_pairwise_matcher():
    """pairwiseAnchorSearch's MemHash::FindMatches (rank-0 seed of the gap's
    default weight, LM/ProgressiveAligner.cpp:590-679) hashes exactly the
    seeds unique in both gap sequences, so its list equals the pairwise
    matcher's (the oracle) with that seed on every fixture gap."""
    g = load_golden("gapsearch.npz")
    for k in range(int(g["count"])):
        a, b, w = g["a%d" % k], g["b%d" % k], int(g["w%d" % k])
        assert w == O.default_seed_weight((len(a) + len(b)) // 2)
        if w < 5:
            assert len(g["anc%d" % k]) == 0
            continue
        np.testing.assert_array_equal(O.pairwise_matches(a, b, O.get_seed(w, 0)), g["mh%d" % k], err_msg="gap %d" % k)


def test_gap_anchor_search_matches_reference():
    """The oracle's gap anchor search (matches, EliminateOverlaps_v2,
    LengthFilter(12)) gives the reference's anchors, in order."""
    g = load_golden("gapsearch.npz")
    for k in range(int(g["count"])):
        w, anc = O.gap_anchor_search(g["a%d" % k], g["b%d" % k])
        assert w == int(g["w%d" % k])
        if anc is None:
            assert len(g["anc%d" % k]) == 0
            continue
        np.testing.assert_array_equal(anc, g["anc%d" % k], err_msg="gap %d" % k)
        np.testing.assert_array_equal(O.gap_anchor_filter(g["mh%d" % k]), g["anc%d" % k])


def test_gap_dp_paths_match_reference():
    g = load_golden("gapdp.npz")
    sa, sb, oa, ob, paths, op = g["seq_a"], g["seq_b"], g["off_a"], g["off_b"], g["paths"], g["off_p"]
    for k in range(len(oa) - 1):
        a, b = sa[oa[k]:oa[k + 1]], sb[ob[k]:ob[k + 1]]
        path, score = O.nw_align(a, b)
        assert path == paths[op[k]:op[k + 1]].tobytes().decode(), k
        assert path.count("M") + path.count("D") == len(a)
        assert path.count("M") + path.count("I") == len(b)


def test_pack_layout():
    w = O.pack(b"ACGTACGTACGTACGTC")
    assert w[0] == 0x1B1B1B1B and w[1] == 0x40000000 and len(w) == 2 + 2
    with pytest.raises(ValueError):
        O.pack(b"AC-GT")


def test_oracle_matches_on_the_reference_mds42_pair():
    """The reference's own recoded E. coli fixture pair (3.98 Mbp each):
    the oracle's match list equals the reference's."""
    from conftest import load_mds42
    a, b, seed, want = load_mds42()
    got = O.pairwise_matches(a, b, seed)
    np.testing.assert_array_equal(got, want)
