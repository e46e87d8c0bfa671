"""The LUT oracle (oracle/lut_oracle.c) against the golden vectors produced
by the reference's own buildIndex() and compiled indexutils (CPU only)."""
import numpy as np
import pytest

import oracle as O
from conftest import load_golden


@pytest.fixture(scope="module")
def g():
    return load_golden("lut.npz")


def _blocks(g, k):
    return (g["b%d_gs" % k], g["b%d_rs" % k], g["b%d_off" % k], g["b%d_rg" % k], g["b%d_rr" % k])


def oracle_build(g, k, fill, width, smooth, radius):
    gs, rs, off, rg, rr = _blocks(g, k)
    n = len(g["b%d_genome" % k])
    L = O.lib()
    lut = np.empty(n, np.int32)
    rc = L.mo_lut_from_blocks(O._p(gs), O._p(rs), O._p(off), O._p(rg), O._p(rr), len(gs), O._p(lut), n)
    assert rc == 0
    if fill:
        O.fix_zero_idx(lut, g["b%d_genome" % k], g["b%d_ref" % k])
        O.fill_gaps(lut, width)
    if smooth:
        O.smooth_edges(lut, radius)
    return lut


def test_build_index_variants(g):
    for k in range(int(g["n_build"])):
        for v, (fill, width, smooth, radius) in enumerate(g["build_variants"]):
            got = oracle_build(g, k, fill, width, smooth, radius)
            np.testing.assert_array_equal(got, g["b%d_v%d" % (k, v)], err_msg="case %d variant %d" % (k, v))


def test_cleanup_passes(g):
    for k in range(int(g["n_lut"])):
        lut0 = g["l%d_in" % k]
        for name, w in (("fill300", 300), ("fill40", 40), ("fill3", 3), ("fill0", 0), ("fillneg", -5)):
            x = lut0.copy()
            O.fill_gaps(x, w)
            np.testing.assert_array_equal(x, g["l%d_%s" % (k, name)])
        for name, r in (("smooth20", 20), ("smooth5", 5), ("smoothneg", -1)):
            x = lut0.copy()
            O.smooth_edges(x, r)
            np.testing.assert_array_equal(x, g["l%d_%s" % (k, name)])
        x = lut0.copy()
        gaps = O.find_gaps(x)
        np.testing.assert_array_equal(x, g["l%d_findgaps_lut" % k])
        np.testing.assert_array_equal(gaps, g["l%d_findgaps" % k])
        np.testing.assert_array_equal(O.find_mismatches(lut0, g["l%d_genome" % k], g["l%d_ref" % k]),
                                      g["l%d_mism" % k])
        assert O.find_duplicate_mappings(lut0.copy()) == int(g["l%d_dups" % k])


def test_fix_zero_idx(g):
    for i in range(int(g["n_fz"])):
        x = g["fz%d_in" % i].copy()
        if int(g["fz%d_status" % i]) == -999:
            with pytest.raises(IndexError):
                O.fix_zero_idx(x, g["fz%d_genome" % i], g["fz%d_ref" % i])
        else:
            O.fix_zero_idx(x, g["fz%d_genome" % i], g["fz%d_ref" % i])
            np.testing.assert_array_equal(x, g["fz%d_out" % i])


def test_find_edges_restated():
    lut = np.array([3, 4, 5, -1, 7, 8, 2, 3, 2147483647, -2147483648], np.int32)
    e = O.find_edges(lut)
    np.testing.assert_array_equal(e, [1, 0, 0, 1, 1, 0, 1, 0, 1, 0])


def test_error_cases():
    with pytest.raises(IndexError):
        O.lut_from_blocks([(-5, 1, b"--", b"--")], 3)
    with pytest.raises(OverflowError):
        O.lut_from_blocks([(1, 2 ** 31 + 5, b"A", b"A")], 3)
    with pytest.raises(IndexError):
        O.fix_zero_idx(np.full(10, -1, np.int32), b"A", b"A")
    # a both-gap column at genome index -1 writes the last entry
    lut = O.lut_from_blocks([(0, 7, b"-A", b"-A")], 4)
    np.testing.assert_array_equal(lut, [7, -1, -1, 6])


def test_xmfa_parser_matches_reference(g, tmp_path):
    """buildindex.parseXMFA against mauve/xmfa.py's output on the reference's
    example file and on synthetic files (wrapped rows, CRLF, score notes)."""
    import json

    import buildindex as B
    for k in range(int(g["n_xmfa"])):
        want = json.loads(bytes(g["x%d_parse" % k]).decode())
        path = tmp_path / ("x%d.xmfa" % k)
        path.write_bytes(bytes(g["x%d_text" % k]))
        got = B.parseXMFA(str(path))  # text-mode read: CRLF becomes LF, as in the reference
        assert [[gr.notes, [list(a) for a in gr.alignments]] for gr in got] == want, k


def test_xmfa_lut_oracle(g):
    """The oracle's LUT on the parsed groups equals the reference buildIndex
    run on the reference parse."""
    import buildindex as B
    for k in range(1, int(g["n_xmfa"])):
        groups = B.parse_xmfa_text(bytes(g["x%d_text" % k]).decode("latin-1").replace("\r\n", "\n"))
        blocks = []
        for gr in groups:
            d = {a.seq_num: a for a in gr.alignments}
            if 1 in d and 2 in d:
                blocks.append((d[1].start_idx, d[2].start_idx, d[1].seq.encode(), d[2].seq.encode()[:len(d[1].seq)]))
        genome, ref = g["x%d_genome" % k], g["x%d_ref" % k]
        lut = O.lut_from_blocks(blocks, len(genome))
        O.fix_zero_idx(lut, genome, ref)
        O.fill_gaps(lut, 300)
        O.smooth_edges(lut, 20)
        np.testing.assert_array_equal(lut, g["x%d_lut" % k])
