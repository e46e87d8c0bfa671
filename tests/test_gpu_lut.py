"""GPU index LUT against the golden vectors of the reference's own
buildIndex()/indexutils and against the C oracle at genome size."""
import numpy as np
import pytest

import oracle as O
import synth
from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    import mvg
    c = mvg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def g():
    return load_golden("lut.npz")


@pytest.fixture(scope="module")
def iu():
    import indexutils
    return indexutils


def _blocks(iu, g, k):
    return iu.Blocks(g["b%d_gs" % k], g["b%d_rs" % k], g["b%d_off" % k], g["b%d_rg" % k], g["b%d_rr" % k])


def test_build_index_matches_reference(ctx, g, iu):
    for k in range(int(g["n_build"])):
        blocks = _blocks(iu, g, k)
        genome, ref = g["b%d_genome" % k], g["b%d_ref" % k]
        for v, (fill, width, smooth, radius) in enumerate(g["build_variants"]):
            lut = iu.buildIndexFromGroups(blocks, len(genome), genome, ref, fill_gaps=bool(fill),
                                          max_gap_width=int(width), smooth_edges=bool(smooth),
                                          smoothing_radius=int(radius), ctx=ctx)
            np.testing.assert_array_equal(lut, g["b%d_v%d" % (k, v)], err_msg="case %d variant %d" % (k, v))
        np.testing.assert_array_equal(iu.lutFromBlocks(blocks, len(genome), ctx=ctx), g["b%d_v0" % k])


def test_groups_to_blocks(ctx, g, iu):
    """Blocks.from_groups applies lookupSubAlignment like buildindex.py:116-120."""
    import types
    groups, genome, ref = synth.lut_alignment(1, n_ref=6000, sub=0.02, indel=0.005, nblocks=6, extras=True)
    objs = [types.SimpleNamespace(alignments=[types.SimpleNamespace(seq_num=s, start_idx=st, seq=row.decode())
                                              for s, st, row in grp]) for grp in groups]
    lut = iu.buildIndexFromGroups(objs, len(genome), genome.decode(), ref.decode(), ctx=ctx)
    # the oracle on the blocks of the groups that hold both sequences
    both = [grp for grp in groups if {s for s, _, _ in grp} >= {1, 2}]
    blocks = [(dict((s, st) for s, st, _ in grp)[1], dict((s, st) for s, st, _ in grp)[2],
               dict((s, row) for s, _, row in grp)[1], dict((s, row) for s, _, row in grp)[2]) for grp in both]
    want = O.lut_from_blocks(blocks, len(genome))
    O.fix_zero_idx(want, genome, ref)
    O.fill_gaps(want, 300)
    O.smooth_edges(want, 20)
    np.testing.assert_array_equal(lut, want)


def test_cleanup_passes_host_and_device(ctx, g, iu):
    import torch
    for k in range(int(g["n_lut"])):
        lut0 = g["l%d_in" % k]
        for name, w in (("fill300", 300), ("fill40", 40), ("fill3", 3), ("fill0", 0), ("fillneg", -5)):
            x = lut0.copy()
            iu.fillGaps(x, max_gap_width=w, ctx=ctx)
            np.testing.assert_array_equal(x, g["l%d_%s" % (k, name)], err_msg=name)
            d = torch.from_numpy(lut0.copy()).cuda()
            iu.fillGaps(d, max_gap_width=w, ctx=ctx)
            np.testing.assert_array_equal(d.cpu().numpy(), g["l%d_%s" % (k, name)], err_msg=name + " dev")
        for name, r in (("smooth20", 20), ("smooth5", 5), ("smoothneg", -1)):
            x = lut0.copy()
            iu.smoothEdges(x, smoothing_radius=r, ctx=ctx)
            np.testing.assert_array_equal(x, g["l%d_%s" % (k, name)], err_msg=name)
            d = torch.from_numpy(lut0.copy()).cuda()
            iu.smoothEdges(d, smoothing_radius=r, ctx=ctx)
            np.testing.assert_array_equal(d.cpu().numpy(), g["l%d_%s" % (k, name)], err_msg=name + " dev")
        x = lut0.copy()
        gaps = iu.findGaps(x, ctx=ctx)
        np.testing.assert_array_equal(x, g["l%d_findgaps_lut" % k])
        np.testing.assert_array_equal(gaps, g["l%d_findgaps" % k])
        d = torch.from_numpy(lut0.copy()).cuda()
        dg = iu.findGaps(d, ctx=ctx)
        np.testing.assert_array_equal(dg.cpu().numpy(), g["l%d_findgaps" % k])
        mm = iu.findMismatches(lut0, g["l%d_genome" % k], g["l%d_ref" % k], ctx=ctx)
        np.testing.assert_array_equal(mm.astype(np.uint8), g["l%d_mism" % k])
        assert iu.findDuplicateMappings(lut0, ctx=ctx) == int(g["l%d_dups" % k])
        np.testing.assert_array_equal(iu.findEdges(lut0, ctx=ctx).astype(np.uint8), O.find_edges(lut0))


def test_fix_zero_idx(ctx, g, iu):
    import torch
    for i in range(int(g["n_fz"])):
        lut0, gen, ref = g["fz%d_in" % i], g["fz%d_genome" % i], g["fz%d_ref" % i]
        if int(g["fz%d_status" % i]) == -999:
            with pytest.raises(IndexError):
                iu.fixZeroIdx(lut0.copy(), gen, ref, ctx=ctx)
            continue
        x = lut0.copy()
        iu.fixZeroIdx(x, gen, ref, ctx=ctx)
        np.testing.assert_array_equal(x, g["fz%d_out" % i])
        d = torch.from_numpy(lut0.copy()).cuda()
        iu.fixZeroIdx(d, gen, ref, ctx=ctx)
        np.testing.assert_array_equal(d.cpu().numpy(), g["fz%d_out" % i])


@pytest.mark.parametrize("n,width", [(0, 300), (1, 300), (2, 1), (3, 0), (50, -5), (64, 300), (1000, 1)])
def test_small_and_degenerate(ctx, iu, n, width):
    rng = np.random.default_rng(n + width)
    for trial in range(4):
        lut0 = rng.integers(-1, 8, n).astype(np.int32) if trial < 2 else np.full(n, -1 if trial == 2 else 5,
                                                                                 np.int32)
        for fn_o, fn_g in ((O.fill_gaps, iu.fillGaps), (O.smooth_edges, iu.smoothEdges)):
            a, b = lut0.copy(), lut0.copy()
            fn_o(a, width)
            fn_g(b, width, ctx=ctx)
            np.testing.assert_array_equal(a, b)


def test_clusters_of_overlapping_fills(ctx, iu):
    """Gap starts hidden by an earlier fill, chains of them, and fills that
    share their end position."""
    rng = np.random.default_rng(5)
    for trial in range(40):
        n = 3000
        lut = np.arange(n, dtype=np.int32) + 100
        holes = rng.random(n) < 0.25
        lut[holes] = -1
        isl = rng.random(n) < 0.05
        lut[isl] = rng.integers(0, n + 200, int(isl.sum()))
        for fn_o, fn_g, w in ((O.fill_gaps, iu.fillGaps, 7), (O.smooth_edges, iu.smoothEdges, 5),
                              (O.fill_gaps, iu.fillGaps, 300)):
            a, b = lut.copy(), lut.copy()
            fn_o(a, w)
            fn_g(b, w, ctx=ctx)
            np.testing.assert_array_equal(a, b, err_msg="trial %d width %d" % (trial, w))


def test_genome_size_pipeline_against_oracle(ctx, iu):
    """4.6 Mbp: the whole buildIndex LUT path on the GPU equals the oracle's."""
    gs, rs, off, rg, rr, genome, ref = synth.lut_alignment_fast(11, n_ref=4_600_000, sub=0.02, indel=0.001,
                                                                nblocks=200)
    n = len(genome)
    blocks = iu.Blocks(gs, rs, off, rg, rr)
    lut = iu.buildIndexFromGroups(blocks, n, genome, ref, ctx=ctx)
    ref_lut = np.empty(n, np.int32)
    assert O.lib().mo_lut_from_blocks(O._p(gs), O._p(rs), O._p(off), O._p(rg), O._p(rr), len(gs), O._p(ref_lut),
                                      n) == 0
    raw = ref_lut.copy()
    O.fix_zero_idx(ref_lut, genome, ref)
    O.fill_gaps(ref_lut, 300)
    O.smooth_edges(ref_lut, 20)
    np.testing.assert_array_equal(lut, ref_lut)
    np.testing.assert_array_equal(iu.lutFromBlocks(blocks, n, ctx=ctx), raw)
    import torch
    t = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (gs, rs, off.view(np.int64), rg, rr, genome,
                                                                     ref)]
    d_lut = torch.empty(n, dtype=torch.int32, device="cuda")
    iu.buildIndexLutDev(*[x.data_ptr() for x in t[:5]], len(gs), t[5].data_ptr(), len(genome), t[6].data_ptr(),
                        len(ref), d_lut.data_ptr(), n, ctx=ctx)
    np.testing.assert_array_equal(d_lut.cpu().numpy(), ref_lut)
    # random LUT with dense gap structure at genome size
    big = synth.lut_random(3, n=2_000_000)
    a, b = big.copy(), big.copy()
    O.fill_gaps(a, 300)
    iu.fillGaps(b, ctx=ctx)
    np.testing.assert_array_equal(a, b)
    a, b = big.copy(), big.copy()
    O.smooth_edges(a, 20)
    iu.smoothEdges(b, ctx=ctx)
    np.testing.assert_array_equal(a, b)


def test_errors(ctx, iu):
    # a write at genome index < -1 (start 0 with a leading both-gap column
    # twice) is an IndexError in numpy only when below -n
    blocks = iu.Blocks([-5], [1], [0, 2], np.frombuffer(b"--", np.uint8), np.frombuffer(b"--", np.uint8))
    with pytest.raises(IndexError):
        iu.lutFromBlocks(blocks, 3, ctx=ctx)
    blocks = iu.Blocks([1], [2 ** 31 + 5], [0, 1], np.frombuffer(b"A", np.uint8), np.frombuffer(b"A", np.uint8))
    with pytest.raises(OverflowError):
        iu.lutFromBlocks(blocks, 3, ctx=ctx)
    with pytest.raises(IndexError):
        iu.fixZeroIdx(np.full(10, -1, np.int32), b"A", b"A", ctx=ctx)


def test_build_index_from_xmfa(ctx, g, tmp_path):
    """XMFA file -> parse -> LUT on the GPU equals the reference's buildIndex
    run on its own parse of the same file (the reference's example file and
    synthetic ones)."""
    import buildindex as B
    for k in range(int(g["n_xmfa"])):
        path = tmp_path / ("x%d.xmfa" % k)
        path.write_bytes(bytes(g["x%d_text" % k]))
        if k == 0:
            lut = B.buildIndexFromXMFA(str(path), 700, fill_gaps=False, smooth_edges=True, ctx=ctx)
        else:
            genome, ref = g["x%d_genome" % k], g["x%d_ref" % k]
            lut = B.buildIndexFromXMFA(str(path), len(genome), genome, ref, ctx=ctx)
        np.testing.assert_array_equal(lut, g["x%d_lut" % k], err_msg="xmfa case %d" % k)
