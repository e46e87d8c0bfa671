"""GPU test of the anchored realignment of alignment windows
(Context.anchored_realign): the reference's own AnchoredProfileProfile
output (tests/golden/anchors.npz) reproduced through mvg_anchor_columns, one
batched gap-DP call and mvg_path_rows."""
import numpy as np
import pytest

import mvg
from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


def test_anchored_realign_equals_the_reference(ctx):
    """Every window whose bases are A/C/G/T (either case) realigned in one
    call: rows byte-identical to the reference's ProfileAlignFast(anchored)
    output."""
    g = load_golden("anchors.npz")
    acgt = np.frombuffer(b"ACGTacgt-", np.uint8)
    ids = [k for k in range(int(g["count"]))
           if np.isin(g["a%d" % k], acgt).all() and np.isin(g["b%d" % k], acgt).all()]
    assert len(ids) >= 40
    out = ctx.anchored_realign([(g["a%d" % k], g["b%d" % k]) for k in ids])
    for k, (ra, rb) in zip(ids, out):
        assert ra == g["oa%d" % k].tobytes(), k
        assert rb == g["ob%d" % k].tobytes(), k


def test_refine_alignment_pass_equals_reference_windows(ctx):
    """The gapped-alignment pass over six LCBs (tests/golden/refine.npz):
    refineAlignment's windows, each window that is not a gap window and holds
    bases of both genomes realigned (all windows of all LCBs in one batch),
    equal to the LCB rows built from the reference's own
    ProfileAlignFast(anchored) output for each window."""
    g = load_golden("refine.npz")
    n = int(g["count"])
    by_w = {}
    for k in range(n):
        by_w.setdefault(float(g["w%d" % k]), []).append(k)
    for maxw, ks in by_w.items():
        out = ctx.refine_alignment([(g["a%d" % k], g["b%d" % k]) for k in ks], max_window_size=maxw)
        for k, (ra, rb) in zip(ks, out):
            assert ra == g["oa%d" % k].tobytes(), k
            assert rb == g["ob%d" % k].tobytes(), k
            np.testing.assert_array_equal(mvg.refine_windows(g["a%d" % k], g["b%d" % k], maxw), g["win%d" % k])


def test_iterative_refinement_equals_the_reference(ctx):
    """The final iterative-refinement pass (Context.iterative_refine: every
    RefineFast column window of every LCB in one gap-DP call) and both passes
    together (Context.gapped_alignment) give the reference's own
    refineAlignment rows on 11 LCBs (tests/golden/refine.npz)."""
    g = load_golden("refine.npz")
    by_w = {}
    for k in range(int(g["count"])):
        by_w.setdefault(float(g["w%d" % k]), []).append(k)
    for maxw, ks in by_w.items():
        lcbs = [(g["a%d" % k], g["b%d" % k]) for k in ks]
        for (ra, rb), k in zip(ctx.iterative_refine(lcbs, max_window_size=maxw), ks):
            assert ra == g["ia%d" % k].tobytes() and rb == g["ib%d" % k].tobytes(), k
        for (ra, rb), k in zip(ctx.gapped_alignment(lcbs, max_window_size=maxw), ks):
            assert ra == g["fa%d" % k].tobytes() and rb == g["fb%d" % k].tobytes(), k
