"""GPU tests of the search outside LCBs (mvg_search_lcb_gaps[_dev]): the
reference's own SearchLCBGaps output (tests/golden/lcbgaps.npz) reproduced
through the region gather, the pairwise matcher on the two concatenations
and the host steps; and, at a few Mbp, the properties every result of the
search has."""
import numpy as np
import pytest

import mvg
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


def test_search_lcb_gaps_equals_the_reference(ctx):
    """Six genome pairs: matches (order included) and seed weight equal the
    reference's SearchLCBGaps, with host and with device genomes; the
    matcher's list for the two concatenations equals the reference's
    MaskedMemHash list before transposition."""
    import torch
    g = load_golden("lcbgaps.npz")
    total = 0
    for k in range(int(g["search_count"])):
        a, b = g["s%d_a" % k], g["s%d_b" % k]
        ra, rb = g["s%d_ra" % k], g["s%d_rb" % k]
        got, w = ctx.search_lcb_gaps(a, b, ra, rb)
        assert w == int(g["s%d_w" % k]), k
        np.testing.assert_array_equal(got, g["s%d_fin" % k], err_msg=str(k))
        da, db = torch.from_numpy(a.copy()).cuda(), torch.from_numpy(b.copy()).cuda()
        dev, wd = ctx.search_lcb_gaps_dev(da.data_ptr(), len(a), db.data_ptr(), len(b), ra, rb, len(got) + 8)
        np.testing.assert_array_equal(dev, got)
        ca = np.concatenate([a[l - 1:r - 1] for l, r in ra.reshape(-1, 2)] or [np.zeros(0, np.uint8)])
        cb = np.concatenate([b[l - 1:r - 1] for l, r in rb.reshape(-1, 2)] or [np.zeros(0, np.uint8)])
        if len(g["s%d_raw" % k]):
            raw = ctx.pairwise_matches(ca, cb, mvg.get_seed(w, 0))
            np.testing.assert_array_equal(raw, g["s%d_raw" % k], err_msg=str(k))
        total += len(got)
    assert total > 200


def test_region_outside_the_genome_is_an_error(ctx):
    a = synth.random_bases(np.random.default_rng(3), 1000)
    with pytest.raises(IndexError):
        ctx.search_lcb_gaps(a, a, [900, 1100], [1, 100])
    with pytest.raises(ValueError):
        ctx.search_lcb_gaps(a, a, [1, 10, 20], [1, 100])
    m, w = ctx.search_lcb_gaps(a, a, [], [])
    assert m.shape == (0, 3)


def test_search_outside_lcbs_of_a_rearranged_pair_at_4_mbp(ctx):
    """4 Mbp pair with 40 rearrangements; the regions outside 300 stand-in
    LCBs (every LCB's unaligned flanks, collected and sorted as alignPP
    does).  Every match lies inside one region of each genome, is at least 9
    long, no two overlap in either genome, and the result equals the host
    steps applied to the matcher's list for the two concatenations."""
    rng = np.random.default_rng(77)
    b = synth.random_bases(rng, 4_000_000)
    a = synth.mutate(rng, b, 0.02, 400, 5.0, 40, (2_000, 40_000))
    na, nb = len(a), len(b)

    def flanks(n):
        cuts = np.sort(rng.choice(np.arange(2, n - 2000), 300, replace=False))
        out = []
        for c in cuts:
            ln = int(rng.integers(0, 4000))
            out += [int(c), int(min(n + 1, c + ln))]
        r = np.array(out, np.int64).reshape(-1, 2)
        # no overlap between consecutive flanks after the per-genome sort
        keep = np.ones(len(r), bool)
        keep[1:] = r[1:, 0] >= np.maximum.accumulate(r[:, 1])[:-1]
        return np.sort(r[keep].reshape(-1))

    ra, rb = flanks(na), flanks(nb)
    got, w = ctx.search_lcb_gaps(a, b, ra, rb)
    assert len(got) > 100 and (got[:, 2] >= 9).all()
    for q, reg in ((0, ra), (1, rb)):
        lo = np.abs(got[:, q])
        hi = lo + got[:, 2] - 1
        r = reg.reshape(-1, 2)
        idx = np.searchsorted(r[:, 0], lo, side="right") - 1
        assert (idx >= 0).all()
        assert (hi < r[idx, 1]).all(), q
        order = np.argsort(lo, kind="stable")
        assert (lo[order][1:] > hi[order][:-1]).all(), q
    ca = np.concatenate([a[l - 1:r - 1] for l, r in ra.reshape(-1, 2)])
    cb = np.concatenate([b[l - 1:r - 1] for l, r in rb.reshape(-1, 2)])
    raw = ctx.pairwise_matches(ca, cb, mvg.get_seed(w, 0))
    np.testing.assert_array_equal(mvg.lcb_gap_finish(raw, ra, rb), got)
