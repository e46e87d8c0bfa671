"""LCBs with greedy breakpoint elimination for collinear genomes
(mvg_collinear_lcbs) against the reference's own collinear branch of
alignProfileToProfile (libMems/ProgressiveAligner.cpp:2281-2303;
tests/golden/lcbs.npz).  No GPU."""
import numpy as np
import pytest

import mvg
from conftest import load_golden


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as pkg_build
    pkg_build.build()


def _cases(g):
    mo, lc, do = g["match_off"], g["lcb_case"], g["deleted_off"]
    for k in range(len(mo) - 1):
        off = g["lcb_off"][lc[k]:lc[k + 1]]
        lcbs = [g["lcb_matches"][off[j]:off[j + 1]] for j in range(len(off) - 1)]
        yield g["matches"][mo[k]:mo[k + 1]], lcbs, g["deleted"][do[k]:do[k + 1]]


def test_lcbs_equal_the_reference():
    """48 match lists (hand-made edge cases, then permuted and inverted
    blocks with random extra matches): the LCBs, their matches' order and
    the deleted matches equal the reference's."""
    g = load_golden("lcbs.npz")
    deleted = kept = 0
    for k, (m, want, want_del) in enumerate(_cases(g)):
        got, got_del = mvg.collinear_lcbs(m)
        assert len(got) == len(want), k
        for x, y in zip(got, want):
            np.testing.assert_array_equal(x, y, err_msg=str(k))
        np.testing.assert_array_equal(got_del, want_del, err_msg=str(k))
        deleted += len(got_del)
        kept += sum(len(x) for x in got)
    assert deleted > 1000 and kept > 1000


def test_every_match_is_kept_or_deleted_once():
    """The LCBs and the deleted list partition the input."""
    g = load_golden("lcbs.npz")
    for m, _, _ in _cases(g):
        got, got_del = mvg.collinear_lcbs(m)
        both = np.concatenate(got + [got_del]) if got else got_del
        key = lambda a: sorted(map(tuple, a.tolist()))  # noqa: E731
        assert key(both) == key(m)


def test_collinear_blocks_stay_one_lcb_with_nothing_deleted():
    """Matches in the same order and strand in both genomes form one LCB
    with no breakpoint to remove; a reversed pair in an inverted order is
    collinear too."""
    m = np.array([(10 + 100 * i, 50 + 120 * i, 30) for i in range(20)], np.int64)
    got, dl = mvg.collinear_lcbs(m[::-1])
    assert len(got) == 1 and len(dl) == 0
    np.testing.assert_array_equal(got[0], m)
    got, dl = mvg.collinear_lcbs([(5, -300, 20), (100, -7, 20)])
    assert len(got) == 1 and len(dl) == 0


def test_rejects_undefined_and_empty_matches():
    with pytest.raises(ValueError):
        mvg.collinear_lcbs([(5, 0, 20)])
    with pytest.raises(ValueError):
        mvg.collinear_lcbs([(5, 9, 0)])
    got, dl = mvg.collinear_lcbs(np.zeros((0, 3), np.int64))
    assert got == [] and len(dl) == 0
