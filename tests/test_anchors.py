"""Anchor columns of two-genome alignment windows (mvg_anchor_columns)
against the reference's own MUSCLE (tests/golden/anchors.npz, written by
make_golden_anchors.py from FindAnchorColsPP compiled from the reference's
sources).  Host code only: no GPU."""
import numpy as np
import pytest

import mvg
from conftest import load_golden


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as pkg_build
    pkg_build.build()


def test_anchor_columns_equal_the_reference():
    """60 windows of 30-6,000 columns at 1-30% divergence, with lowercase
    bases, N and IUPAC codes, terminal gaps and long one-sided gap runs: the
    same anchor columns, in order, as the reference's MUSCLE."""
    g = load_golden("anchors.npz")
    total = 0
    for k in range(int(g["count"])):
        got = mvg.anchor_columns(g["a%d" % k], g["b%d" % k])
        np.testing.assert_array_equal(got, g["cols%d" % k], err_msg="window %d" % k)
        total += len(got)
    assert total > 500


def test_problems_cover_the_window():
    """The ranges between anchor columns tile the window, and each range's
    problem is its two rows without gap characters."""
    g = load_golden("anchors.npz")
    for k in range(0, int(g["count"]), 7):
        ra, rb = g["a%d" % k], g["b%d" % k]
        probs = mvg.anchored_problems(ra, rb)
        edges = [p[0] for p in probs]
        assert edges[0][0] == 0 and edges[-1][1] == len(ra)
        assert all(x[1] == y[0] for x, y in zip(edges[:-1], edges[1:]))
        for (lo, hi), a, b in probs:
            np.testing.assert_array_equal(a, ra[lo:hi][ra[lo:hi] != ord("-")])
            np.testing.assert_array_equal(b, rb[lo:hi][rb[lo:hi] != ord("-")])


def test_short_and_empty_windows():
    assert len(mvg.anchor_columns(b"", b"")) == 0
    assert len(mvg.anchor_columns(b"ACGT" * 5, b"ACGT" * 5)) == 0  # 21 columns or fewer: nothing smooths
    with pytest.raises(ValueError):
        mvg.anchor_columns(b"ACG", b"AC")
