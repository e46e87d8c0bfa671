"""Backbone detection's homology HMM (mvg_hmm_backbone_params,
mvg_homologous_segments) against the reference's own findHssHomologyHMM and
parameter set-up (tests/golden/homology.npz).  Host only: no GPU."""
import numpy as np
import pytest

import mvg
from conftest import load_golden


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as pkg_build
    pkg_build.build()


def test_parameters_equal_the_reference_bit_for_bit():
    """applyBackbone's parameters (adapted HOXD matrix, progressiveMauve's
    transition defaults, adaptToPercentIdentity) for 5 GC contents x 3
    identities, every double identical."""
    g = load_golden("homology.npz")
    for (gc, ident), want in zip(g["param_grid"], g["params"]):
        got = mvg.hmm_backbone_params(gc, 1e-5, 1e-9, ident).to_array()
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (gc, ident)


def test_segments_equal_the_reference():
    """Homologous column ranges of 30 alignments (homologous, unrelated and
    one-genome stretches; lowercase and N; one of 150,000 columns), all in
    one call per flag setting, for both-sides homologous (as
    detectAndApplyBackbone runs it) and the two one-sided settings (the
    symbol string reversed when only the right end is homologous)."""
    g = load_golden("homology.npz")
    n = int(g["count"])
    params = []
    for k in range(n):
        gc, ident = g["param_grid"][int(g["p%d" % k])]
        params.append(mvg.hmm_backbone_params(gc, 1e-5, 1e-9, ident))
    total = 0
    for lh, rh in ((1, 1), (0, 1), (1, 0)):
        for k in range(n):
            got = mvg.homologous_segments([(g["a%d" % k], g["b%d" % k])], params[k], bool(lh), bool(rh))[0]
            np.testing.assert_array_equal(got, g["s%d_%d%d" % (k, lh, rh)], err_msg="%d %d%d" % (k, lh, rh))
            total += len(got)
    assert total > 100


def test_many_lcbs_in_one_call_and_edge_cases():
    """LCBs batched in one call give each LCB's own segments; an empty LCB
    and an all-gap-in-one-genome LCB have none; bad identities are refused."""
    g = load_golden("homology.npz")
    p = mvg.hmm_backbone_params(0.5)
    lcbs = [(g["a%d" % k], g["b%d" % k]) for k in range(6)]
    batch = mvg.homologous_segments(lcbs, p)
    for k in range(6):
        np.testing.assert_array_equal(batch[k], mvg.homologous_segments([lcbs[k]], p)[0])
    empty = np.zeros(0, np.uint8)
    one = np.frombuffer(b"ACGTACGT" * 50, np.uint8)
    assert mvg.homologous_segments([(empty, empty)], p)[0].shape == (0, 2)
    segs = mvg.homologous_segments([(one, np.full(len(one), ord("-"), np.uint8))], p)[0]
    assert segs.shape == (0, 2)
    with pytest.raises(ValueError):
        mvg.hmm_backbone_params(0.5, pct_identity=0.0)
