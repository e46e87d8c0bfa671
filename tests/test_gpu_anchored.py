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
