"""GPU tests of the XMFA writer (csrc/xmfa.cu): the text equals what the
reference's own WriteStandardAlignment wrote for the same blocks
(tests/golden/xmfa.npz), and the written file reads back through the
buildIndex reader with the same rows and coordinates."""
import numpy as np
import pytest

import buildindex
import mvg
from conftest import load_golden

pytestmark = pytest.mark.gpu

COMP = bytes.maketrans(b"ACGT", b"TGCA")


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


def fill_rows(genomes, starts, cols, patterns):
    """The rows the reference's GetAlignment makes from the genomes: the
    pattern's base columns filled in order, reverse complement for a
    reverse-strand start, all gaps for an absent sequence."""
    rows = [p.copy() for p in patterns]
    lengths = np.zeros(len(starts), np.int64)
    for b in range(len(cols) - 1):
        c0, c1 = int(cols[b]), int(cols[b + 1])
        for q in range(2):
            pat = rows[q][c0:c1]
            at = np.nonzero(pat != ord("-"))[0]
            s = int(starts[2 * b + q])
            lengths[2 * b + q] = len(at)
            if s == 0:
                continue
            seg = genomes[q][abs(s) - 1:abs(s) - 1 + len(at)].tobytes()
            if s < 0:
                seg = seg.translate(COMP)[::-1]
            pat[at] = np.frombuffer(seg, np.uint8)
    return rows, lengths


def test_xmfa_text_equals_reference_writer(ctx):
    g = load_golden("xmfa.npz")
    genomes = (g["ga"], g["gb"])
    for k in range(int(g["count"])):
        (ra, rb), lengths = fill_rows(genomes, g["starts%d" % k], g["cols%d" % k], [g["ra%d" % k], g["rb%d" % k]])
        text = ctx.xmfa_write(g["fa%d" % k].tobytes().decode(), g["fb%d" % k].tobytes().decode(), g["starts%d" % k],
                              lengths, ra, rb, g["cols%d" % k], backbone_file=g["bb%d" % k].tobytes().decode())
        assert text == g["text%d" % k].tobytes(), "case %d" % k


def test_xmfa_reads_back(ctx):
    """Written, then parsed by the buildIndex reader (the in-repo stand-in
    for libnano's parser): one group per block, the rows and coordinates of
    each written sequence."""
    g = load_golden("xmfa.npz")
    k = 1  # both sequences in every block
    starts, cols = g["starts%d" % k], g["cols%d" % k]
    (ra, rb), lengths = fill_rows((g["ga"], g["gb"]), starts, cols, [g["ra%d" % k], g["rb%d" % k]])
    text = ctx.xmfa_write("A.fa", "B.fa", starts, lengths, ra, rb, cols).decode()
    groups = buildindex.parse_xmfa_text(text)
    assert len(groups) == len(cols) - 1
    for b, grp in enumerate(groups):
        for q, sub in enumerate(grp.alignments):
            s = int(starts[2 * b + q])
            assert sub.seq_num == q + 1 and sub.start_idx == abs(s) and sub.end_idx == abs(s) + lengths[2 * b + q] - 1
            assert sub.strand == ("+" if s > 0 else "-")
            assert sub.seq == (ra if q == 0 else rb)[int(cols[b]):int(cols[b + 1])].tobytes().decode()


def test_xmfa_device_rows_into_pinned_memory(ctx):
    """Context.xmfa_write_dev with the rows in device memory writes the
    reference's text into a pinned host buffer; with no buffer it returns
    the size needed, and a buffer one byte short is refused."""
    import torch
    g = load_golden("xmfa.npz")
    for k in range(int(g["count"])):
        (ra, rb), lengths = fill_rows((g["ga"], g["gb"]), g["starts%d" % k], g["cols%d" % k],
                                      [g["ra%d" % k], g["rb%d" % k]])
        names = (g["fa%d" % k].tobytes().decode(), g["fb%d" % k].tobytes().decode())
        bb = g["bb%d" % k].tobytes().decode()
        d_a = torch.from_numpy(np.concatenate([ra, np.zeros(1, np.uint8)])).cuda()
        d_b = torch.from_numpy(np.concatenate([rb, np.zeros(1, np.uint8)])).cuda()
        args = (*names, g["starts%d" % k], lengths, d_a.data_ptr(), d_b.data_ptr(), g["cols%d" % k])
        need = ctx.xmfa_write_dev(*args, backbone_file=bb)
        want = g["text%d" % k].tobytes()
        assert need == len(want)
        out = torch.zeros(need + 1, dtype=torch.uint8, pin_memory=True)
        if need > 1:
            with pytest.raises(OverflowError):
                ctx.xmfa_write_dev(*args, out.data_ptr(), need - 1, backbone_file=bb)
        assert ctx.xmfa_write_dev(*args, out.data_ptr(), need, backbone_file=bb) == need
        assert out[:need].numpy().tobytes() == want, "case %d" % k
