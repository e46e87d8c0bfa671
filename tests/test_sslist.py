"""The .sslist cache file (FileSML::Create / LoadFile2,
libMems/FileSML.cpp:401-459, 120-195) against what the reference's own code
puts in it (tests/golden/sslist.npz, made by make_golden_sslist.py).

CPU tests: files laid out by the reference's compiled SMLHeader are read
back with every field, and damaged files give LoadFile2's failure codes.
GPU test: mvg_sslist_write's header, packed words and positions match the
reference's."""
import os
import struct

import numpy as np
import pytest

import mvg

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "sslist.npz"))
LAYOUT = GOLD["layout"]  # sizeof(SMLHeader), offsets of its members in order
(SIZE, O_VERSION, O_ABITS, O_SEED, O_SLEN, O_SWEIGHT, O_LENGTH, O_UNIQUE, O_WORDSIZE, O_ENDIAN, O_ID, O_CIRC,
 O_TABLE, O_DESC, TABLE_LEN) = [int(x) for x in LAYOUT]


def ref_file(k, version=5):
    hdr = bytearray(GOLD["s%d_header" % k].tobytes())
    hdr[O_VERSION:O_VERSION + 4] = struct.pack("<I", version)
    return bytes(hdr) + GOLD["s%d_words" % k].tobytes() + GOLD["s%d_pos" % k].tobytes()


def test_header_layout_is_the_reference_struct():
    assert SIZE == 2352 and TABLE_LEN == 255
    assert (O_VERSION, O_ABITS, O_SEED, O_SLEN, O_SWEIGHT, O_LENGTH, O_UNIQUE) == (0, 4, 8, 16, 20, 24, 32)
    assert (O_WORDSIZE, O_ENDIAN, O_ID, O_CIRC, O_TABLE, O_DESC) == (36, 40, 42, 44, 45, 300)


@pytest.mark.parametrize("k", range(int(GOLD["n"])))
def test_reader_parses_reference_layout(tmp_path, k):
    mvg.load_library()
    p = tmp_path / "x.sslist"
    p.write_bytes(ref_file(k))
    info, words, pos = mvg.sslist_read(str(p))
    seq = GOLD["s%d_seq" % k]
    assert info.seed == int(GOLD["s%d_seed" % k])
    assert info.length == len(seq)
    assert info.seed_length == mvg.seed_length(info.seed) and info.seed_weight == mvg.seed_weight(info.seed)
    assert info.circular == 0 and info.status == 0
    np.testing.assert_array_equal(words, GOLD["s%d_words" % k])
    np.testing.assert_array_equal(pos, GOLD["s%d_pos" % k])


def test_reader_failure_codes(tmp_path):
    mvg.load_library()
    good = ref_file(1)
    cases = {2: good[:SIZE - 1], 3: ref_file(1, version=4), 4: good[:SIZE + 4]}
    for status, data in cases.items():
        p = tmp_path / ("bad%d.sslist" % status)
        p.write_bytes(data)
        with pytest.raises(RuntimeError, match="status %d" % status):
            mvg.sslist_read(str(p))
    with pytest.raises(RuntimeError, match="status 1"):
        mvg.sslist_read(str(tmp_path / "missing.sslist"))


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(int(GOLD["n"])))
def test_writer_matches_reference(tmp_path, k):
    import build as pkg_build
    pkg_build.build()
    ctx = mvg.Context(0)
    try:
        seq = GOLD["s%d_seq" % k]
        seed = int(GOLD["s%d_seed" % k])
        p = tmp_path / "w.sslist"
        ctx.sslist_write(seq.tobytes(), seed, str(p))
    finally:
        ctx.close()
    data = np.frombuffer(p.read_bytes(), np.uint8)
    ref_hdr = GOLD["s%d_header" % k]
    # every member the reference sets; word_size and little_endian it leaves
    # uninitialised (written here as 32 and 1)
    mine = data[:SIZE].copy()
    assert struct.unpack_from("<I", mine, O_VERSION)[0] == 5
    assert struct.unpack_from("<I", mine, O_WORDSIZE)[0] == 32 and mine[O_ENDIAN] == 1
    mine[O_VERSION:O_VERSION + 4] = 0
    mine[O_WORDSIZE:O_WORDSIZE + 4] = 0
    mine[O_ENDIAN] = 0
    np.testing.assert_array_equal(mine, ref_hdr)
    words = GOLD["s%d_words" % k]
    mw = np.frombuffer(data[SIZE:SIZE + 4 * len(words)].tobytes(), np.uint32)
    # the two pad words after the sequence are uninitialised in the reference
    np.testing.assert_array_equal(mw[:-2], words[:-2])
    pos = np.frombuffer(data[SIZE + 4 * len(words):].tobytes(), np.uint32)
    ref_pos, ref_mer = GOLD["s%d_pos" % k], GOLD["s%d_mer" % k]
    assert len(pos) == len(ref_pos)
    # same mer order; the reference's sort is unstable, so positions with
    # equal mers may come in another order: compare each run as a set
    starts = np.flatnonzero(np.concatenate([[True], ref_mer[1:] != ref_mer[:-1]]))
    ends = np.concatenate([starts[1:], [len(ref_mer)]])
    for a, b in zip(starts, ends):
        assert sorted(pos[a:b]) == sorted(ref_pos[a:b])
