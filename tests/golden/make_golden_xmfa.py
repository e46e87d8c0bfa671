#!/usr/bin/env python3
"""Writes tests/golden/xmfa.npz: XMFA text from the reference's own writer
(GenericIntervalList::WriteStandardAlignment, libMems/IntervalList.h:353-440,
compiled into oracle/_ref/libmauveref.so as ref_xmfa_write) for pairwise
block lists over two seeded random genomes.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_xmfa.py

Each case stores the file names, the backbone name, per block the two signed
starts (negative = reverse strand, 0 = absent), the column offsets, the two
gap-patterned rows ('N' = a base, '-' = a gap) and the text the reference
wrote; the reference fills the rows from the genomes itself (reverse
complement for the reverse strand).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
vp, u64, i64, cp = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_char_p
R.ref_xmfa_write.restype = i64
R.ref_xmfa_write.argtypes = [cp, u64, cp, u64, cp, cp, cp, i64, vp, vp, cp, cp, vp, u64]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def pattern(rng, nbase, ncol):
    """A row of ncol columns holding nbase bases at random columns."""
    row = np.full(ncol, ord("-"), np.uint8)
    row[np.sort(rng.choice(ncol, nbase, replace=False))] = ord("N")
    return row


def make_case(rng, la, lb, nblocks, absent_first=False, absent_later=False, empty_block=False):
    starts, rows_a, rows_b, cols = [], [], [], [0]
    for k in range(nblocks):
        ncol = int(rng.choice([1, 79, 80, 81, 160, 250, int(rng.integers(2, 400))]))
        na = int(rng.integers(max(1, ncol // 2), ncol + 1))
        nb = int(rng.integers(max(1, ncol // 2), ncol + 1))
        if empty_block and k == 2:
            ncol, na, nb = 0, 0, 0
        sa = int(rng.integers(1, la - na)) if na else 0
        sb = int(rng.integers(1, lb - nb)) if nb else 0
        if rng.random() < 0.4:
            sb = -sb
        if (absent_first and k == 0) or (absent_later and k == 3):
            sa, na = 0, 0
        starts += [sa, sb]
        rows_a.append(pattern(rng, na, ncol))
        rows_b.append(pattern(rng, nb, ncol))
        cols.append(cols[-1] + ncol)
    return (np.array(starts, np.int64), np.array(cols, np.uint64),
            np.concatenate(rows_a) if rows_a else np.zeros(0, np.uint8),
            np.concatenate(rows_b) if rows_b else np.zeros(0, np.uint8))


def main():
    rng = np.random.default_rng(20261205)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    ga, gb = rng.choice(acgt, 5000), rng.choice(acgt, 4500)
    specs = [("/data/genome.fa", "/data/ref.fasta", "out.xmfa.backbone", dict(nblocks=7, absent_first=True,
                                                                              absent_later=True, empty_block=True)),
             ("/data/both.gbk", "/data/both.gbk", "", dict(nblocks=5)),
             ("x/a.seq", "x/b.raw", "bb", dict(nblocks=4, absent_later=True)),
             ("a.FAS", "dir.v2/b", "", dict(nblocks=6)),
             ("a.gb", "b.GB", "", dict(nblocks=0))]
    g = {"ga": ga, "gb": gb}
    for k, (fa, fb, bb, kw) in enumerate(specs):
        starts, cols, ra, rb = make_case(rng, len(ga), len(gb), **kw)
        out = ctypes.create_string_buffer(1 << 20)
        n = R.ref_xmfa_write(ga.tobytes(), len(ga), gb.tobytes(), len(gb), fa.encode(), fb.encode(), bb.encode(),
                             len(cols) - 1, _p(starts), _p(cols), ra.tobytes(), rb.tobytes(), out, 1 << 20)
        assert n >= 0
        g.update({"fa%d" % k: np.frombuffer(fa.encode(), np.uint8), "fb%d" % k: np.frombuffer(fb.encode(), np.uint8),
                  "bb%d" % k: np.frombuffer(bb.encode(), np.uint8), "starts%d" % k: starts, "cols%d" % k: cols,
                  "ra%d" % k: ra, "rb%d" % k: rb, "text%d" % k: np.frombuffer(out.raw[:n], np.uint8)})
    g["count"] = np.int64(len(specs))
    np.savez_compressed(os.path.join(HERE, "xmfa.npz"), **g)
    print("xmfa.npz: %d cases" % len(specs))


if __name__ == "__main__":
    main()
