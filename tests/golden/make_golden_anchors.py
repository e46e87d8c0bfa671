#!/usr/bin/env python3
"""Writes tests/golden/anchors.npz: anchor columns from the reference's own
MUSCLE (FindAnchorColsPP after PrepareMSAforScoring, set up as
MuscleInterface::ProfileAlignFast does; compiled into
oracle/_ref/libmauveref.so as ref_anchor_cols) for windows of two-genome
alignments.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_anchors.py

Windows: the optimal NWSmall alignment (the oracle's) of a seeded random
sequence and a mutated copy, at 1-30% divergence and 30-6,000 bases, some
with lowercase bases, N and IUPAC codes, terminal gaps and long one-sided
gap runs; each case stores the two rows, the reference's anchor columns and
the reference's anchored realignment of the window (ProfileAlignFast with
anchored = true: AnchoredProfileProfile, as ref_anchored_align).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")):
    sys.path.insert(0, _p)
import oracle as O  # noqa: E402
import synth  # noqa: E402

R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
R.ref_anchor_cols.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
R.ref_anchor_cols.restype = ctypes.c_int
R.ref_anchored_align.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                                 ctypes.c_int]
R.ref_anchored_align.restype = ctypes.c_int
ACGT = np.frombuffer(b"ACGT", np.uint8)


def rows_of(a, b, path):
    ra, rb, i, j = [], [], 0, 0
    for e in path:
        if e == "M":
            ra.append(a[i])
            rb.append(b[j])
            i += 1
            j += 1
        elif e == "D":
            ra.append(a[i])
            rb.append(ord("-"))
            i += 1
        else:
            ra.append(ord("-"))
            rb.append(b[j])
            j += 1
    return np.array(ra, np.uint8), np.array(rb, np.uint8)


def window(rng, n, div, nindel, mean_indel):
    a = synth.random_bases(rng, n)
    b = synth.mutate(rng, a, div, nindel, mean_indel, 0, (1, 2))
    path, _ = O.nw_align(np.searchsorted(ACGT, a).astype(np.uint8), np.searchsorted(ACGT, b).astype(np.uint8))
    return rows_of(a, b, path)


def ref_cols(ra, rb):
    out = np.zeros(max(1, len(ra)), np.uint32)
    n = R.ref_anchor_cols(ra.tobytes(), rb.tobytes(), len(ra), out.ctypes.data, len(out))
    assert n >= 0
    return out[:n].copy()


def ref_realign(ra, rb):
    cap = 2 * len(ra) + 16
    oa, ob = ctypes.create_string_buffer(cap), ctypes.create_string_buffer(cap)
    n = R.ref_anchored_align(ra.tobytes(), rb.tobytes(), len(ra), oa, ob, cap)
    assert n >= 0
    return np.frombuffer(oa.raw[:n], np.uint8).copy(), np.frombuffer(ob.raw[:n], np.uint8).copy()


def main():
    rng = np.random.default_rng(96)
    cases = []
    for k in range(60):
        n = int(np.exp(rng.uniform(np.log(30), np.log(6000))))
        ra, rb = window(rng, n, float(rng.uniform(0.01, 0.30)), int(rng.integers(0, max(1, n // 150))), 3.0)
        if k % 5 == 1:  # lowercase runs
            m = rng.random(len(ra)) < 0.2
            ra = np.where(m & (ra != ord("-")), ra | 0x20, ra).astype(np.uint8)
        if k % 5 == 2:  # wildcards and IUPAC codes
            for r in (ra, rb):
                m = (rng.random(len(r)) < 0.03) & (r != ord("-"))
                r[m] = rng.choice(np.frombuffer(b"NRYKMSWN", np.uint8), int(m.sum()))
        if k % 5 == 3:  # a long one-sided run in the middle and terminal gaps
            mid = len(ra) // 2
            run = int(rng.integers(50, 400))
            ra = np.concatenate([np.full(7, ord("-"), np.uint8), ra[:mid], synth.random_bases(rng, run), ra[mid:]])
            rb = np.concatenate([synth.random_bases(rng, 7), rb[:mid], np.full(run, ord("-"), np.uint8), rb[mid:]])
        cases.append((ra, rb, ref_cols(ra, rb), *ref_realign(ra, rb)))
    out = {"count": np.int64(len(cases))}
    for k, (ra, rb, cols, oa, ob) in enumerate(cases):
        out["a%d" % k], out["b%d" % k], out["cols%d" % k] = ra, rb, cols
        out["oa%d" % k], out["ob%d" % k] = oa, ob
    np.savez_compressed(os.path.join(HERE, "anchors.npz"), **out)
    print("wrote %d windows, %d anchor columns" % (len(cases), sum(len(c[2]) for c in cases)))


if __name__ == "__main__":
    main()
