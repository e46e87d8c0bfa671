#!/usr/bin/env python3
"""Writes tests/golden/recursion.npz: the reference's own
ProgressiveAligner::recurseOnPairs (libMems/ProgressiveAligner.cpp:682-924,
compiled into oracle/_ref/libmauveref.so by oracle/ref_progressive_driver.cpp)
on LCBs of two genomes: the anchors its gap searches find (pairwiseAnchorSearch
per gap, in gap order) and the regions outside the LCB it records.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_recursion.py

Genomes: a random 60 kbp genome and a copy with 3% substitutions (a second
pair at 10%).  LCBs: rows over stretches of both genomes in all four strand
combinations, with stretches where the genomes are not aligned to each other
(one genome's bases, then the other's: the gaps recurseOnPairs searches),
unaligned ends (the regions outside the LCB), LCBs at the first base of a
genome and at its last, one with no column where both genomes are aligned,
and minimum gap lengths 200 (the default) and 60.  Rows are stored as
bitmasks of the columns that hold a base (recurseOnPairs reads nothing else
of them).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import synth  # noqa: E402

R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
P, U, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64
R.ref_recurse_on_pairs.argtypes = [ctypes.c_char_p, U, ctypes.c_char_p, U, ctypes.c_char_p, ctypes.c_char_p, U, I, I,
                                   U, P, U, P, U, P]
R.ref_recurse_on_pairs.restype = I
GAP = ord("-")


def rows(rng, seq_a, seq_b, pre_a, suf_b, n_unalign, lo, hi):
    """Rows for bases seq_a (pre_a bases alone, then the body) and seq_b (the
    body, then suf_b bases alone), the body aligned column by column except
    n_unalign stretches of lo..hi bases shown as A-only then B-only."""
    body = len(seq_a) - pre_a
    assert body == len(seq_b) - suf_b
    ca = [seq_a[:pre_a]]
    cb = [np.full(pre_a, GAP, np.uint8)]
    cuts = np.sort(rng.choice(np.arange(0, max(1, body - hi)), min(n_unalign, max(0, body - hi)), replace=False))
    p = 0
    for c in cuts:
        if c < p:
            continue
        L = int(rng.integers(lo, hi + 1))
        ca += [seq_a[pre_a + p:pre_a + c], seq_a[pre_a + c:pre_a + c + L], np.full(L, GAP, np.uint8)]
        cb += [seq_b[p:c], np.full(L, GAP, np.uint8), seq_b[c:c + L]]
        p = c + L
    ca += [seq_a[pre_a + p:pre_a + body], np.full(suf_b, GAP, np.uint8)]
    cb += [seq_b[p:body], seq_b[body:body + suf_b]]
    return np.concatenate(ca), np.concatenate(cb)


def case(rng, a, b, start, body, pre_a, suf_b, rev_a, rev_b, n_unalign, min_gap, lo=150, hi=1200):
    """An LCB over A[start - pre_a, start + body) and B[start, start + body +
    suf_b) (0-based), in the given strands."""
    sa = a[start - pre_a:start + body]
    sb = b[start:start + body + suf_b]
    row_a, row_b = rows(rng, synth.revcomp(sa) if rev_a else sa, synth.revcomp(sb) if rev_b else sb,
                        pre_a, suf_b, n_unalign, lo, hi)
    left_a, left_b = start - pre_a + 1, start + 1
    out = np.zeros(3 * 200000, np.int64)
    reg = np.zeros(64, np.int64)
    nreg = np.zeros(2, np.uint64)
    n = R.ref_recurse_on_pairs(a.tobytes(), len(a), b.tobytes(), len(b), row_a.tobytes(), row_b.tobytes(), len(row_a),
                               -left_a if rev_a else left_a, -left_b if rev_b else left_b, min_gap,
                               out.ctypes.data, 200000, reg.ctypes.data, 64, nreg.ctypes.data)
    assert n >= 0
    return dict(mask_a=np.packbits(row_a != GAP), mask_b=np.packbits(row_b != GAP), ncols=np.int64(len(row_a)),
                left=np.array([left_a, left_b, int(rev_a), int(rev_b), min_gap], np.int64),
                anchors=out[:3 * n].reshape(-1, 3).copy(), ra=reg[:int(nreg[0])].copy(),
                rb=reg[int(nreg[0]):int(nreg[0] + nreg[1])].copy())


def main():
    rng = np.random.default_rng(682)
    out = {}
    pairs = []
    for div in (0.03, 0.10):
        b = synth.random_bases(rng, 60_000)
        a = synth._substitute(rng, b, rng.random(len(b)) < div)
        pairs.append((a, b))
    cases = []
    for p, (a, b) in enumerate(pairs):
        for rev_a in (False, True):
            for rev_b in (False, True):
                cases.append((p, case(rng, a, b, 5_000, 30_000, 0, 0, rev_a, rev_b, 12, 200)))
                cases.append((p, case(rng, a, b, 8_000, 20_000, 700, 450, rev_a, rev_b, 10, 60, lo=40, hi=600)))
        cases.append((p, case(rng, a, b, 0, 25_000, 0, 300, False, False, 8, 200)))  # first base of A
        cases.append((p, case(rng, a, b, 40_000, 19_000, 900, 1000, True, False, 6, 200)))  # last base of B
        cases.append((p, case(rng, a, b, 3_000, 0, 1500, 1200, False, True, 0, 200)))  # no aligned column
    for k, (p, c) in enumerate(cases):
        out["pair%d" % k] = np.int64(p)
        for key, v in c.items():
            out["c%d_%s" % (k, key)] = v
    for p, (a, b) in enumerate(pairs):
        out["a%d" % p], out["b%d" % p] = a, b
    out["count"] = np.int64(len(cases))
    np.savez_compressed(os.path.join(HERE, "recursion.npz"), **out)
    print("wrote %d LCBs, %d anchors, %d region boundaries" %
          (len(cases), sum(len(c["anchors"]) for _, c in cases), sum(len(c["ra"]) + len(c["rb"]) for _, c in cases)))


if __name__ == "__main__":
    main()
