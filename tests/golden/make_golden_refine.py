#!/usr/bin/env python3
"""Writes tests/golden/refine.npz: the gapped-alignment pass over LCBs of two
genomes, each window realigned by the reference's own
ProfileAlignFast(anchored) (MUSCLE's AnchoredProfileProfile compiled from the
reference's sources, oracle/_ref/libmauveref.so ref_anchored_align).

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_refine.py

The windows are refineAlignment's (LM/ProgressiveAligner.cpp:1119-1165), from
the library's mvg_refine_windows checked here against the oracle's
restatement (oracle/recursion_oracle.py); windows that are gap windows or
hold bases of one genome only stay as they are.  LCBs: optimal alignments of
seeded random sequences and mutated copies, joined by stretches where one
genome only has bases (up to 6,500 columns, so that some become gap windows).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "mauve-py_gb300")):
    sys.path.insert(0, _p)
import mvg  # noqa: E402
import recursion_oracle as RO  # noqa: E402
import synth  # noqa: E402
from make_golden_anchors import ref_realign, window  # noqa: E402


def lcb(rng, nseg):
    ra, rb = [], []
    for s in range(nseg):
        a, b = window(rng, int(rng.integers(300, 4000)), float(rng.uniform(0.01, 0.2)), int(rng.integers(0, 20)), 3.0)
        ra.append(a)
        rb.append(b)
        if s + 1 < nseg:
            run = int(rng.choice([200, 1500, 5200, 6500]))
            one = synth.random_bases(rng, run)
            gaps = np.full(run, ord("-"), np.uint8)
            ra.append(one if s % 2 == 0 else gaps)
            rb.append(gaps if s % 2 == 0 else one)
    return np.concatenate(ra), np.concatenate(rb)


def main():
    mvg.load_library()
    rng = np.random.default_rng(1119)
    out = {}
    k = 0
    for nseg, maxw in ((3, 20000.0), (4, 20000.0), (2, 1000.0), (5, 3000.0), (3, 600.0), (6, 20000.0)):
        ra, rb = lcb(rng, nseg)
        wins = mvg.refine_windows(ra, rb, maxw)
        assert [tuple(w) for w in wins.tolist()] == [(a, b, int(g)) for a, b, g in RO.refine_windows(ra, rb, maxw)]
        rows_a, rows_b = [], []
        for lo, hi, gap in wins.tolist():
            wa, wb = ra[lo:hi], rb[lo:hi]
            if not gap and (wa != ord("-")).any() and (wb != ord("-")).any():
                wa, wb = ref_realign(wa, wb)
            rows_a.append(wa)
            rows_b.append(wb)
        out["a%d" % k], out["b%d" % k] = ra, rb
        out["w%d" % k] = np.float64(maxw)
        out["oa%d" % k], out["ob%d" % k] = np.concatenate(rows_a), np.concatenate(rows_b)
        out["win%d" % k] = wins
        k += 1
    out["count"] = np.int64(k)
    np.savez_compressed(os.path.join(HERE, "refine.npz"), **out)
    print("wrote %d LCBs, %d windows" % (k, sum(len(out["win%d" % i]) for i in range(k))))


if __name__ == "__main__":
    main()
