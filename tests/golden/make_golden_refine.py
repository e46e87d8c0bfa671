#!/usr/bin/env python3
"""Writes tests/golden/refine.npz: the gapped-alignment pass over LCBs of two
genomes, each window realigned by the reference's own
ProfileAlignFast(anchored) (MUSCLE's AnchoredProfileProfile compiled from the
reference's sources, oracle/_ref/libmauveref.so ref_anchored_align).

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_refine.py

The expected rows are the reference's own refineAlignment
(LM/ProgressiveAligner.cpp:1119-1230, compiled from its sources with
oracle/ref_progressive_driver.cpp as ref_refine_alignment): oa/ob after the
gapped-alignment pass (profile_aln = true), ia/ib after the final
iterative-refinement pass alone (profile_aln = false: RefineFast per
window), fa/fb after the first pass then the second, as a two-genome
progressiveMauve run makes them.  The
script also rebuilds them window by window -- refineAlignment's windows
(:1015-1165) from the library's mvg_refine_windows, checked against the
oracle's restatement (oracle/recursion_oracle.py), each window that is not a
gap window and holds bases of both genomes realigned by ref_anchored_align --
and requires the two to agree, which pins the windows to the reference.
LCBs: optimal alignments of seeded random sequences and mutated copies,
joined by stretches where one genome only has bases (up to 6,500 columns, so
that some become gap windows); three of them made worse by splitting 2-10%
of their aligned columns into one-sided pairs.
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
from make_golden_anchors import R, ref_realign, window  # noqa: E402

R.ref_refine_alignment.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                   ctypes.c_uint64, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint64]
R.ref_refine_alignment.restype = ctypes.c_int64


def ref_refine(ra, rb, maxw, mode=0):
    cap = 2 * len(ra) + 64
    oa, ob = ctypes.create_string_buffer(cap), ctypes.create_string_buffer(cap)
    n = R.ref_refine_alignment(ra.tobytes(), rb.tobytes(), len(ra), 1, 1, int(maxw), mode, oa, ob, cap)
    assert n >= 0
    return np.frombuffer(oa.raw[:n], np.uint8).copy(), np.frombuffer(ob.raw[:n], np.uint8).copy()


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


def unalign(rng, ra, rb, frac):
    """A worse alignment of the same rows: a fraction of the columns where
    both genomes have a base split into two one-sided columns."""
    both = np.nonzero((ra != ord("-")) & (rb != ord("-")))[0]
    pick = np.zeros(len(ra), bool)
    pick[rng.choice(both, int(frac * len(both)), replace=False)] = True
    oa, ob = [], []
    for c in range(len(ra)):
        if pick[c]:
            oa += [ra[c], ord("-")]
            ob += [ord("-"), rb[c]]
        else:
            oa.append(ra[c])
            ob.append(rb[c])
    return np.array(oa, np.uint8), np.array(ob, np.uint8)


def main():
    mvg.load_library()
    rng = np.random.default_rng(1119)
    out = {}
    k = 0
    for nseg, maxw, frac in ((3, 20000.0, 0), (4, 20000.0, 0), (2, 1000.0, 0), (5, 3000.0, 0), (3, 600.0, 0),
                             (6, 20000.0, 0), (4, 400.0, 0), (7, 2500.0, 0), (3, 20000.0, 0.05), (4, 1500.0, 0.02),
                             (5, 600.0, 0.1)):
        ra, rb = lcb(rng, nseg)
        if frac:
            ra, rb = unalign(rng, ra, rb, frac)
        wins = mvg.refine_windows(ra, rb, maxw)
        assert [tuple(w) for w in wins.tolist()] == [(a, b, int(g)) for a, b, g in RO.refine_windows(ra, rb, maxw)]
        rows_a, rows_b = [], []
        for lo, hi, gap in wins.tolist():
            wa, wb = ra[lo:hi], rb[lo:hi]
            if not gap and (wa != ord("-")).any() and (wb != ord("-")).any():
                wa, wb = ref_realign(wa, wb)
            rows_a.append(wa)
            rows_b.append(wb)
        oa, ob = ref_refine(ra, rb, maxw)
        assert oa.tobytes() == np.concatenate(rows_a).tobytes() and ob.tobytes() == np.concatenate(rows_b).tobytes()
        out["a%d" % k], out["b%d" % k] = ra, rb
        out["w%d" % k] = np.float64(maxw)
        out["oa%d" % k], out["ob%d" % k] = oa, ob
        # the final iterative-refinement pass alone (mode 1) and after the
        # gapped-alignment pass (mode 2, a two-genome progressiveMauve run)
        out["ia%d" % k], out["ib%d" % k] = ref_refine(ra, rb, maxw, 1)
        out["fa%d" % k], out["fb%d" % k] = ref_refine(ra, rb, maxw, 2)
        out["win%d" % k] = wins
        k += 1
    out["count"] = np.int64(k)
    np.savez_compressed(os.path.join(HERE, "refine.npz"), **out)
    print("wrote %d LCBs, %d windows" % (k, sum(len(out["win%d" % i]) for i in range(k))))


if __name__ == "__main__":
    main()
