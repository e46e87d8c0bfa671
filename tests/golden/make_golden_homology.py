#!/usr/bin/env python3
"""Writes tests/golden/homology.npz: the reference's own backbone-detection
HMM (findHssHomologyHMM, libMems/Islands.h:122-196, with HomologyHMM's
forward/backward passes; compiled into oracle/_ref/libmauveref.so by
oracle/ref_homology_driver.cpp) on synthetic two-genome alignments, and the
parameters applyBackbone sets up for several GC contents and identities.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_homology.py

Alignments: concatenations of homologous stretches (a random sequence and a
copy with 1-30% substitutions and short gaps), unrelated aligned stretches
(two random sequences, some gaps) and one-genome runs, 50-3,000 columns
each; some with lowercase bases and N; one of 150,000 columns.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
P, U = ctypes.c_void_p, ctypes.c_uint64
R.ref_hmm_params.argtypes = [ctypes.c_double] * 4 + [P]
R.ref_homologous_segments.argtypes = [ctypes.c_char_p, ctypes.c_char_p, U, P, ctypes.c_int, ctypes.c_int, P, U]
R.ref_homologous_segments.restype = ctypes.c_int64
ACGT = np.frombuffer(b"ACGT", np.uint8)
GAP = ord("-")


def stretch(rng):
    kind = rng.random()
    n = int(rng.integers(50, 3000))
    if kind < 0.5:  # homologous
        a = ACGT[rng.integers(0, 4, n)]
        b = a.copy()
        sub = rng.random(n) < rng.uniform(0.01, 0.3)
        b[sub] = ACGT[rng.integers(0, 4, int(sub.sum()))]
        for c in np.nonzero(rng.random(n) < 0.01)[0]:
            (a if rng.random() < 0.5 else b)[c:c + int(rng.geometric(0.3))] = GAP
    elif kind < 0.8:  # unrelated
        a, b = ACGT[rng.integers(0, 4, n)], ACGT[rng.integers(0, 4, n)]
        for c in np.nonzero(rng.random(n) < 0.05)[0]:
            (a if rng.random() < 0.5 else b)[c:c + int(rng.geometric(0.2))] = GAP
    else:  # one genome only
        a, b = ACGT[rng.integers(0, 4, n)], np.full(n, GAP, np.uint8)
        if rng.random() < 0.5:
            a, b = b, a
    return a, b


def lcb(rng, nseg):
    parts = [stretch(rng) for _ in range(nseg)]
    ra = np.concatenate([p[0] for p in parts])
    rb = np.concatenate([p[1] for p in parts])
    if rng.random() < 0.7:  # drop the columns gapped in both
        keep = ~((ra == GAP) & (rb == GAP))
        ra, rb = ra[keep], rb[keep]
    return ra, rb


def segments(ra, rb, params, lh, rh):
    out = np.zeros(2 * 100000, np.int64)
    n = R.ref_homologous_segments(ra.tobytes(), rb.tobytes(), len(ra), params.ctypes.data, lh, rh, out.ctypes.data,
                                  100000)
    assert n >= 0
    return out[:2 * n].reshape(-1, 2).copy()


def main():
    rng = np.random.default_rng(1081)
    out = {}
    grid = [(gc, ident) for gc in (0.3, 0.38, 0.5, 0.508, 0.65) for ident in (0.5, 0.7, 0.9)]
    pv = np.zeros((len(grid), 21))
    for k, (gc, ident) in enumerate(grid):
        R.ref_hmm_params(gc, 1e-5, 1e-9, ident, pv[k].ctypes.data)
    out["param_grid"] = np.array(grid)
    out["params"] = pv
    k = 0
    for it in range(30):
        ra, rb = lcb(rng, int(rng.integers(1, 8)) if it < 29 else 120)
        if it % 5 == 4:
            m = rng.random(len(ra)) < 0.1
            ra = np.where(m & (ra != GAP), ra | 0x20, ra).astype(np.uint8)
            m = rng.random(len(rb)) < 0.01
            rb = np.where(m & (rb != GAP), ord("N"), rb).astype(np.uint8)
        pi = int(rng.integers(0, len(grid)))
        out["a%d" % k], out["b%d" % k], out["p%d" % k] = ra, rb, np.int64(pi)
        for lh, rh in ((1, 1), (0, 1), (1, 0)):
            out["s%d_%d%d" % (k, lh, rh)] = segments(ra, rb, pv[pi], lh, rh)
        k += 1
    out["count"] = np.int64(k)
    np.savez_compressed(os.path.join(HERE, "homology.npz"), **out)
    print("wrote %d alignments (%d columns), %d segments" %
          (k, sum(len(out["a%d" % i]) for i in range(k)), sum(len(out["s%d_11" % i]) for i in range(k))))


if __name__ == "__main__":
    main()
