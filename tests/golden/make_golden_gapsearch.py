#!/usr/bin/env python3
"""Writes tests/golden/gapsearch.npz: the reference's own gap anchor search
(ProgressiveAligner::pairwiseAnchorSearch, libMems/ProgressiveAligner.cpp:590-679)
on seeded synthetic inter-anchor gaps of 200 bp to 50 kbp.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_gapsearch.py

For each gap pair (a, b) it stores
  * the seed weight getDefaultSeedWeight((|a| + |b|) / 2) the search uses,
  * the MemHash match list before the filters (rank-0 seed of that weight,
    oracle/ref_driver.cpp ref_memhash_matches), and
  * the anchors after EliminateOverlaps_v2 and LengthFilter(12)
    (oracle/ref_gap_driver.cpp ref_gap_anchor_search),
as (start in a, start in b, length) rows, 1-based, negative = reverse strand,
in the reference's list order.
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
R.ref_get_seed.restype = ctypes.c_uint64
R.ref_memhash_matches.restype = ctypes.c_int64
R.ref_gap_anchor_search.restype = ctypes.c_int64
U64 = ctypes.c_uint64


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ref_gap(a, b):
    cap = max(len(a), len(b)) + 16
    out = np.zeros(3 * cap, np.int64)
    w = ctypes.c_uint32(0)
    k = R.ref_gap_anchor_search(a.tobytes(), U64(len(a)), b.tobytes(), U64(len(b)), _p(out), U64(cap), ctypes.byref(w))
    if k == -2:
        return int(w.value), np.zeros((0, 3), np.int64), np.zeros((0, 3), np.int64)
    assert k >= 0
    anchors = out[:3 * k].reshape(-1, 3).copy()
    seed = int(R.ref_get_seed(int(w.value), 0))
    k2 = R.ref_memhash_matches(a.tobytes(), U64(len(a)), b.tobytes(), U64(len(b)), U64(seed), _p(out), U64(cap))
    assert k2 >= 0
    return int(w.value), out[:3 * k2].reshape(-1, 3).copy(), anchors


def main():
    rng = np.random.default_rng(20261204)
    pairs = []
    # log-uniform gap lengths over the recursion's range, mixed divergence
    for _ in range(40):
        n = int(np.exp(rng.uniform(np.log(200), np.log(50_000))))
        b = synth.random_bases(rng, n, gc=float(rng.uniform(0.35, 0.65)))
        if rng.random() < 0.4:
            b = synth.insert_repeats(rng, b, int(rng.integers(20, max(21, min(600, n // 4)))), int(rng.integers(2, 8)))
        ninv = int(rng.integers(0, 3)) if n > 3000 else 0
        a = synth.mutate(rng, b, float(rng.uniform(0.0, 0.25)), int(rng.integers(0, 1 + n // 400)), 3.0, ninv,
                         (100, max(101, n // 10)))
        if rng.random() < 0.3:
            a, b = b, a
        pairs.append((a, b))
    # edge cases: tiny gaps (weight below the minimum), identical, unrelated, tandem repeat
    pairs.append((synth.random_bases(rng, 9), synth.random_bases(rng, 14)))
    x = synth.random_bases(rng, 4000)
    pairs.append((x, x.copy()))
    pairs.append((synth.random_bases(rng, 3000), synth.random_bases(rng, 3500)))
    unit = synth.random_bases(rng, 37)
    t = np.tile(unit, 60)
    pairs.append((synth.mutate(rng, t, 0.03, 3, 2.0, 0, (10, 20)), t))
    g = {}
    for k, (a, b) in enumerate(pairs):
        w, mh, anchors = ref_gap(a, b)
        g["a%d" % k], g["b%d" % k] = a, b
        g["w%d" % k] = np.int64(w)
        g["mh%d" % k] = mh
        g["anc%d" % k] = anchors
    g["count"] = np.int64(len(pairs))
    np.savez_compressed(os.path.join(HERE, "gapsearch.npz"), **g)
    print("gapsearch.npz: %d gap pairs, %d anchors" % (len(pairs), sum(len(g["anc%d" % k]) for k in range(len(pairs)))))


if __name__ == "__main__":
    main()
