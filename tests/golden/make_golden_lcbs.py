#!/usr/bin/env python3
"""Writes tests/golden/lcbs.npz: the reference's own LCB computation with
greedy breakpoint elimination for collinear genomes (the collinear branch of
alignProfileToProfile, libMems/ProgressiveAligner.cpp:2281-2303, compiled
into oracle/_ref/libmauveref.so by oracle/ref_lcbs_driver.cpp) on seeded
synthetic match lists.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_lcbs.py

A case is a two-genome match list: K blocks of genome A (200-5,000 bp)
placed into genome B in a random order (or in order), some inverted, each
carrying ungapped matches of 9-60 bp along it, plus a few random matches
between the genomes; the list is shuffled in half the cases.  A handful of
hand-made lists (empty, one match, two matches in either order and strand)
come first.  Stored per case: the input, the LCBs (matches concatenated,
offsets per LCB) and the deleted matches, all in the reference's order.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
U64P = ctypes.POINTER(ctypes.c_uint64)
R.ref_collinear_lcbs.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_uint64, U64P, ctypes.c_void_p, U64P]

HAND = [[], [(5, 7, 20)], [(5, -7, 20)], [(5, 7, 20), (100, 300, 20)], [(100, 300, 20), (5, 7, 20)],
        [(5, 300, 20), (100, 7, 20)], [(5, -300, 20), (100, -7, 20)], [(5, -7, 20), (100, 300, 20)]]


def reference(m):
    m = np.ascontiguousarray(m, np.int64).reshape(-1, 3)
    n = len(m)
    out, dl = np.zeros(3 * max(n, 1), np.int64), np.zeros(3 * max(n, 1), np.int64)
    off = np.zeros(n + 2, np.uint64)
    nl, nd = ctypes.c_uint64(0), ctypes.c_uint64(0)
    assert R.ref_collinear_lcbs(m.ctypes.data, n, out.ctypes.data, off.ctypes.data, len(off), ctypes.byref(nl),
                                dl.ctypes.data, ctypes.byref(nd)) == 0
    o = off[:nl.value + 1].astype(np.int64)
    return out[:3 * int(o[-1])].reshape(-1, 3), o, dl[:3 * nd.value].reshape(-1, 3)


def synthetic(rng):
    K = int(rng.integers(1, 25))
    lens = rng.integers(200, 5000, K)
    perm = rng.permutation(K) if rng.random() < 0.7 else np.arange(K)
    inv = rng.random(K) < rng.choice([0.0, 0.2, 0.5])
    pos_a = np.concatenate([[1], 1 + np.cumsum(lens)[:-1]])
    pos_b, p = np.zeros(K, np.int64), 1
    for k in np.argsort(perm):
        pos_b[k] = p
        p += lens[k] + int(rng.integers(0, 50))
    m = []
    for k in range(K):
        x = 0
        while x < lens[k] - 20:
            L = min(int(rng.integers(9, 60)), int(lens[k] - x))
            if rng.random() < 0.8:
                sb = -(pos_b[k] + lens[k] - x - L) if inv[k] else pos_b[k] + x
                m.append((pos_a[k] + x, sb, L))
            x += L + int(rng.integers(0, 40))
    for _ in range(int(rng.integers(0, 15))):
        L = int(rng.integers(9, 30))
        sa = int(rng.integers(1, pos_a[-1] + lens[-1] - L))
        sb = int(rng.integers(1, p)) * (1 if rng.random() < 0.5 else -1)
        m.append((sa, sb, L))
    m = np.array(m, np.int64).reshape(-1, 3)
    return m[rng.permutation(len(m))] if rng.random() < 0.5 else m


def main():
    rng = np.random.default_rng(20261204)
    cases = [np.array(h, np.int64).reshape(-1, 3) for h in HAND] + [synthetic(rng) for _ in range(40)]
    cols = {k: [] for k in ("m", "m_off", "lcb", "lcb_off", "lcb_case", "dl", "dl_off")}
    cols["m_off"], cols["lcb_case"], cols["dl_off"], cols["lcb_off"] = [0], [0], [0], []
    lcb_base = 0
    for m in cases:
        lcb, off, dl = reference(m)
        cols["m"].append(m)
        cols["m_off"].append(cols["m_off"][-1] + len(m))
        cols["lcb"].append(lcb)
        cols["lcb_off"].append(off + lcb_base)
        lcb_base += int(off[-1])
        cols["lcb_case"].append(cols["lcb_case"][-1] + len(off))
        cols["dl"].append(dl)
        cols["dl_off"].append(cols["dl_off"][-1] + len(dl))
    np.savez_compressed(os.path.join(HERE, "lcbs.npz"),
                        matches=np.concatenate(cols["m"]), match_off=np.array(cols["m_off"], np.int64),
                        lcb_matches=np.concatenate(cols["lcb"]), lcb_off=np.concatenate(cols["lcb_off"]),
                        lcb_case=np.array(cols["lcb_case"], np.int64), deleted=np.concatenate(cols["dl"]),
                        deleted_off=np.array(cols["dl_off"], np.int64))


if __name__ == "__main__":
    main()
