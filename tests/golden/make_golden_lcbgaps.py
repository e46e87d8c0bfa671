#!/usr/bin/env python3
"""Writes tests/golden/lcbgaps.npz: the reference's own search outside LCBs
(SearchLCBGaps, libMems/Aligner.cpp:784-928, with transposeMatches and
EliminateOverlaps; compiled into oracle/_ref/libmauveref.so by
oracle/ref_lcbgap_driver.cpp) on seeded synthetic inputs.

    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden_lcbgaps.py

Two kinds of case:
  post   -- random two-genome match lists in the coordinates of two region
            concatenations (lengths 1-60, forward and reverse B starts,
            repeated A starts, exact duplicates, zero-length and touching
            regions) and the reference's transposeMatches for A and for B,
            EliminateOverlaps, and the full finishing sequence
            (transpose A, transpose B, EliminateOverlaps, MultiplicityFilter,
            LengthFilter(9)).
  search -- genome pairs (a random genome and a mutated, partly rearranged
            copy; one pair with lowercase, N and IUPAC codes) with regions
            outside imaginary LCBs, the reference's SearchLCBGaps output, its
            seed weight and the raw match list of the two concatenations
            before transposition.
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
P, U = ctypes.c_void_p, ctypes.c_uint64
R.ref_search_lcb_gaps.argtypes = [ctypes.c_char_p, U, ctypes.c_char_p, U, P, U, P, U, P, U]
R.ref_search_lcb_gaps.restype = ctypes.c_int64
R.ref_gap_concat_matches.argtypes = [ctypes.c_char_p, U, ctypes.c_char_p, U, P, U, P]
R.ref_gap_concat_matches.restype = ctypes.c_int64
R.ref_transpose_matches.argtypes = [P, U, ctypes.c_uint, P, U, P, U]
R.ref_transpose_matches.restype = ctypes.c_int64
R.ref_eliminate_overlaps.argtypes = [P, U, P, U]
R.ref_eliminate_overlaps.restype = ctypes.c_int64
R.ref_lcb_gap_finish.argtypes = [P, U, P, U, P, U, P, U]
R.ref_lcb_gap_finish.restype = ctypes.c_int64


def call(fn, *args, cap):
    out = np.zeros(3 * cap + 3, np.int64)
    n = fn(*args, out.ctypes.data, cap)
    assert n >= 0, n
    return out[:3 * n].reshape(-1, 3)


def regions(rng, nreg, maxlen, gap=500, start=1):
    lens = rng.integers(0, maxlen, nreg)
    pos, r = start, []
    for L in lens:
        pos += int(rng.integers(0, gap))
        r += [pos, pos + int(L)]
        pos += int(L)
    return np.array(r, np.int64)


def post_case(rng):
    nreg = int(rng.integers(1, 12))
    ra, rb = regions(rng, nreg, 400), regions(rng, nreg, 400)
    ta, tb = int(np.diff(ra.reshape(-1, 2)).sum()), int(np.diff(rb.reshape(-1, 2)).sum())
    m = []
    for _ in range(int(rng.integers(0, 90))):
        L = int(rng.integers(1, 60))
        if ta < L + 1 or tb < L + 1:
            break
        sa, sb = int(rng.integers(1, ta - L + 2)), int(rng.integers(1, tb - L + 2))
        if rng.random() < 0.4:
            sb = -sb
        m.append((sa, sb, L))
        if rng.random() < 0.15:  # another match from the same A position
            m.append((sa, int(rng.integers(1, tb - L + 2)), int(rng.integers(1, L + 1))))
        if rng.random() < 0.05:
            m.append(m[-1])
    m = np.array(m, np.int64).reshape(-1, 3)
    cap = 4 * len(m) + 64
    t0 = call(R.ref_transpose_matches, m.ctypes.data, len(m), 0, ra.ctypes.data, len(ra), cap=cap)
    t1 = call(R.ref_transpose_matches, m.ctypes.data, len(m), 1, rb.ctypes.data, len(rb), cap=cap)
    eo = call(R.ref_eliminate_overlaps, m.ctypes.data, len(m), cap=cap)
    fin = call(R.ref_lcb_gap_finish, m.ctypes.data, len(m), ra.ctypes.data, len(ra), rb.ctypes.data, len(rb),
               cap=cap)
    return dict(m=m, ra=ra, rb=rb, t0=t0, t1=t1, eo=eo, fin=fin)


def cut(rng, r, pieces):
    """Each region cut into touching pieces at random points."""
    out = []
    for l, h in np.asarray(r).reshape(-1, 2):
        pts = np.sort(rng.integers(l, h + 1, pieces - 1)) if h > l else np.zeros(0, np.int64)
        edges = [int(l)] + [int(x) for x in pts] + [int(h)]
        for x, y in zip(edges[:-1], edges[1:]):
            out += [x, y]
    return np.array(out, np.int64)


def search_case(rng, n, nreg, maxlen, div, iupac=False, empty_b=False, shift=200, pieces=1, nrearr=4, nindel=None):
    a = synth.random_bases(rng, n)
    b = synth.mutate(rng, a, div, n // 2000 if nindel is None else nindel, 4.0, nrearr, (300, 3000))
    if iupac:
        for s in (a, b):
            k = rng.random(len(s))
            s[k < 0.01] = ord("N")
            s[(k >= 0.01) & (k < 0.015)] = rng.choice(np.frombuffer(b"RYKMSWBDHV", np.uint8),
                                                       int(((k >= 0.01) & (k < 0.015)).sum()))
            low = rng.random(len(s)) < 0.1
            s[low] = s[low] | 0x20
    ra = regions(rng, nreg, maxlen, gap=max(1, n // (nreg + 1) - maxlen // 2))
    ra = ra[ra <= len(a) + 1].copy()
    ra = ra[: len(ra) // 2 * 2]
    # B's regions near A's (a mutated copy keeps most coordinates), some
    # shifted, some touching their neighbour, one of zero length
    rb = []
    for l, r in ra.reshape(-1, 2):
        d = int(rng.integers(-shift, shift + 1))
        l2 = max(1, min(len(b) + 1, l + d))
        r2 = max(l2, min(len(b) + 1, r + d + int(rng.integers(-shift // 4, shift // 4 + 1))))
        if rb and l2 < rb[-1]:
            l2 = rb[-1]
            r2 = max(r2, l2)
        rb += [l2, r2]
    rb = np.array([] if empty_b else rb, np.int64)
    if pieces > 1:
        ra, rb = cut(rng, ra, pieces), cut(rng, rb, pieces)
    for r in (ra, rb):
        if len(r) >= 4 and rng.random() < 0.7:
            r[3] = max(r[3], r[2])
            r[2] = r[1]  # touching regions
    raw_a = np.concatenate([a[l - 1:r - 1] for l, r in ra.reshape(-1, 2)] or [np.zeros(0, np.uint8)])
    raw_b = np.concatenate([b[l - 1:r - 1] for l, r in rb.reshape(-1, 2)] or [np.zeros(0, np.uint8)])
    w = ctypes.c_uint32(0)
    cap = len(raw_a) + len(raw_b) + 16
    out = np.zeros(3 * cap, np.int64)
    k = R.ref_gap_concat_matches(raw_a.tobytes(), len(raw_a), raw_b.tobytes(), len(raw_b), out.ctypes.data, cap,
                                 ctypes.byref(w))
    raw = out[:3 * max(k, 0)].reshape(-1, 3).copy()
    fin = call(R.ref_search_lcb_gaps, a.tobytes(), len(a), b.tobytes(), len(b), ra.ctypes.data, len(ra),
               rb.ctypes.data, len(rb), cap=cap)
    return dict(a=a, b=b, ra=ra, rb=rb, raw=raw, fin=fin, w=np.int64(w.value))


def main():
    rng = np.random.default_rng(2024)
    out = {}
    posts = [post_case(rng) for _ in range(80)]
    for key in ("m", "ra", "rb", "t0", "t1", "eo", "fin"):
        arrs = [p[key].reshape(-1) for p in posts]
        out["post_" + key] = np.concatenate(arrs).astype(np.int32)
        out["post_" + key + "_off"] = np.concatenate([[0], np.cumsum([len(x) for x in arrs])]).astype(np.int64)
    searches = [
        search_case(rng, 60_000, 12, 3000, 0.03, shift=20, nrearr=0, nindel=0),
        search_case(rng, 80_000, 30, 1500, 0.10),
        search_case(rng, 60_000, 6, 6000, 0.02, shift=8, pieces=7, nrearr=0, nindel=0),
        search_case(rng, 50_000, 8, 6000, 0.01, iupac=True),
        search_case(rng, 40_000, 6, 2000, 0.05, empty_b=True),
        search_case(rng, 3_000, 3, 12, 0.02),  # too short to search
    ]
    out["search_count"] = np.int64(len(searches))
    for k, c in enumerate(searches):
        for key, v in c.items():
            out["s%d_%s" % (k, key)] = v
    np.savez_compressed(os.path.join(HERE, "lcbgaps.npz"), **out)
    print("post cases: %d lists, %d matches in, %d after finishing" %
          (len(posts), sum(len(p["m"]) for p in posts), sum(len(p["fin"]) for p in posts)))
    for k, c in enumerate(searches):
        print("search %d: |A| %d |B| %d, regions %d/%d, weight %d, raw %d, final %d" %
              (k, len(c["a"]), len(c["b"]), len(c["ra"]) // 2, len(c["rb"]) // 2, int(c["w"]), len(c["raw"]),
               len(c["fin"])))


if __name__ == "__main__":
    main()
