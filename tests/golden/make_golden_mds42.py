#!/usr/bin/env python3
"""Writes tests/golden/mds42.npz: the reference's pairwise match list for
its own recoded E. coli fixture pair (tests/mds42_recoded.fa vs
tests/mds42_full.fa in the reference tree), with both genomes packed.

    make -f oracle/Makefile.ref REF=<reference checkout>
    python tests/golden/make_golden_mds42.py <reference checkout>

The match list comes from the reference's own PairwiseMatchFinder (compiled
into oracle/_ref/libmauveref.so) with progressiveMauve's default seed: the
coding seed of the default weight for the pair's average length.  Genomes
are stored 2-bit (A,C,G,T = 0..3, four bases per byte, first base in the
high bits); both are pure ACGT.
"""
import ctypes
import os
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MAUVE_REFERENCE", "")
if not os.path.isdir(os.path.join(REF, "mauve")):
    sys.exit("give the reference checkout as the first argument or in MAUVE_REFERENCE")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
R.ref_get_seed.restype = ctypes.c_uint64
R.ref_default_seed_weight.restype = ctypes.c_uint
R.ref_pairwise_matches.restype = ctypes.c_int64
U64 = ctypes.c_uint64


def read_fasta(path):
    with open(path) as f:
        lines = f.read().split("\n")
    return "".join(l.strip() for l in lines[1:] if not l.startswith(">")).encode()


def pack2(seq):
    codes = np.frombuffer(seq, np.uint8)
    lut = np.full(256, 255, np.uint8)
    for i, c in enumerate(b"ACGT"):
        lut[c] = i
    v = lut[codes]
    assert (v < 4).all()
    pad = (-len(v)) % 4
    v = np.concatenate([v, np.zeros(pad, np.uint8)]).reshape(-1, 4)
    return (v[:, 0] << 6) | (v[:, 1] << 4) | (v[:, 2] << 2) | v[:, 3]


def main():
    a = read_fasta(os.path.join(REF, "tests", "mds42_recoded.fa"))
    b = read_fasta(os.path.join(REF, "tests", "mds42_full.fa"))
    w = int(R.ref_default_seed_weight(U64((len(a) + len(b)) // 2)))
    seed = int(R.ref_get_seed(w, 3))
    cap = 3 * 2_000_000
    out = np.zeros(cap, np.int64)
    n = R.ref_pairwise_matches(a, U64(len(a)), b, U64(len(b)), U64(seed), out.ctypes.data_as(ctypes.c_void_p),
                               U64(cap // 3))
    assert n >= 0
    m = out[:3 * n].reshape(-1, 3).copy()
    path = os.path.join(HERE, "mds42.npz")
    np.savez_compressed(path, a=pack2(a), na=np.int64(len(a)), b=pack2(b), nb=np.int64(len(b)),
                        seed=np.uint64(seed), weight=np.int32(w), matches=m)
    print("wrote", path, os.path.getsize(path), "bytes;", n, "matches, seed %#x (w=%d)" % (seed, w))


if __name__ == "__main__":
    main()
