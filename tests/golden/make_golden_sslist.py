#!/usr/bin/env python3
"""Writes tests/golden/sslist.npz: what the reference's own code puts in a
.sslist file (FileSML::Create, libMems/FileSML.cpp:401-459) for a few
sequences: the SMLHeader layout (sizeof and member offsets of the compiled
struct, libMems/SortedMerList.h:48-63), the header members an SML holds
after Create (members the reference never sets are zero), the packed
sequence words, and the sorted positions with their mers.

    make -f oracle/Makefile.ref REF=<reference checkout>
    python tests/golden/make_golden_sslist.py
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
R.ref_sml_file_image.restype = ctypes.c_int64
R.ref_sml_build.restype = ctypes.c_int64
R.ref_get_seed.restype = ctypes.c_uint64
VP = ctypes.c_void_p


def main():
    out = {}
    layout = np.zeros(15, np.int64)
    R.ref_sml_header_layout(layout.ctypes.data_as(VP))
    out["layout"] = layout
    rng = np.random.default_rng(5)
    cases = [(b"ACGTTGCAACGGTTACGTAGCTAGCTAGGATCGATCGATTTACG", 15, 3),
             (bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), 3000)), 15, 3),
             (bytes(rng.choice(np.frombuffer(b"ACGTNacgtn", np.uint8), 5000)), 11, 0),
             (bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), 777)), 17, 0)]
    for k, (seq, w, rank) in enumerate(cases):
        seed = R.ref_get_seed(w, rank)
        hdr = np.zeros(int(layout[0]), np.uint8)
        words = np.zeros(len(seq) // 16 + 8, np.uint32)
        nw = R.ref_sml_file_image(seq, len(seq), ctypes.c_uint64(seed), hdr.ctypes.data_as(VP),
                                  words.ctypes.data_as(VP), ctypes.c_uint64(len(words)))
        assert nw > 0
        cap = len(seq)
        pos = np.zeros(cap, np.uint32)
        mer = np.zeros(cap, np.uint64)
        n = R.ref_sml_build(seq, len(seq), ctypes.c_uint64(seed), pos.ctypes.data_as(VP), mer.ctypes.data_as(VP),
                            ctypes.c_uint64(cap))
        assert n >= 0
        out["s%d_seq" % k] = np.frombuffer(seq, np.uint8)
        out["s%d_seed" % k] = np.uint64(seed)
        out["s%d_header" % k] = hdr
        out["s%d_words" % k] = words[:nw]
        out["s%d_pos" % k] = pos[:n]
        out["s%d_mer" % k] = mer[:n]
    out["n"] = np.int32(len(cases))
    path = os.path.join(HERE, "sslist.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
