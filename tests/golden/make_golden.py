"""Generates the golden fixtures in tests/golden/ by running the reference's
own C++ code (oracle/_ref/libmauveref.so, built from the reference sources by
oracle/Makefile.ref) on seeded synthetic inputs.

Run from the repository root in a container that has the reference checkout:
    make -f oracle/Makefile.ref -j8 REF=<reference checkout>
    python tests/golden/make_golden.py
The fixtures are committed; the tests read them without the reference.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "tests"))
import synth  # noqa: E402

R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmauveref.so"))
R.ref_get_seed.restype = ctypes.c_uint64
R.ref_default_seed_weight.restype = ctypes.c_uint
for _f in ("ref_sml_build", "ref_pairwise_matches", "ref_seed_mers"):
    getattr(R, _f).restype = ctypes.c_int64
R.ref_profile_align.restype = ctypes.c_int
U64 = ctypes.c_uint64


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ref_sml(seq, seed):
    cap = len(seq)
    pos = np.zeros(cap, np.uint32)
    mer = np.zeros(cap, np.uint64)
    k = R.ref_sml_build(seq.tobytes(), U64(len(seq)), U64(seed), _p(pos), _p(mer), U64(cap))
    return pos[:k], mer[:k]


def ref_seed_mers(seq, seed):
    out = np.zeros(len(seq), np.uint64)
    k = R.ref_seed_mers(seq.tobytes(), U64(len(seq)), U64(seed), _p(out), U64(len(seq)))
    return out[:k]


def ref_matches(a, b, seed):
    cap = max(len(a), len(b))
    out = np.zeros(3 * cap, np.int64)
    k = R.ref_pairwise_matches(a.tobytes(), U64(len(a)), b.tobytes(), U64(len(b)), U64(seed), _p(out), U64(cap))
    assert k >= 0
    return out[: 3 * k].reshape(-1, 3)


def ref_path(a_codes, b_codes):
    sa = bytes(b"ACGT"[x] for x in a_codes)
    sb = bytes(b"ACGT"[x] for x in b_codes)
    cap = len(sa) + len(sb) + 1
    oa = ctypes.create_string_buffer(cap)
    ob = ctypes.create_string_buffer(cap)
    n = R.ref_profile_align(sa, len(sa), sb, len(sb), oa, ob, cap)
    ra, rb = oa.raw[:n], ob.raw[:n]
    return "".join("M" if x != 45 and y != 45 else ("D" if y == 45 else "I") for x, y in zip(ra, rb))


def main():
    rng = np.random.default_rng(20261203)
    # --- seeds table and default weights (LM/SeedMasks.h)
    seeds = np.array([[R.ref_get_seed(w, r) for r in range(6)] for w in range(3, 32)], np.uint64)
    lens = np.array([1, 2, 10, 100, 200, 1000, 5000, 30000, 1000000, 4600000, 12000000, 2 ** 40], np.uint64)
    weights = np.array([R.ref_default_seed_weight(U64(int(x))) for x in lens], np.uint32)
    np.savez_compressed(os.path.join(OUT, "seeds.npz"), table=seeds, lens=lens, weights=weights)

    # --- sorted mer lists: (sequence, seed) -> sorted (mer, pos) and the per-position fill
    sml = {}
    cases = [(15, 3), (17, 3), (11, 0), (7, 0), (13, 0), (21, 0), (31, 0), (5, 0)]
    for ci, (w, r) in enumerate(cases):
        seed = int(R.ref_get_seed(w, r))
        n = int(rng.integers(800, 3000))
        seq = synth.random_bases(rng, n, gc=float(rng.uniform(0.3, 0.7)))
        if ci == 0:  # IUPAC codes and lower case go through the translation table
            idx = rng.choice(n, 40, replace=False)
            seq[idx] = rng.choice(np.frombuffer(b"acgtNnRYKMSWbB", np.uint8), 40)
        pos, mer = ref_sml(seq, seed)
        sml["seq%d" % ci] = seq
        sml["seed%d" % ci] = np.uint64(seed)
        sml["pos%d" % ci] = pos
        sml["mer%d" % ci] = mer
        sml["fill%d" % ci] = ref_seed_mers(seq, seed)
    sml["count"] = np.int64(len(cases))
    np.savez_compressed(os.path.join(OUT, "sml.npz"), **sml)

    # --- pairwise match lists on mutated pairs
    mt = {}
    k = 0
    specs = []
    for _ in range(14):
        specs.append(dict(n=int(rng.integers(2000, 40000)), sub=float(rng.uniform(0, 0.08)),
                          nindel=int(rng.integers(0, 25)), ninv=int(rng.integers(0, 3)),
                          swap=bool(rng.random() < 0.3), repeat=bool(rng.random() < 0.4)))
    specs.append(dict(n=5000, sub=0.0, nindel=0, ninv=0, swap=False, repeat=False))   # identical pair
    specs.append(dict(n=3000, sub=0.75, nindel=0, ninv=0, swap=False, repeat=False))  # unrelated pair
    for sp in specs:
        b = synth.random_bases(rng, sp["n"], gc=0.5)
        if sp["repeat"]:
            b = synth.insert_repeats(rng, b, family_len=int(rng.integers(50, 400)), copies=int(rng.integers(2, 12)))
        a = synth.mutate(rng, b, sp["sub"], sp["nindel"], 4.0, sp["ninv"], (100, 1500))
        if sp["swap"]:
            a, b = b, a
        w = int(R.ref_default_seed_weight(U64((len(a) + len(b)) // 2)))
        seed = int(R.ref_get_seed(w, 3))
        m = ref_matches(a, b, seed)
        mt["a%d" % k], mt["b%d" % k], mt["seed%d" % k], mt["m%d" % k] = a, b, np.uint64(seed), m
        k += 1
    # one rank-0 (gap-search) seed case
    b = synth.random_bases(rng, 6000, gc=0.45)
    a = synth.mutate(rng, b, 0.05, 6, 3.0, 1, (200, 800))
    seed = int(R.ref_get_seed(9, 0))
    mt["a%d" % k], mt["b%d" % k], mt["seed%d" % k], mt["m%d" % k] = a, b, np.uint64(seed), ref_matches(a, b, seed)
    k += 1
    mt["count"] = np.int64(k)
    np.savez_compressed(os.path.join(OUT, "matches.npz"), **mt)

    # --- gap DP paths (MUSCLE NWSmall via ProfileProfile)
    dp_a, dp_b, dp_paths = [], [], []
    shapes = [(1, 1), (1, 2), (2, 1), (1, 7), (7, 1), (2, 2), (3, 9), (9, 3)]
    for la, lb in shapes:
        for _ in range(4):
            dp_a.append(rng.integers(0, 4, la).astype(np.uint8))
            dp_b.append(rng.integers(0, 4, lb).astype(np.uint8))
    for _ in range(300):
        la = int(rng.integers(1, 64))
        a = rng.integers(0, 4, la).astype(np.uint8)
        if rng.random() < 0.6:
            b = synth.mutate_codes(rng, a, float(rng.uniform(0, 0.3)), int(rng.integers(0, 4)), 3.0)
        else:
            b = rng.integers(0, 4, int(rng.integers(1, 64))).astype(np.uint8)
        dp_a.append(a)
        dp_b.append(b)
    for la in (300, 1000, 2500):
        a = rng.integers(0, 4, la).astype(np.uint8)
        dp_a.append(a)
        dp_b.append(synth.mutate_codes(rng, a, 0.1, 8, 3.0))
    for a, b in zip(dp_a, dp_b):
        dp_paths.append(ref_path(a, b))
    off_a = np.concatenate([[0], np.cumsum([len(x) for x in dp_a])]).astype(np.int64)
    off_b = np.concatenate([[0], np.cumsum([len(x) for x in dp_b])]).astype(np.int64)
    off_p = np.concatenate([[0], np.cumsum([len(x) for x in dp_paths])]).astype(np.int64)
    np.savez_compressed(os.path.join(OUT, "gapdp.npz"), seq_a=np.concatenate(dp_a), seq_b=np.concatenate(dp_b),
                        off_a=off_a, off_b=off_b, paths=np.frombuffer("".join(dp_paths).encode(), np.uint8),
                        off_p=off_p)
    print("wrote fixtures:", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
