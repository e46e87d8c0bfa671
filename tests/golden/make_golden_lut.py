#!/usr/bin/env python3
"""Writes tests/golden/lut.npz from the reference's own code.

    sh oracle/build_ref_indexutils.sh <reference checkout>
    python tests/golden/make_golden_lut.py <reference checkout>

Runs, in this container only:
  * mauve/buildindex.py's buildIndex() itself, compiled from the reference
    source with its external steps replaced (running progressiveMauve and
    parsing its XMFA become "return these sub-alignment groups"; reading
    FASTA files becomes "return this sequence"), on synthetic alignments;
  * the reference's compiled mauve/indexutils.pyx (oracle/_ref) on
    synthetic LUTs: fixZeroIdx, fillGaps, smoothEdges, findGaps,
    findMismatches and findDuplicateMappings.
findEdges is not run: it calls ndarray.tostring, which NumPy 2 removed.
"""
import ast
import os
import sys
import types

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MAUVE_REFERENCE", "")
if not os.path.isdir(os.path.join(REF, "mauve")):
    sys.exit("give the reference checkout as the first argument or in MAUVE_REFERENCE")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle", "refshim_py"), os.path.join(ROOT, "oracle", "_ref"),
                os.path.join(ROOT, "tests")]

import indexutils as ref_iu  # noqa: E402  the reference's compiled module
import synth  # noqa: E402


def load_build_index(groups_box, seqs_box):
    """buildIndex from the reference source, with the external steps bound
    to in-memory data."""
    src = open(os.path.join(REF, "mauve", "buildindex.py")).read()
    tree = ast.parse(src)
    fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "buildIndex"][0]

    class TempDirs:
        def __init__(self, n):
            self.n = n

        def __enter__(self):
            return ["/nonexistent"] * self.n

        def __exit__(self, *exc):
            return False

    ns = {
        "os": os, "np": np, "IDX_ARRAY_DTYPE": np.int32, "indexutils": ref_iu, "TempDirs": TempDirs,
        "runMauve": lambda files, flags={}: None,
        "parseXMFA": lambda fp: groups_box[0],
        "getGenomeLength": lambda fp: len(seqs_box[0]),
        "getSeqFromFile": lambda fp: seqs_box[0] if fp.endswith("genome.fa") else seqs_box[1],
    }
    exec(compile(ast.Module(body=[fn], type_ignores=[]), "mauve/buildindex.py", "exec"), ns)
    return ns["buildIndex"]


def as_groups(groups):
    out = []
    for g in groups:
        out.append(types.SimpleNamespace(alignments=[
            types.SimpleNamespace(seq_num=s, start_idx=st, seq=row.decode("latin-1")) for s, st, row in g]))
    return out


def flatten(groups):
    """Blocks the way buildIndex consumes them (both sequences present)."""
    gs, rs, rg, rr = [], [], [], []
    for g in groups:
        d = {s: (st, row) for s, st, row in g}
        if 1 in d and 2 in d:
            gs.append(d[1][0])
            rs.append(d[2][0])
            rg.append(d[1][1])
            rr.append(d[2][1][:len(d[1][1])])
    off = np.zeros(len(gs) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in rg])
    return (np.array(gs, np.int64), np.array(rs, np.int64), off, np.frombuffer(b"".join(rg), np.uint8),
            np.frombuffer(b"".join(rr), np.uint8))


BUILD_CASES = [
    # seed, n_ref, sub, indel, nblocks, extras
    (0, 3000, 0.01, 0.002, 1, False),
    (1, 6000, 0.02, 0.005, 6, True),
    (2, 6000, 0.08, 0.02, 10, True),
    (3, 12000, 0.005, 0.001, 4, True),
    (4, 4000, 0.15, 0.03, 12, True),
    (5, 20000, 0.03, 0.004, 8, True),
]
VARIANTS = [  # fill_gaps, max_gap_width, smooth_edges, smoothing_radius
    (False, 300, False, 20), (True, 300, False, 20), (False, 300, True, 20), (True, 300, True, 20),
    (True, 25, True, 4),
]


def main():
    out = {}
    groups_box, seqs_box = [None], [None, None]
    build_index = load_build_index(groups_box, seqs_box)
    for k, (seed, n_ref, sub, indel, nb, extras) in enumerate(BUILD_CASES):
        groups, genome, ref = synth.lut_alignment(seed, n_ref=n_ref, sub=sub, indel=indel, nblocks=nb, extras=extras)
        groups_box[0] = as_groups(groups)
        seqs_box[0], seqs_box[1] = genome.decode("latin-1"), ref.decode("latin-1")
        gs, rs, off, rg, rr = flatten(groups)
        out["b%d_gs" % k], out["b%d_rs" % k], out["b%d_off" % k] = gs, rs, off
        out["b%d_rg" % k], out["b%d_rr" % k] = rg, rr
        out["b%d_genome" % k] = np.frombuffer(genome, np.uint8)
        out["b%d_ref" % k] = np.frombuffer(ref, np.uint8)
        for v, (fg, mg, se, sr) in enumerate(VARIANTS):
            lut = build_index("genome.fa", "ref.fa", fill_gaps=fg, max_gap_width=mg, smooth_edges=se,
                              smoothing_radius=sr)
            out["b%d_v%d" % (k, v)] = np.asarray(lut, np.int32)
    out["build_variants"] = np.array([[int(a), b, int(c), d] for a, b, c, d in VARIANTS], np.int32)
    out["n_build"] = np.int32(len(BUILD_CASES))

    # clean-up passes on synthetic LUTs
    nl = 0
    for seed in range(6):
        lut0 = synth.lut_random(100 + seed, n=4000 if seed < 5 else 20000)
        out["l%d_in" % nl] = lut0.copy()
        for name, w in (("fill300", 300), ("fill40", 40), ("fill3", 3), ("fill0", 0), ("fillneg", -5)):
            x = lut0.copy()
            ref_iu.fillGaps(x, max_gap_width=w)
            out["l%d_%s" % (nl, name)] = x
        for name, r in (("smooth20", 20), ("smooth5", 5), ("smoothneg", -1)):
            x = lut0.copy()
            ref_iu.smoothEdges(x, smoothing_radius=r)
            out["l%d_%s" % (nl, name)] = x
        x = lut0.copy()
        gaps = ref_iu.findGaps(x)
        out["l%d_findgaps_lut" % nl], out["l%d_findgaps" % nl] = x, np.asarray(gaps, np.int32)
        rng = np.random.default_rng(seed)
        genome = rng.choice(np.frombuffer(b"ACGT", np.uint8), len(lut0)).tobytes()
        ref = rng.choice(np.frombuffer(b"ACGT", np.uint8), int(lut0.max()) + 5).tobytes()
        mm = ref_iu.findMismatches(lut0.copy(), genome, ref)
        out["l%d_genome" % nl] = np.frombuffer(genome, np.uint8)
        out["l%d_ref" % nl] = np.frombuffer(ref, np.uint8)
        out["l%d_mism" % nl] = np.array([bool(b) for b in mm], np.uint8)
        out["l%d_dups" % nl] = np.int64(ref_iu.findDuplicateMappings(lut0.copy()))
        nl += 1
    out["n_lut"] = np.int32(nl)

    # fixZeroIdx: (lut, genome, ref) -> lut or IndexError (-999 marker)
    fz = []
    rng = np.random.default_rng(7)
    base = np.frombuffer(b"ACGT", np.uint8)
    for case in range(24):
        n = [5, 10, 11, 12, 40, 200][case % 6]
        lut = np.full(n, -1, np.int32)
        k = int(rng.integers(0, n))
        if case % 4 != 3:
            lut[k:] = np.arange(n - k) + int(rng.integers(-3, 30))
        if case % 5 == 0:
            lut[0] = 7
        genome = rng.choice(base, n).tobytes()
        ref = rng.choice(base, int(rng.integers(1, 60))).tobytes()
        if case % 3 == 0:
            genome = ref[:1] + genome[1:]
        x = lut.copy()
        try:
            ref_iu.fixZeroIdx(x, genome.decode(), ref.decode())
            status = 0
        except IndexError:
            status = -999
        fz.append((lut, genome, ref, x, status))
    out["n_fz"] = np.int32(len(fz))
    for i, (lut, g, r, x, st) in enumerate(fz):
        out["fz%d_in" % i], out["fz%d_out" % i] = lut, x
        out["fz%d_genome" % i] = np.frombuffer(g, np.uint8)
        out["fz%d_ref" % i] = np.frombuffer(r, np.uint8)
        out["fz%d_status" % i] = np.int32(st)
    # XMFA: the reference's own parser (mauve/xmfa.py) on its example file
    # and on synthetic files, and its buildIndex loop on the parse
    sys.path.insert(0, os.path.join(REF, "mauve"))
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import xmfa as ref_xmfa
    import json
    import tempfile
    texts = [open(os.path.join(REF, "tests", "example.xmfa"), "rb").read()]
    for k, (seed, crlf, width) in enumerate(((21, False, 80), (22, True, 60), (23, False, 7))):
        groups, genome, ref = synth.lut_alignment(seed, n_ref=3000, sub=0.03, indel=0.01, nblocks=5, extras=True)
        texts.append(synth.xmfa_text(groups, width=width, crlf=crlf, seed=seed))
        out["x%d_genome" % (k + 1)] = np.frombuffer(genome, np.uint8)
        out["x%d_ref" % (k + 1)] = np.frombuffer(ref, np.uint8)
    for k, txt in enumerate(texts):
        with tempfile.NamedTemporaryFile("wb", suffix=".xmfa", delete=False) as f:
            f.write(txt)
        parsed = ref_xmfa.parseXMFA(f.name)
        os.unlink(f.name)
        out["x%d_text" % k] = np.frombuffer(txt, np.uint8)
        out["x%d_parse" % k] = np.frombuffer(json.dumps(
            [[g.notes, [list(a) for a in g.alignments]] for g in parsed]).encode(), np.uint8)
        genome_len = len(out["x%d_genome" % k]) if k > 0 else 700
        groups_box[0] = parsed
        if k > 0:
            seqs_box[0] = bytes(out["x%d_genome" % k]).decode("latin-1")
            seqs_box[1] = bytes(out["x%d_ref" % k]).decode("latin-1")
            lut = build_index("genome.fa", "ref.fa")
        else:
            seqs_box[0] = "A" * genome_len
            lut = build_index("genome.fa", "ref.fa", fill_gaps=False, smooth_edges=True)
        out["x%d_lut" % k] = np.asarray(lut, np.int32)
    out["n_xmfa"] = np.int32(len(texts))
    path = os.path.join(HERE, "lut.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
