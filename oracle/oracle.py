"""ctypes binding of the CPU oracle (oracle/mauve_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker that tests/, __graft_entry__.smoke()
and bench.py's CPU baseline compare the CUDA path against.  The product
package never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmauve_oracle.so")
_lib = None


def build(force=False):
    """Compile oracle/mauve_oracle.c into oracle/lib/libmauve_oracle.so."""
    srcs = [os.path.join(_HERE, f) for f in ("mauve_oracle.c", "lut_oracle.c", "gap_oracle.cpp", "mauve_oracle.h")]
    if not force and os.path.exists(LIB_PATH) and all(
            os.path.getmtime(LIB_PATH) >= os.path.getmtime(s) for s in srcs):
        return LIB_PATH
    objdir = os.path.join(os.path.dirname(LIB_PATH), "obj")
    os.makedirs(objdir, exist_ok=True)
    objs = []
    for src in srcs[:3]:
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cc = ["g++", "-std=c++17"] if src.endswith(".cpp") else ["gcc"]
        subprocess.check_call([*cc, "-O2", "-fPIC", "-c", src, "-o", obj])
        objs.append(obj)
    subprocess.check_call(["g++", "-shared", "-o", LIB_PATH, *objs, "-lm", "-lpthread"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u64, i64, vp = ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p
        L.mo_get_seed.restype = u64
        L.mo_get_seed.argtypes = [ctypes.c_int, ctypes.c_int]
        L.mo_seed_length.argtypes = [u64]
        L.mo_seed_weight.argtypes = [u64]
        L.mo_default_seed_weight.argtypes = [u64]
        L.mo_default_seed_weight.restype = ctypes.c_uint
        L.mo_pack.restype = i64
        L.mo_pack.argtypes = [vp, u64, vp]
        L.mo_seed_mers.restype = i64
        L.mo_seed_mers.argtypes = [vp, u64, u64, vp]
        L.mo_sml_build.restype = i64
        L.mo_sml_build.argtypes = [vp, u64, u64, vp, vp]
        L.mo_pairwise_matches.restype = i64
        L.mo_pairwise_matches.argtypes = [vp, u64, vp, u64, u64, vp, u64]
        L.mo_unique_pairs.restype = i64
        L.mo_unique_pairs.argtypes = [vp, u64, vp, u64, u64, vp, vp, u64]
        L.mo_gap_anchor_filter.restype = i64
        L.mo_gap_anchor_filter.argtypes = [vp, i64]
        L.mo_gap_anchor_search.restype = i64
        L.mo_gap_anchor_search.argtypes = [vp, u64, vp, u64, vp, u64, vp]
        L.mo_nw_align.restype = i64
        L.mo_nw_align.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp, vp]
        L.mo_nw_score.restype = ctypes.c_int32
        L.mo_nw_score.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int]
        L.mo_nw_batch.restype = i64
        L.mo_nw_batch.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp, vp, ctypes.c_int]
        L.mo_lut_from_blocks.restype = i64
        L.mo_lut_from_blocks.argtypes = [vp, vp, vp, vp, vp, u64, vp, u64]
        L.mo_fix_zero_idx.argtypes = [vp, u64, vp, u64, vp, u64]
        L.mo_fill_gaps.argtypes = [vp, u64, ctypes.c_int]
        L.mo_fill_gaps.restype = None
        L.mo_smooth_edges.argtypes = [vp, u64, ctypes.c_int]
        L.mo_smooth_edges.restype = None
        L.mo_find_gaps.argtypes = [vp, u64, vp]
        L.mo_find_gaps.restype = None
        L.mo_find_edges.argtypes = [vp, u64, vp]
        L.mo_find_edges.restype = None
        L.mo_find_mismatches.argtypes = [vp, u64, vp, u64, vp, u64, vp]
        L.mo_find_duplicate_mappings.restype = i64
        L.mo_find_duplicate_mappings.argtypes = [vp, u64, vp, u64]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _u8(seq):
    if isinstance(seq, (bytes, bytearray)):
        return np.frombuffer(bytes(seq), np.uint8)
    return np.ascontiguousarray(seq, dtype=np.uint8)


def get_seed(weight, rank):
    return int(lib().mo_get_seed(weight, rank))


def seed_length(seed):
    return int(lib().mo_seed_length(seed))


def seed_weight(seed):
    return int(lib().mo_seed_weight(seed))


def default_seed_weight(avg_len):
    return int(lib().mo_default_seed_weight(avg_len))


def pack(seq):
    s = _u8(seq)
    out = np.zeros(len(s) // 16 + 3, np.uint32)
    n = lib().mo_pack(_p(s), len(s), _p(out))
    if n < 0:
        raise ValueError("gap character in genome sequence")
    return out[:n]


def seed_mers(seq, seed):
    s = _u8(seq)
    out = np.zeros(max(len(s), 1), np.uint64)
    n = lib().mo_seed_mers(_p(s), len(s), seed, _p(out))
    return out[:n]


def sml_build(seq, seed):
    s = _u8(seq)
    pos = np.zeros(max(len(s), 1), np.uint32)
    mer = np.zeros(max(len(s), 1), np.uint64)
    n = lib().mo_sml_build(_p(s), len(s), seed, _p(pos), _p(mer))
    return pos[:n], mer[:n]


def unique_pairs(a, b, seed):
    a, b = _u8(a), _u8(b)
    cap = max(min(len(a), len(b)), 1)
    pa = np.zeros(cap, np.uint32)
    pb = np.zeros(cap, np.uint32)
    n = lib().mo_unique_pairs(_p(a), len(a), _p(b), len(b), seed, _p(pa), _p(pb), cap)
    if n < 0:
        raise RuntimeError("mo_unique_pairs failed: %d" % n)
    return pa[:n], pb[:n]


def pairwise_matches(a, b, seed):
    """(start0, start1, length) rows in the reference's MatchList order."""
    a, b = _u8(a), _u8(b)
    cap = max(min(len(a), len(b)), 16)
    out = np.zeros(3 * cap, np.int64)
    n = lib().mo_pairwise_matches(_p(a), len(a), _p(b), len(b), seed, _p(out), cap)
    if n < 0:
        raise RuntimeError("mo_pairwise_matches failed: %d" % n)
    return out[: 3 * n].reshape(-1, 3)


def gap_anchor_filter(rows):
    """EliminateOverlaps_v2 + LengthFilter(12) on (start0, start1, length) rows."""
    m = np.ascontiguousarray(rows, np.int64).reshape(-1, 3).copy()
    n = lib().mo_gap_anchor_filter(_p(m), len(m))
    return m[:n]


def gap_anchor_search(a, b):
    """pairwiseAnchorSearch on two gap sequences: (weight, anchors rows);
    anchors is None when the weight is below the minimum (no search)."""
    a, b = _u8(a), _u8(b)
    cap = max(min(len(a), len(b)), 16)
    out = np.zeros(3 * cap, np.int64)
    w = ctypes.c_uint32(0)
    n = lib().mo_gap_anchor_search(_p(a), len(a), _p(b), len(b), _p(out), cap, ctypes.byref(w))
    if n == -2:
        return int(w.value), None
    if n < 0:
        raise RuntimeError("mo_gap_anchor_search failed: %d" % n)
    return int(w.value), out[:3 * n].reshape(-1, 3)


def nw_align(a, b):
    """(path string of 'M'/'D'/'I', score) for base codes 0..3."""
    a, b = _u8(a), _u8(b)
    path = ctypes.create_string_buffer(len(a) + len(b) + 1)
    score = ctypes.c_int32(0)
    n = lib().mo_nw_align(_p(a), len(a), _p(b), len(b), path, ctypes.byref(score))
    if n < 0:
        raise ValueError("bad DP input")
    return path.raw[:n].decode(), int(score.value)


def nw_score(a, b):
    a, b = _u8(a), _u8(b)
    return int(lib().mo_nw_score(_p(a), len(a), _p(b), len(b)))


def nw_batch(seq_a, off_a, seq_b, off_b, with_paths=True, nthreads=0):
    """Batch of problems; returns (scores, path_len, paths, path_off)."""
    seq_a, seq_b = _u8(seq_a), _u8(seq_b)
    off_a = np.ascontiguousarray(off_a, np.uint64)
    off_b = np.ascontiguousarray(off_b, np.uint64)
    nprob = len(off_a) - 1
    la = np.diff(off_a.astype(np.int64))
    lb = np.diff(off_b.astype(np.int64))
    path_off = np.zeros(nprob + 1, np.uint64)
    path_off[1:] = np.cumsum(la + lb)
    paths = np.zeros(int(path_off[-1]) if with_paths else 1, np.uint8)
    plen = np.zeros(max(nprob, 1), np.int64)
    scores = np.zeros(max(nprob, 1), np.int32)
    lib().mo_nw_batch(_p(seq_a), _p(off_a), _p(seq_b), _p(off_b), nprob,
                      _p(paths) if with_paths else None, _p(path_off), _p(plen), _p(scores), nthreads)
    return scores[:nprob], plen[:nprob], paths, path_off


# ---- index LUT (lut_oracle.c) ------------------------------------------


class LutIndexError(IndexError):
    pass


def _lut(lut):
    if not (isinstance(lut, np.ndarray) and lut.dtype == np.int32 and lut.ndim == 1 and lut.flags.c_contiguous):
        raise TypeError("LUT must be a contiguous 1-D int32 array")
    return lut


def _check(rc, what):
    if rc == -2:
        raise LutIndexError(what + ": index out of range")
    if rc == -3:
        raise OverflowError(what + ": value does not fit int32")
    if rc < 0:
        raise ValueError(what + ": error %d" % rc)
    return rc


def blocks_arrays(blocks):
    """(g_start, r_start, col_off, g_rows, r_rows) from a list of
    (genome_start, ref_start, genome_row, ref_row) blocks."""
    gs = np.array([b[0] for b in blocks], np.int64)
    rs = np.array([b[1] for b in blocks], np.int64)
    lens = [len(b[2]) for b in blocks]
    for b in blocks:
        if len(b[2]) != len(b[3]):
            raise ValueError("rows of a block differ in length")
    off = np.zeros(len(blocks) + 1, np.uint64)
    off[1:] = np.cumsum(lens, dtype=np.uint64)
    g = np.frombuffer(b"".join(bytes(b[2]) for b in blocks), np.uint8).copy()
    r = np.frombuffer(b"".join(bytes(b[3]) for b in blocks), np.uint8).copy()
    return gs, rs, off, g, r


def lut_from_blocks(blocks, genome_length):
    gs, rs, off, g, r = blocks_arrays(blocks)
    lut = np.empty(genome_length, np.int32)
    _check(lib().mo_lut_from_blocks(_p(gs), _p(rs), _p(off), _p(g), _p(r), len(gs), _p(lut), genome_length),
           "lut_from_blocks")
    return lut


def fix_zero_idx(lut, genome, ref):
    g, r = _u8(genome), _u8(ref)
    _check(lib().mo_fix_zero_idx(_p(_lut(lut)), len(lut), _p(g), len(g), _p(r), len(r)), "fix_zero_idx")


def fill_gaps(lut, max_gap_width=300):
    lib().mo_fill_gaps(_p(_lut(lut)), len(lut), int(max_gap_width))


def smooth_edges(lut, smoothing_radius=20):
    lib().mo_smooth_edges(_p(_lut(lut)), len(lut), int(smoothing_radius))


def find_gaps(lut):
    gaps = np.zeros(len(lut), np.int32)
    lib().mo_find_gaps(_p(_lut(lut)), len(lut), _p(gaps))
    return gaps


def find_edges(lut):
    e = np.zeros(len(lut), np.uint8)
    lib().mo_find_edges(_p(_lut(lut)), len(lut), _p(e))
    return e


def find_mismatches(lut, genome, ref):
    g, r = _u8(genome), _u8(ref)
    m = np.zeros(len(lut), np.uint8)
    _check(lib().mo_find_mismatches(_p(_lut(lut)), len(lut), _p(g), len(g), _p(r), len(r), _p(m)),
           "find_mismatches")
    return m


def find_duplicate_mappings(lut):
    _lut(lut)
    nc = int(max(int(lut.max()), 0)) + 1 if len(lut) else 1
    counts = np.zeros(nc, np.uint32)
    if len(lut) == 0:
        return -1
    rc = lib().mo_find_duplicate_mappings(_p(lut), len(lut), _p(counts), nc)
    if rc == -2:
        raise LutIndexError("find_duplicate_mappings: count table too small")
    return int(rc)
