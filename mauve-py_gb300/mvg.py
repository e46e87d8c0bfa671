"""Python binding of libmauve_gb300 (the C ABI in include/mauve_gb300.h).

Mirrors the reference's seams for the pairwise anchoring and gap-alignment
path of progressiveMauve:

  SortedMerList.create(seq, seed)      -> SortedMerList::Create + Read order
                                          (libMems/SortedMerList.h:89)
  pairwise_matches(a, b, seed)         -> PairwiseMatchFinder::FindMatches
                                          (libMems/MemHash.h:55), the match
                                          list as (start0, start1, length) rows
  gap_align_batch(...)                 -> muscle::GlobalAlign per range
                                          (muscle/libMUSCLE/glbalign.cpp:69)

Every call runs on the GPU through the compiled library; there is no CPU
fallback.  Importing this module on a machine without the built library or
without a CUDA device raises.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmauve_gb300.so")

MVG_OK = 0
MVG_ERR_CAPACITY = 5
_ERRORS = {1: ValueError, 2: RuntimeError, 3: ValueError, 4: ValueError, 5: OverflowError, 6: MemoryError,
           7: RuntimeError, 8: IndexError, 9: OverflowError}

CODING_SEED = 3  # libMems/SeedMasks.h:262
SOLID_SEED = 2 ** 31 - 1

_lib = None
EXPORTS = ["mvg_create", "mvg_destroy", "mvg_last_error", "mvg_stream", "mvg_kernel_launches", "mvg_get_seed",
           "mvg_default_seed_weight", "mvg_seed_length", "mvg_seed_weight", "mvg_sml_build", "mvg_sml_build_dev",
           "mvg_pairwise_matches", "mvg_pairwise_matches_dev", "mvg_pairwise_stats", "mvg_gapdp_batch",
           "mvg_gapdp_batch_dev", "mvg_set_tb_arena", "mvg_probe_int32_peak", "mvg_set_profiling",
           "mvg_stage_times", "mvg_gapdp_banded", "mvg_gapdp_banded_dev", "mvg_set_dp_rows", "mvg_mlp_num_params",
           "mvg_mlp_set_params", "mvg_mlp_get_params", "mvg_band_features_dev", "mvg_mlp_forward_dev",
           "mvg_mlp_grad_dev", "mvg_mlp_train_step_dev", "mvg_band_propose_dev", "mvg_gapdp_envelope_dev",
           "mvg_sml_build_noalloc", "mvg_lut_from_blocks", "mvg_lut_from_blocks_dev", "mvg_lut_fix_zero_idx",
           "mvg_lut_fix_zero_idx_dev", "mvg_lut_fill_gaps", "mvg_lut_fill_gaps_dev", "mvg_lut_smooth_edges",
           "mvg_lut_smooth_edges_dev", "mvg_lut_find_gaps", "mvg_lut_find_gaps_dev", "mvg_lut_find_edges",
           "mvg_lut_find_mismatches", "mvg_lut_find_duplicate_mappings", "mvg_build_index_lut",
           "mvg_build_index_lut_dev", "mvg_set_band_whole_fraction", "mvg_set_band_ring",
           "mvg_set_band_gate", "mvg_sslist_write", "mvg_sslist_read", "mvg_set_pair_bucket_cap",
           "mvg_set_dp_spin_limit", "mvg_gap_anchor_search", "mvg_gap_anchor_search_dev", "mvg_set_dp_graph",
           "mvg_set_dp_coop_strips", "mvg_path_rows", "mvg_path_rows_dev",
           "mvg_xmfa_write", "mvg_xmfa_write_dev", "mvg_set_mlp_tcgen05", "mvg_mlp_tcgen05_passes",
           "mvg_set_dp_checkpoint", "mvg_set_band_whole_full_rows", "mvg_set_ring_max_rows",
           "mvg_recursion_gaps", "mvg_anchor_columns", "mvg_refine_windows", "mvg_search_lcb_gaps",
           "mvg_refine_fast_ranges", "mvg_gapped_alignment", "mvg_search_lcb_gaps_dev", "mvg_lcb_gap_finish",
           "mvg_transpose_matches", "mvg_eliminate_overlaps", "mvg_hmm_backbone_params",
           "mvg_homologous_segments", "mvg_collinear_lcbs"]

TUNING_PATH = os.path.join(HERE, "dp_tuning.json")


class HmmParams(ctypes.Structure):
    """mvg_hmm_params: the backbone-detection HMM's parameters (the members
    of the reference's Params, libMems/HomologyHMM/homology.h:169-177)."""
    _fields_ = [("start_homologous", ctypes.c_double), ("go_homologous", ctypes.c_double),
                ("go_unrelated", ctypes.c_double), ("go_stop_from_unrelated", ctypes.c_double),
                ("go_stop_from_homologous", ctypes.c_double), ("emit_homologous", ctypes.c_double * 8),
                ("emit_unrelated", ctypes.c_double * 8)]

    def to_array(self):
        return np.array([self.start_homologous, self.go_homologous, self.go_unrelated, self.go_stop_from_unrelated,
                         self.go_stop_from_homologous, *self.emit_homologous, *self.emit_unrelated], np.float64)


def load_library(path=LIB_PATH):
    """Loads the shared library (raises OSError if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("libmauve_gb300.so is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    vp, u64, i64, ci = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int
    sig = {
        "mvg_create": (ci, [ctypes.POINTER(vp), ci]),
        "mvg_destroy": (ci, [vp]),
        "mvg_last_error": (ctypes.c_char_p, []),
        "mvg_stream": (vp, [vp]),
        "mvg_kernel_launches": (u64, [vp]),
        "mvg_get_seed": (u64, [ci, ci]),
        "mvg_default_seed_weight": (ctypes.c_uint, [u64]),
        "mvg_seed_length": (ci, [u64]),
        "mvg_seed_weight": (ci, [u64]),
        "mvg_sml_build": (ci, [vp, vp, u64, u64, vp, vp, u64, ctypes.POINTER(u64)]),
        "mvg_sml_build_dev": (ci, [vp, vp, u64, u64, vp, vp, u64, ctypes.POINTER(u64)]),
        "mvg_pairwise_matches": (ci, [vp, vp, u64, vp, u64, u64, vp, u64, ctypes.POINTER(u64)]),
        "mvg_pairwise_matches_dev": (ci, [vp, vp, u64, vp, u64, u64, vp, u64, ctypes.POINTER(u64)]),
        "mvg_pairwise_stats": (ci, [vp, vp]),
        "mvg_gap_anchor_search": (ci, [vp, vp, u64, vp, u64, vp, u64, vp, u64, vp, ctypes.POINTER(u64)]),
        "mvg_gap_anchor_search_dev": (ci, [vp, vp, u64, vp, u64, vp, u64, vp, u64, vp, ctypes.POINTER(u64)]),
        "mvg_gapdp_batch": (ci, [vp, vp, vp, vp, vp, i64, vp, vp, vp, vp]),
        "mvg_gapdp_batch_dev": (ci, [vp, vp, vp, vp, vp, i64, vp, vp, vp, vp]),
        "mvg_set_tb_arena": (ci, [vp, u64]),
        "mvg_probe_int32_peak": (ci, [vp, ctypes.POINTER(ctypes.c_double)]),
        "mvg_gapdp_banded": (ci, [vp, vp, vp, vp, vp, i64, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(u64)]),
        "mvg_gapdp_banded_dev": (ci, [vp, vp, vp, vp, vp, i64, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(u64)]),
        "mvg_set_dp_rows": (ci, [vp, ci, ci]),
        "mvg_set_band_whole_fraction": (ci, [vp, ctypes.c_double]),
        "mvg_set_band_ring": (ci, [vp, ci]),
        "mvg_set_band_gate": (ci, [vp, ci]),
        "mvg_set_pair_bucket_cap": (ci, [vp, ci]),
        "mvg_set_dp_spin_limit": (ci, [vp, ctypes.c_longlong]),
        "mvg_set_dp_graph": (ci, [vp, ci]),
        "mvg_set_dp_checkpoint": (ci, [vp, ci]),
        "mvg_set_band_whole_full_rows": (ci, [vp, i64]),
        "mvg_set_ring_max_rows": (ci, [vp, ci]),
        "mvg_recursion_gaps": (ci, [vp, vp, u64, i64, ci, i64, ci, u64, u64, i64, vp, u64, ctypes.POINTER(u64), vp]),
        "mvg_anchor_columns": (ci, [vp, vp, u64, vp, u64, ctypes.POINTER(u64)]),
        "mvg_refine_windows": (ci, [vp, vp, u64, ctypes.c_double, vp, u64, ctypes.POINTER(u64)]),
        "mvg_refine_fast_ranges": (ci, [vp, vp, u64, ctypes.c_double, vp, u64, ctypes.POINTER(u64)]),
        "mvg_gapped_alignment": (ci, [vp, vp, vp, vp, i64, ctypes.c_double, ci, vp, vp, vp, u64]),
        "mvg_hmm_backbone_params": (ci, [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.POINTER(HmmParams)]),
        "mvg_homologous_segments": (ci, [vp, vp, vp, i64, ctypes.POINTER(HmmParams), ci, ci, vp, u64,
                                         ctypes.POINTER(u64), vp]),
        "mvg_search_lcb_gaps": (ci, [vp, vp, u64, vp, u64, vp, u64, vp, u64, vp, u64, ctypes.POINTER(u64),
                                     ctypes.POINTER(ctypes.c_uint32)]),
        "mvg_search_lcb_gaps_dev": (ci, [vp, vp, u64, vp, u64, vp, u64, vp, u64, vp, u64, ctypes.POINTER(u64),
                                         ctypes.POINTER(ctypes.c_uint32)]),
        "mvg_lcb_gap_finish": (ci, [vp, u64, vp, u64, vp, u64, vp, u64, ctypes.POINTER(u64)]),
        "mvg_transpose_matches": (ci, [vp, u64, ctypes.c_uint, vp, u64, vp, u64, ctypes.POINTER(u64)]),
        "mvg_eliminate_overlaps": (ci, [vp, u64, vp, u64, ctypes.POINTER(u64)]),
        "mvg_collinear_lcbs": (ci, [vp, u64, vp, vp, u64, ctypes.POINTER(u64), vp, ctypes.POINTER(u64)]),
        "mvg_set_mlp_tcgen05": (ci, [vp, ci]),
        "mvg_mlp_tcgen05_passes": (ci, [vp, ctypes.POINTER(ctypes.c_uint64)]),
        "mvg_set_dp_coop_strips": (ci, [vp, ci]),
        "mvg_path_rows": (ci, [vp, vp, vp, vp, vp, i64, vp, vp, vp, vp, vp]),
        "mvg_xmfa_write": (ci, [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i64, vp, vp, vp, vp, vp, vp,
                                u64, ctypes.POINTER(u64)]),
        "mvg_xmfa_write_dev": (ci, [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i64, vp, vp, vp, vp, vp,
                                    vp, u64, ctypes.POINTER(u64)]),
        "mvg_path_rows_dev": (ci, [vp, vp, vp, vp, vp, i64, vp, vp, vp, vp, vp]),
        "mvg_sslist_write": (ci, [vp, vp, u64, u64, ctypes.c_char_p]),
        "mvg_sslist_read": (ci, [ctypes.c_char_p, vp, vp, u64, vp, u64]),
        "mvg_gapdp_envelope_dev": (ci, [vp, vp, vp, vp, vp, i64, vp, vp]),
        "mvg_mlp_num_params": (i64, []),
        "mvg_mlp_set_params": (ci, [vp, vp]),
        "mvg_mlp_get_params": (ci, [vp, vp]),
        "mvg_band_features_dev": (ci, [vp, vp, vp, vp, vp, i64, vp]),
        "mvg_mlp_forward_dev": (ci, [vp, vp, i64, vp]),
        "mvg_mlp_grad_dev": (ci, [vp, vp, vp, i64, vp, vp]),
        "mvg_mlp_train_step_dev": (ci, [vp, vp, vp, i64, ctypes.c_float, ci, vp]),
        "mvg_band_propose_dev": (ci, [vp, vp, vp, vp, vp, i64, ctypes.c_float, ctypes.c_float, vp, vp]),
        "mvg_set_profiling": (ci, [vp, ci]),
        "mvg_stage_times": (ci, [vp, ctypes.c_char_p, ctypes.c_size_t, vp, ci, ctypes.POINTER(ci)]),
        "mvg_lut_from_blocks": (ci, [vp, vp, vp, vp, vp, vp, u64, vp, u64]),
        "mvg_lut_from_blocks_dev": (ci, [vp, vp, vp, vp, vp, vp, u64, vp, u64]),
        "mvg_lut_fix_zero_idx": (ci, [vp, vp, u64, vp, u64, vp, u64]),
        "mvg_lut_fix_zero_idx_dev": (ci, [vp, vp, u64, vp, u64, vp, u64]),
        "mvg_lut_fill_gaps": (ci, [vp, vp, u64, ci]),
        "mvg_lut_fill_gaps_dev": (ci, [vp, vp, u64, ci]),
        "mvg_lut_smooth_edges": (ci, [vp, vp, u64, ci]),
        "mvg_lut_smooth_edges_dev": (ci, [vp, vp, u64, ci]),
        "mvg_lut_find_gaps": (ci, [vp, vp, u64, vp]),
        "mvg_lut_find_gaps_dev": (ci, [vp, vp, u64, vp]),
        "mvg_lut_find_edges": (ci, [vp, vp, u64, vp]),
        "mvg_lut_find_mismatches": (ci, [vp, vp, u64, vp, u64, vp, u64, vp]),
        "mvg_lut_find_duplicate_mappings": (ci, [vp, vp, u64, ctypes.POINTER(i64)]),
        "mvg_build_index_lut": (ci, [vp, vp, vp, vp, vp, vp, u64, vp, u64, vp, u64, ci, ci, ci, ci, vp, u64]),
        "mvg_build_index_lut_dev": (ci, [vp, vp, vp, vp, vp, vp, u64, vp, u64, vp, u64, ci, ci, ci, ci, vp, u64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != MVG_OK:
        msg = load_library().mvg_last_error().decode(errors="replace")
        raise _ERRORS.get(rc, RuntimeError)("libmauve_gb300 error %d: %s" % (rc, msg))


def wait_producers():
    """Device inputs reach the library as raw pointers, usually written by
    torch kernels on torch's current stream, while the library runs on the
    handle's own stream: finish that producer work before a device call."""
    t = sys.modules.get("torch")
    if t is not None and t.cuda.is_initialized():
        t.cuda.current_stream().synchronize()


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _u8(seq):
    if isinstance(seq, (bytes, bytearray)):
        return np.frombuffer(bytes(seq), np.uint8)
    if isinstance(seq, str):
        return np.frombuffer(seq.encode(), np.uint8)
    return np.ascontiguousarray(seq, dtype=np.uint8)


def get_seed(weight, rank=0):
    """getSeed (libMems/SeedMasks.h:298-321)."""
    return int(load_library().mvg_get_seed(weight, rank))


def default_seed_weight(avg_len):
    """getDefaultSeedWeight (libMems/SeedMasks.h:389-401)."""
    return int(load_library().mvg_default_seed_weight(avg_len))


def seed_length(seed):
    return int(load_library().mvg_seed_length(seed))


def seed_weight(seed):
    return int(load_library().mvg_seed_weight(seed))


def recursion_gaps(row_a, row_b, left_end_a, reverse_a, left_end_b, reverse_b, genome_len_a, genome_len_b,
                   min_gap=200):
    """recurseOnPairs' gap finding for one LCB of two genomes (no GPU needed;
    see mvg_recursion_gaps).  Returns (gaps int64[k, 4] as (start A, length A,
    start B, length B), ready for Context.gap_anchor_search, and the flanks
    int64[2, 2, 2]: per genome up to two 1-based [start, end) stretches)."""
    a, b = _u8(row_a), _u8(row_b)
    if len(a) != len(b):
        raise ValueError("rows of different length")
    L = load_library()
    n = ctypes.c_uint64(0)
    flanks = np.zeros(8, np.int64)
    args = (_ptr(a), _ptr(b), len(a), int(left_end_a), int(bool(reverse_a)), int(left_end_b), int(bool(reverse_b)),
            int(genome_len_a), int(genome_len_b), int(min_gap))
    cap = max(1, len(a) // max(1, int(min_gap)) + 2)
    gaps = np.zeros(4 * cap, np.int64)
    rc = L.mvg_recursion_gaps(*args, _ptr(gaps), cap, ctypes.byref(n), _ptr(flanks))
    if rc == MVG_ERR_CAPACITY:
        cap = int(n.value)
        gaps = np.zeros(4 * cap, np.int64)
        rc = L.mvg_recursion_gaps(*args, _ptr(gaps), cap, ctypes.byref(n), _ptr(flanks))
    _check(rc)
    return gaps[:4 * int(n.value)].reshape(-1, 4), flanks.reshape(2, 2, 2)


def _matches(m):
    return np.ascontiguousarray(m, np.int64).reshape(-1, 3)


def _regions(r):
    return np.ascontiguousarray(r if r is not None else [], np.int64).reshape(-1)


def _host_matches(call, n_in):
    """Runs a host match-list step with a growing output buffer."""
    cap = 2 * n_in + 16
    cnt = ctypes.c_uint64(0)
    while True:
        out = np.zeros(3 * cap, np.int64)
        rc = call(out, cap, cnt)
        if rc == MVG_ERR_CAPACITY and cnt.value > cap:
            cap = int(cnt.value)
            continue
        _check(rc)
        return out[:3 * int(cnt.value)].reshape(-1, 3)


def transpose_matches(matches, seq, regions):
    """transposeMatches (libMems/Aligner.cpp:973-1045) for genome seq of
    two-genome matches (rows: start A, start B, length; libMems' signed
    1-based starts) given the 1-based (left, right + 1) regions the
    concatenation was cut from (no GPU needed)."""
    m, r = _matches(matches), _regions(regions)
    L = load_library()
    return _host_matches(lambda out, cap, cnt: L.mvg_transpose_matches(_ptr(m), len(m), int(seq), _ptr(r), len(r),
                                                                       _ptr(out), cap, ctypes.byref(cnt)), len(m))


def eliminate_overlaps(matches):
    """EliminateOverlaps (libMems/Aligner.cpp:62-176) for two-genome matches
    (no GPU needed)."""
    m = _matches(matches)
    L = load_library()
    return _host_matches(lambda out, cap, cnt: L.mvg_eliminate_overlaps(_ptr(m), len(m), _ptr(out), cap,
                                                                        ctypes.byref(cnt)), len(m))


def collinear_lcbs(matches):
    """LCBs of a two-genome match list for collinear genomes, with greedy
    breakpoint elimination (the collinear branch of alignProfileToProfile,
    libMems/ProgressiveAligner.cpp:2281-2303; no GPU needed).  Returns (the
    LCBs, each an int64[k, 3] match list in the reference's order, the
    deleted matches as int64[d, 3])."""
    m = _matches(matches)
    L = load_library()
    n = len(m)
    out = np.zeros(3 * max(n, 1), np.int64)
    deleted = np.zeros(3 * max(n, 1), np.int64)
    off = np.zeros(n + 2, np.uint64)
    nlcb, ndel = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(L.mvg_collinear_lcbs(_ptr(m), n, _ptr(out), _ptr(off), len(off), ctypes.byref(nlcb), _ptr(deleted),
                                ctypes.byref(ndel)))
    o = off[:nlcb.value + 1].astype(np.int64)
    rows = out.reshape(-1, 3)
    return [rows[o[k]:o[k + 1]].copy() for k in range(nlcb.value)], deleted[:3 * ndel.value].reshape(-1, 3)


def lcb_gap_finish(matches, regions_a, regions_b):
    """The steps SearchLCBGaps takes after its search (no GPU needed; see
    mvg_lcb_gap_finish): matches of the two concatenations -> matches in
    genome coordinates."""
    m, ra, rb = _matches(matches), _regions(regions_a), _regions(regions_b)
    L = load_library()
    return _host_matches(lambda out, cap, cnt: L.mvg_lcb_gap_finish(_ptr(m), len(m), _ptr(ra), len(ra), _ptr(rb),
                                                                    len(rb), _ptr(out), cap, ctypes.byref(cnt)),
                         len(m))


def lcb_gap_regions(flanks):
    """The regions outside the LCBs, as alignPP hands them to SearchLCBGaps
    (libMems/ProgressiveAligner.cpp:2474-2488): every LCB's flanks (the
    second value recursion_gaps returns, int64[2, 2, 2]) collected per genome
    and each genome's boundary list sorted.  Returns (regions A, regions B)."""
    per = [[], []]
    for fl in flanks:
        fl = np.asarray(fl, np.int64).reshape(2, 2, 2)
        for q in range(2):
            for lo, hi in fl[q]:
                if lo < hi:
                    per[q] += [int(lo), int(hi)]
    return tuple(np.sort(np.array(p, np.int64)) for p in per)


def anchor_columns(row_a, row_b):
    """Anchor columns of a window of a two-genome alignment (no GPU needed;
    see mvg_anchor_columns): uint32 array, ascending."""
    a, b = _u8(row_a), _u8(row_b)
    if len(a) != len(b):
        raise ValueError("rows of different length")
    n = ctypes.c_uint64(0)
    cols = np.zeros(max(1, len(a)), np.uint32)
    _check(load_library().mvg_anchor_columns(_ptr(a), _ptr(b), len(a), _ptr(cols), len(cols), ctypes.byref(n)))
    return cols[:int(n.value)].copy()


def refine_windows(row_a, row_b, max_window_size=20000.0):
    """refineAlignment's windows of one LCB of two genomes (no GPU needed;
    see mvg_refine_windows): int64[k, 3] rows (first column, end column,
    1 for a gap window)."""
    a, b = _u8(row_a), _u8(row_b)
    if len(a) != len(b):
        raise ValueError("rows of different length")
    L = load_library()
    n = ctypes.c_uint64(0)
    cap = 16
    while True:
        w = np.zeros(3 * cap, np.int64)
        rc = L.mvg_refine_windows(_ptr(a), _ptr(b), len(a), float(max_window_size), _ptr(w), cap, ctypes.byref(n))
        if rc == MVG_ERR_CAPACITY:
            cap = int(n.value)
            continue
        _check(rc)
        return w[:3 * int(n.value)].reshape(-1, 3)


def refine_fast_ranges(row_a, row_b, max_window_size=20000.0):
    """The column ranges the final iterative-refinement pass realigns in one
    LCB of two genomes (no GPU needed; see mvg_refine_fast_ranges):
    int64[k, 2] rows (first column, end column)."""
    a, b = _u8(row_a), _u8(row_b)
    if len(a) != len(b):
        raise ValueError("rows of different length")
    L = load_library()
    n = ctypes.c_uint64(0)
    cap = max(16, len(a) // 200 + 8)
    while True:
        r = np.zeros(2 * cap, np.int64)
        rc = L.mvg_refine_fast_ranges(_ptr(a), _ptr(b), len(a), float(max_window_size), _ptr(r), cap,
                                      ctypes.byref(n))
        if rc == MVG_ERR_CAPACITY:
            cap = int(n.value)
            continue
        _check(rc)
        return r[:2 * int(n.value)].reshape(-1, 2)


def hmm_backbone_params(gc_content, go_homologous=0.00001, go_unrelated=0.000000001, pct_identity=0.7):
    """The backbone HMM's parameters as progressiveMauve's applyBackbone sets
    them (mauveAligner/src/progressiveMauve.cpp:226-238; its defaults)."""
    p = HmmParams()
    _check(load_library().mvg_hmm_backbone_params(float(gc_content), float(go_homologous), float(go_unrelated),
                                                   float(pct_identity), ctypes.byref(p)))
    return p


def homologous_segments(lcbs, params, left_homologous=True, right_homologous=True):
    """findHssHomologyHMM for LCBs of two genomes (no GPU needed; see
    mvg_homologous_segments): for each (row A, row B), the homologous column
    ranges as int64[k, 2] (first, last column, inclusive)."""
    rows = [(_u8(ra), _u8(rb)) for ra, rb in lcbs]
    if not rows:
        return []
    ra = np.concatenate([r[0] for r in rows])
    rb = np.concatenate([r[1] for r in rows])
    off = np.zeros(len(rows) + 1, np.uint64)
    off[1:] = np.cumsum([len(r[0]) for r in rows])
    seg_off = np.zeros(len(rows) + 1, np.uint64)
    n = ctypes.c_uint64(0)
    cap = max(16, len(ra) // 64)
    L = load_library()
    while True:
        segs = np.zeros(2 * cap, np.int64)
        rc = L.mvg_homologous_segments(_ptr(ra), _ptr(rb), _ptr(off), len(rows), ctypes.byref(params),
                                       int(bool(left_homologous)), int(bool(right_homologous)), _ptr(segs), cap,
                                       ctypes.byref(n), _ptr(seg_off))
        if rc == MVG_ERR_CAPACITY:
            cap = int(n.value)
            continue
        _check(rc)
        return [segs[2 * int(seg_off[k]):2 * int(seg_off[k + 1])].reshape(-1, 2) for k in range(len(rows))]


def anchored_problems(row_a, row_b):
    """The gap-DP problems of a window cut at its anchor columns: a list of
    (column range (left, right), A's bases, B's bases) for every range of at
    least one column, in order (AnchoredProfileProfile's loop)."""
    a, b = _u8(row_a), _u8(row_b)
    cols = anchor_columns(a, b)
    edges = [0] + [int(c) for c in cols] + [len(a)]
    out = []
    gap = np.frombuffer(b"-.", np.uint8)
    for lo, hi in zip(edges[:-1], edges[1:]):
        if hi <= lo:
            continue
        ra, rb = a[lo:hi], b[lo:hi]
        out.append(((lo, hi), ra[~np.isin(ra, gap)], rb[~np.isin(rb, gap)]))
    return out


class SslistInfo(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("seed_length", ctypes.c_uint32), ("seed_weight", ctypes.c_uint32),
                ("length", ctypes.c_uint64), ("words", ctypes.c_uint64), ("entries", ctypes.c_uint64),
                ("circular", ctypes.c_int), ("status", ctypes.c_int)]


def sslist_read(path):
    """(info, packed words, positions) of a .sslist file (no GPU needed)."""
    L = load_library()
    info = SslistInfo()
    p = os.fsencode(path)
    rc = L.mvg_sslist_read(p, ctypes.byref(info), None, 0, None, 0)
    if rc:
        raise RuntimeError("mvg error %d (status %d): %s" % (rc, info.status, L.mvg_last_error().decode()))
    words = np.zeros(max(int(info.words), 1), np.uint32)
    pos = np.zeros(max(int(info.entries), 1), np.uint32)
    _check(L.mvg_sslist_read(p, ctypes.byref(info), _ptr(words), int(info.words), _ptr(pos), int(info.entries)))
    return info, words[:info.words], pos[:info.entries]


class Context:
    """A CUDA device, a stream and the device workspaces (opaque handle)."""

    def __init__(self, device=0):
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.mvg_create(ctypes.byref(h), device))
        self._h = h
        self.device = device
        self.full_rows, self.band_rows = 8, 4
        if os.path.exists(TUNING_PATH):  # committed autotuner choice
            import json
            with open(TUNING_PATH) as f:
                t = json.load(f)
            self.set_dp_rows(int(t.get("full_rows_per_lane", 8)), int(t.get("band_rows_per_lane", 4)))
            self.set_dp_coop_strips(int(t.get("coop_min_strips", 16)))

    def set_band_whole_fraction(self, fraction):
        """Bands covering at least this share of their matrix run whole (default 0.5)."""
        _check(load_library().mvg_set_band_whole_fraction(self._h, float(fraction)))

    def set_pair_bucket_cap(self, cap):
        """Largest seed-join bucket sorted in shared memory (32..3072); see mvg_set_pair_bucket_cap."""
        _check(load_library().mvg_set_pair_bucket_cap(self._h, int(cap)))

    def set_band_gate(self, min_match):
        """Divergence gate of the band proposal (0 = off); see mvg_set_band_gate."""
        _check(load_library().mvg_set_band_gate(self._h, int(min_match)))

    def set_dp_spin_limit(self, polls=1 << 26):
        """Polls before a whole-CTA gap-DP wait gives up (watchdog); see mvg_set_dp_spin_limit."""
        _check(load_library().mvg_set_dp_spin_limit(self._h, int(polls)))

    def set_dp_coop_strips(self, strips):
        """Full-DP problems of at least this many strips go to a whole CTA; see mvg_set_dp_coop_strips."""
        _check(load_library().mvg_set_dp_coop_strips(self._h, int(strips)))

    def set_mlp_tcgen05(self, on=True):
        """MLP forward hidden layers on tcgen05 (default) or on mma.sync GEMMs; see mvg_set_mlp_tcgen05."""
        _check(load_library().mvg_set_mlp_tcgen05(self._h, 1 if on else 0))

    def mlp_tcgen05_passes(self):
        """Forward passes of this handle's MLP that ran on tcgen05."""
        n = ctypes.c_uint64(0)
        _check(load_library().mvg_mlp_tcgen05_passes(self._h, ctypes.byref(n)))
        return n.value

    def set_ring_max_rows(self, rows):
        """Banded calls: tallest ring group height used (taller bands run in the strip kernel)."""
        _check(load_library().mvg_set_ring_max_rows(self._h, int(rows)))

    def set_band_whole_full_rows(self, rows):
        """Banded calls: whole-matrix problems from this many rows of A run in the full DP."""
        _check(load_library().mvg_set_band_whole_full_rows(self._h, int(rows)))

    def set_dp_checkpoint(self, on=True):
        """Full gap-DP passes checkpointed (default) or with stored traceback bits; see mvg_set_dp_checkpoint."""
        _check(load_library().mvg_set_dp_checkpoint(self._h, 1 if on else 0))

    def set_dp_graph(self, on=True):
        """Gap-DP waves as one recorded CUDA graph (default) or launched one by one."""
        _check(load_library().mvg_set_dp_graph(self._h, 1 if on else 0))

    def set_band_ring(self, on=True):
        """Banded passes on the ring schedule (default) or all in the strip kernel."""
        _check(load_library().mvg_set_band_ring(self._h, 1 if on else 0))

    def set_dp_rows(self, full_rows, band_rows=None):
        band_rows = self.band_rows if band_rows is None else band_rows
        _check(load_library().mvg_set_dp_rows(self._h, int(full_rows), int(band_rows)))
        self.full_rows, self.band_rows = int(full_rows), int(band_rows)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self):
        return load_library().mvg_stream(self._h)

    def kernel_launches(self):
        return int(load_library().mvg_kernel_launches(self._h))

    def close(self):
        if self._h:
            load_library().mvg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ seeds
    def sml_build(self, seq, seed, with_mers=True):
        """Sorted mer list: (positions sorted by canonical mer, canonical mers)."""
        s = _u8(seq)
        L = seed_length(seed)
        cnt = len(s) - L + 1 if len(s) >= L else 0
        pos = np.zeros(max(cnt, 1), np.uint32)
        mer = np.zeros(max(cnt, 1), np.uint64) if with_mers else None
        out = ctypes.c_uint64(0)
        _check(load_library().mvg_sml_build(self._h, _ptr(s), len(s), seed, _ptr(pos), _ptr(mer), cnt,
                                            ctypes.byref(out)))
        return pos[:cnt], (mer[:cnt] if with_mers else None)

    def sslist_write(self, seq, seed, path):
        """Builds the SML of seq and writes it as a .sslist file."""
        a = _u8(seq)
        _check(load_library().mvg_sslist_write(self._h, _ptr(a), len(a), int(seed), os.fsencode(path)))

    def sml_build_dev(self, d_seq_ptr, n, seed, d_pos_ptr, d_mer_ptr, cap):
        wait_producers()
        out = ctypes.c_uint64(0)
        _check(load_library().mvg_sml_build_dev(self._h, d_seq_ptr, n, seed, d_pos_ptr, d_mer_ptr, cap,
                                                ctypes.byref(out)))
        return int(out.value)

    # ---------------------------------------------------------- matches
    def pairwise_matches(self, a, b, seed, cap=None):
        """MatchList of the genome pair as int64 rows (start0, start1, length)."""
        a, b = _u8(a), _u8(b)
        if cap is None:
            cap = max(min(len(a), len(b)) // 4, 1024)
        while True:
            out = np.zeros(3 * cap, np.int64)
            cnt = ctypes.c_uint64(0)
            rc = load_library().mvg_pairwise_matches(self._h, _ptr(a), len(a), _ptr(b), len(b), seed, _ptr(out),
                                                     cap, ctypes.byref(cnt))
            if rc == 5 and cnt.value > cap:
                cap = int(cnt.value)
                continue
            _check(rc)
            return out[: 3 * cnt.value].reshape(-1, 3)

    def pairwise_matches_dev(self, d_a, na, d_b, nb, seed, d_out, cap):
        wait_producers()
        cnt = ctypes.c_uint64(0)
        _check(load_library().mvg_pairwise_matches_dev(self._h, d_a, na, d_b, nb, seed, d_out, cap,
                                                       ctypes.byref(cnt)))
        return int(cnt.value)

    def gap_anchor_search(self, seq_a, seq_b, gaps):
        """Batched pairwiseAnchorSearch over gaps (rows: start A, length A,
        start B, length B; 0-based).  Returns (anchors int64[m, 3] in genome
        coordinates, gap_off uint64[ngaps + 1])."""
        seq_a, seq_b = _u8(seq_a), _u8(seq_b)
        g = np.ascontiguousarray(gaps, np.int64).reshape(-1, 4)
        n = len(g)
        off = np.zeros(n + 1, np.uint64)
        cnt = ctypes.c_uint64(0)
        cap = int(max(16, min(len(seq_a), len(seq_b)) // 4))
        while True:
            out = np.zeros(3 * cap, np.int64)
            rc = load_library().mvg_gap_anchor_search(self._h, _ptr(seq_a), len(seq_a), _ptr(seq_b), len(seq_b),
                                                      _ptr(g), n, _ptr(out), cap, _ptr(off), ctypes.byref(cnt))
            if rc == MVG_ERR_CAPACITY and cnt.value > cap:
                cap = int(cnt.value)
                continue
            _check(rc)
            return out[: 3 * cnt.value].reshape(-1, 3), off

    def gap_anchor_search_dev(self, d_a, na, d_b, nb, gaps, cap):
        """Device-genome variant; gaps and outputs on the host."""
        wait_producers()
        g = np.ascontiguousarray(gaps, np.int64).reshape(-1, 4)
        off = np.zeros(len(g) + 1, np.uint64)
        out = np.zeros(3 * max(cap, 1), np.int64)
        cnt = ctypes.c_uint64(0)
        _check(load_library().mvg_gap_anchor_search_dev(self._h, d_a, na, d_b, nb, _ptr(g), len(g), _ptr(out), cap,
                                                        _ptr(off), ctypes.byref(cnt)))
        return out[: 3 * cnt.value].reshape(-1, 3), off

    def search_lcb_gaps(self, seq_a, seq_b, regions_a, regions_b):
        """SearchLCBGaps for two genomes (mvg_search_lcb_gaps): regions are
        1-based (left, right + 1) boundaries per genome, as lcb_gap_regions
        gives them.  Returns (matches int64[m, 3] as (start A, start B,
        length) in genome coordinates, seed weight)."""
        seq_a, seq_b = _u8(seq_a), _u8(seq_b)
        ra, rb = _regions(regions_a), _regions(regions_b)
        w = ctypes.c_uint32(0)
        L = load_library()
        m = _host_matches(lambda out, cap, cnt: L.mvg_search_lcb_gaps(
            self._h, _ptr(seq_a), len(seq_a), _ptr(seq_b), len(seq_b), _ptr(ra), len(ra), _ptr(rb), len(rb),
            _ptr(out), cap, ctypes.byref(cnt), ctypes.byref(w)), (int(np.diff(ra.reshape(-1, 2)).sum()) if len(ra)
                                                                    else 0) // 8)
        return m, int(w.value)

    def search_lcb_gaps_dev(self, d_a, na, d_b, nb, regions_a, regions_b, cap):
        """Device-genome variant; regions and output on the host."""
        wait_producers()
        ra, rb = _regions(regions_a), _regions(regions_b)
        out = np.zeros(3 * max(cap, 1), np.int64)
        cnt = ctypes.c_uint64(0)
        w = ctypes.c_uint32(0)
        _check(load_library().mvg_search_lcb_gaps_dev(self._h, d_a, na, d_b, nb, _ptr(ra), len(ra), _ptr(rb),
                                                      len(rb), _ptr(out), cap, ctypes.byref(cnt),
                                                      ctypes.byref(w)))
        return out[:3 * int(cnt.value)].reshape(-1, 3), int(w.value)

    def pairwise_stats(self):
        st = np.zeros(4, np.uint64)
        _check(load_library().mvg_pairwise_stats(self._h, _ptr(st)))
        return dict(pairs=int(st[0]), collisions=int(st[1]), matches=int(st[2]), buckets=int(st[3]))

    # ----------------------------------------------------------- gap DP
    def set_tb_arena(self, nbytes):
        _check(load_library().mvg_set_tb_arena(self._h, int(nbytes)))

    def gap_align_batch(self, seq_a, off_a, seq_b, off_b, with_paths=True):
        """Batched NWSmall.  Returns (scores int32[n], paths list of str or None)."""
        seq_a, seq_b = _u8(seq_a), _u8(seq_b)
        off_a = np.ascontiguousarray(off_a, np.uint64)
        off_b = np.ascontiguousarray(off_b, np.uint64)
        n = len(off_a) - 1
        scores = np.zeros(max(n, 1), np.int32)
        if with_paths:
            la = np.diff(off_a.astype(np.int64))
            lb = np.diff(off_b.astype(np.int64))
            path_off = np.zeros(n + 1, np.uint64)
            path_off[1:] = np.cumsum(la + lb)
            paths = np.zeros(int(path_off[-1]) + 1, np.uint8)
            plen = np.zeros(max(n, 1), np.int64)
            _check(load_library().mvg_gapdp_batch(self._h, _ptr(seq_a), _ptr(off_a), _ptr(seq_b), _ptr(off_b), n,
                                                  _ptr(scores), _ptr(paths), _ptr(path_off), _ptr(plen)))
            raw = paths.tobytes()
            out = [raw[int(path_off[k]):int(path_off[k]) + int(plen[k])].decode() for k in range(n)]
            return scores[:n], out
        _check(load_library().mvg_gapdp_batch(self._h, _ptr(seq_a), _ptr(off_a), _ptr(seq_b), _ptr(off_b), n,
                                              _ptr(scores), None, None, None))
        return scores[:n], None

    def gap_align_banded(self, seq_a, off_a, seq_b, off_b, band_delta, band_half, with_paths=True):
        """Banded NWSmall with the exactness check and full-DP fallback.
        Returns (scores, paths or None, status uint8[n], cells computed); status
        1 = banded result kept, 0 = band rejected (full DP), 2 = band not tried."""
        seq_a, seq_b = _u8(seq_a), _u8(seq_b)
        off_a = np.ascontiguousarray(off_a, np.uint64)
        off_b = np.ascontiguousarray(off_b, np.uint64)
        n = len(off_a) - 1
        delta = np.ascontiguousarray(band_delta, np.int32)
        half = np.ascontiguousarray(band_half, np.int32)
        scores = np.zeros(max(n, 1), np.int32)
        used = np.zeros(max(n, 1), np.uint8)
        cells = ctypes.c_uint64(0)
        if with_paths:
            la = np.diff(off_a.astype(np.int64))
            lb = np.diff(off_b.astype(np.int64))
            path_off = np.zeros(n + 1, np.uint64)
            path_off[1:] = np.cumsum(la + lb)
            paths = np.zeros(int(path_off[-1]) + 1, np.uint8)
            plen = np.zeros(max(n, 1), np.int64)
            _check(load_library().mvg_gapdp_banded(self._h, _ptr(seq_a), _ptr(off_a), _ptr(seq_b), _ptr(off_b), n,
                                                   _ptr(delta), _ptr(half), _ptr(scores), _ptr(paths),
                                                   _ptr(path_off), _ptr(plen), _ptr(used), ctypes.byref(cells)))
            raw = paths.tobytes()
            out = [raw[int(path_off[k]):int(path_off[k]) + int(plen[k])].decode() for k in range(n)]
            return scores[:n], out, used[:n].copy(), int(cells.value)
        _check(load_library().mvg_gapdp_banded(self._h, _ptr(seq_a), _ptr(off_a), _ptr(seq_b), _ptr(off_b), n,
                                               _ptr(delta), _ptr(half), _ptr(scores), None, None, None, _ptr(used),
                                               ctypes.byref(cells)))
        return scores[:n], None, used[:n].copy(), int(cells.value)

    def gap_align_banded_dev(self, d_sa, d_oa, d_sb, d_ob, n, band_delta, band_half, d_scores, d_paths, d_path_off,
                             d_path_len):
        """Device-buffer banded call; band arrays and the returned status (1 kept, 0 rejected, 2 not
        tried) are host numpy arrays."""
        wait_producers()
        delta = np.ascontiguousarray(band_delta, np.int32)
        half = np.ascontiguousarray(band_half, np.int32)
        used = np.zeros(max(n, 1), np.uint8)
        cells = ctypes.c_uint64(0)
        _check(load_library().mvg_gapdp_banded_dev(self._h, d_sa, d_oa, d_sb, d_ob, n, _ptr(delta), _ptr(half),
                                                   d_scores, d_paths, d_path_off, d_path_len, _ptr(used),
                                                   ctypes.byref(cells)))
        return used[:n].copy(), int(cells.value)

    def path_rows(self, seq_a, off_a, seq_b, off_b, paths):
        """AlignTwoMSAsGivenPath for a batch: the two gapped rows (bytes, '-'
        for gaps) of each problem from its path (a list of 'M'/'D'/'I' strings)."""
        seq_a, seq_b = _u8(seq_a), _u8(seq_b)
        off_a = np.ascontiguousarray(off_a, np.uint64)
        off_b = np.ascontiguousarray(off_b, np.uint64)
        n = len(off_a) - 1
        plen = np.array([len(p) for p in paths], np.int64)
        poff = np.zeros(n + 1, np.uint64)
        poff[1:] = np.cumsum(plen)
        flat = np.frombuffer("".join(paths).encode() or b"\0", np.uint8)
        ra = np.zeros(max(int(poff[-1]), 1), np.uint8)
        rb = np.zeros(max(int(poff[-1]), 1), np.uint8)
        _check(load_library().mvg_path_rows(self._h, _ptr(seq_a), _ptr(off_a), _ptr(seq_b), _ptr(off_b), n,
                                            _ptr(flat), _ptr(poff), _ptr(plen), _ptr(ra), _ptr(rb)))
        return [(ra[poff[k]:poff[k + 1]].tobytes(), rb[poff[k]:poff[k + 1]].tobytes()) for k in range(n)]

    def anchored_realign(self, windows):
        """ProfileAlignFast(anchored) for windows of a two-genome alignment
        (MuscleInterface::ProfileAlignFast with anchored = true,
        libMems/MuscleInterface.cpp:1053-1109, calling AnchoredProfileProfile,
        muscle/libMUSCLE/anchoredpp.cpp:429-552): each window is cut at its
        anchor columns (mvg_anchor_columns), every range of every window is
        one problem of a single batched gap-DP call on the GPU, the rows come
        from the paths on the GPU (mvg_path_rows) and each window's ranges are
        concatenated in order.  windows: list of (row A, row B) with '-' gaps
        and bases A/C/G/T in either case.  Returns the realigned (row A,
        row B) bytes of each window."""
        code = np.full(256, 255, np.uint8)
        for i, ch in enumerate(b"ACGT"):
            code[ch] = code[ch | 0x20] = i
        pieces = []  # per window: list of ("dp", problem index) or ("fixed", row A, row B)
        sa, sb, oa, ob = [], [], [0], [0]
        for ra, rb in windows:
            parts = []
            for _, a, b in anchored_problems(ra, rb):
                if len(a) == 0 or len(b) == 0:  # nothing to align: the other side against gaps
                    parts.append(("fixed", b"-" * len(b) if len(a) == 0 else a.tobytes(),
                                  b.tobytes() if len(a) == 0 else b"-" * len(a)))
                    continue
                if (code[a] == 255).any() or (code[b] == 255).any():
                    raise ValueError("the gap DP takes A, C, G and T only")
                parts.append(("dp", len(oa) - 1))
                sa.append(a)
                sb.append(b)
                oa.append(oa[-1] + len(a))
                ob.append(ob[-1] + len(b))
            pieces.append(parts)
        rows = []
        if len(oa) > 1:
            chars_a, chars_b = np.concatenate(sa), np.concatenate(sb)
            _, paths = self.gap_align_batch(code[chars_a], oa, code[chars_b], ob)
            rows = self.path_rows(chars_a, oa, chars_b, ob, paths)
        out = []
        for parts in pieces:
            ra = [rows[p[1]][0] if p[0] == "dp" else p[1] for p in parts]
            rb = [rows[p[1]][1] if p[0] == "dp" else p[2] for p in parts]
            out.append((b"".join(ra), b"".join(rb)))
        return out

    def _gapped(self, lcbs, max_window_size, passes):
        """mvg_gapped_alignment over a list of (row A, row B)."""
        rows = [(_u8(ra), _u8(rb)) for ra, rb in lcbs]
        for ra, rb in rows:
            if len(ra) != len(rb):
                raise ValueError("rows of different length")
        if not rows:
            return []
        ra = np.concatenate([r[0] for r in rows])
        rb = np.concatenate([r[1] for r in rows])
        off = np.zeros(len(rows) + 1, np.uint64)
        off[1:] = np.cumsum([len(r[0]) for r in rows])
        out_off = np.zeros(len(rows) + 1, np.uint64)
        cap = int(len(ra) * 1.25) + 1024
        while True:
            oa, ob = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
            rc = load_library().mvg_gapped_alignment(self._h, _ptr(ra), _ptr(rb), _ptr(off), len(rows),
                                                     float(max_window_size), int(passes), _ptr(oa), _ptr(ob),
                                                     _ptr(out_off), cap)
            if rc == MVG_ERR_CAPACITY and int(out_off[-1]) > cap:
                cap = int(out_off[-1])
                continue
            _check(rc)
            return [(oa[out_off[k]:out_off[k + 1]].tobytes(), ob[out_off[k]:out_off[k + 1]].tobytes())
                    for k in range(len(rows))]

    def refine_alignment(self, lcbs, max_window_size=20000.0):
        """The gapped-alignment pass of refineAlignment for LCBs of two
        genomes (LM/ProgressiveAligner.cpp:1119-1230 with profile_aln, as
        doGappedAlignment calls it at step 8 of alignProfileToProfile;
        mvg_gapped_alignment, pass 1): each LCB cut into windows
        (mvg_refine_windows), every window that is not a gap window and holds
        bases of both genomes realigned as ProfileAlignFast(anchored) does
        (all windows of all LCBs in one gap-DP call), and each LCB's windows
        concatenated.  lcbs: list of (row A, row B).  Returns the new
        (row A, row B) bytes of each LCB."""
        return self._gapped(lcbs, max_window_size, 1)

    def iterative_refine(self, lcbs, max_window_size=20000.0):
        """The final iterative-refinement pass for LCBs of two genomes
        (refineAlignment with profile_aln = false,
        LM/ProgressiveAligner.cpp:1119-1230, as alignProfileToProfile ends
        with it, :3750-3755; mvg_gapped_alignment, pass 2): RefineFast's
        column windows (refine_fast_ranges) of every LCB realigned from their
        bases in one gap-DP call, the other columns kept.  lcbs: list of
        (row A, row B).  Returns the new (row A, row B) bytes of each LCB."""
        return self._gapped(lcbs, max_window_size, 2)

    def gapped_alignment(self, lcbs, max_window_size=20000.0, refine=True):
        """Both passes a two-genome progressiveMauve run makes over its LCBs
        in one call (mvg_gapped_alignment): the gapped-alignment pass and,
        unless refine is False, the final iterative refinement on its
        output."""
        return self._gapped(lcbs, max_window_size, 3 if refine else 1)

    def xmfa_write(self, file_a, file_b, starts, lengths, rows_a, rows_b, col_off, backbone_file=""):
        """WriteStandardAlignment for pairwise blocks; returns the XMFA text (bytes)."""
        starts = np.ascontiguousarray(starts, np.int64).reshape(-1)
        lengths = np.ascontiguousarray(lengths, np.int64).reshape(-1)
        col_off = np.ascontiguousarray(col_off, np.uint64)
        ra, rb = _u8(rows_a), _u8(rows_b)
        n = len(col_off) - 1
        cnt = ctypes.c_uint64(0)
        L = load_library()
        args = (self._h, file_a.encode(), file_b.encode(), backbone_file.encode(), n, _ptr(starts), _ptr(lengths),
                _ptr(ra) if len(ra) else None, _ptr(rb) if len(rb) else None, _ptr(col_off))
        rc = L.mvg_xmfa_write(*args, None, 0, ctypes.byref(cnt))
        if rc not in (MVG_OK, MVG_ERR_CAPACITY):
            _check(rc)
        out = ctypes.create_string_buffer(max(int(cnt.value), 1))
        _check(L.mvg_xmfa_write(*args, out, int(cnt.value), ctypes.byref(cnt)))
        return out.raw[:cnt.value]

    def xmfa_write_dev(self, file_a, file_b, starts, lengths, d_rows_a, d_rows_b, col_off, out_ptr=None, cap=0,
                       backbone_file=""):
        """The writer with the rows in device memory (raw pointers), the text
        written into the caller's host buffer out_ptr of cap bytes.  Returns
        the text length; with no buffer (cap 0) only the length needed."""
        starts = np.ascontiguousarray(starts, np.int64).reshape(-1)
        lengths = np.ascontiguousarray(lengths, np.int64).reshape(-1)
        col_off = np.ascontiguousarray(col_off, np.uint64)
        cnt = ctypes.c_uint64(0)
        wait_producers()
        rc = load_library().mvg_xmfa_write_dev(self._h, file_a.encode(), file_b.encode(), backbone_file.encode(),
                                               len(col_off) - 1, _ptr(starts), _ptr(lengths), d_rows_a, d_rows_b,
                                               _ptr(col_off), out_ptr, cap, ctypes.byref(cnt))
        if not (rc == MVG_ERR_CAPACITY and not cap):
            _check(rc)
        return int(cnt.value)

    def gap_align_batch_raw(self, seq_a, off_a, seq_b, off_b, scores, paths, path_off, path_len):
        """Host-buffer call with caller-owned numpy outputs (no per-call Python decoding)."""
        n = len(off_a) - 1
        _check(load_library().mvg_gapdp_batch(self._h, _ptr(seq_a), _ptr(off_a), _ptr(seq_b), _ptr(off_b), n,
                                              _ptr(scores), _ptr(paths), _ptr(path_off), _ptr(path_len)))

    def gap_align_batch_dev(self, d_sa, d_oa, d_sb, d_ob, n, d_scores, d_paths, d_path_off, d_path_len):
        wait_producers()
        _check(load_library().mvg_gapdp_batch_dev(self._h, d_sa, d_oa, d_sb, d_ob, n, d_scores, d_paths, d_path_off,
                                                  d_path_len))

    def set_profiling(self, on=True):
        _check(load_library().mvg_set_profiling(self._h, 1 if on else 0))

    def stage_times(self):
        """{stage name: total ms} of the last call (profiling must be on)."""
        names = ctypes.create_string_buffer(4096)
        ms = np.zeros(64, np.float64)
        n = ctypes.c_int(0)
        _check(load_library().mvg_stage_times(self._h, names, 4096, _ptr(ms), 64, ctypes.byref(n)))
        out = {}
        for name, t in zip(names.value.decode().split(",") if n.value else [], ms[:n.value]):
            out[name] = out.get(name, 0.0) + float(t)
        return out

    def probe_int32_peak(self):
        v = ctypes.c_double(0)
        _check(load_library().mvg_probe_int32_peak(self._h, ctypes.byref(v)))
        return float(v.value)
