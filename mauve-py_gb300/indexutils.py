"""GPU index LUT: the functions of mauve/indexutils.pyx and the LUT part of
mauve/buildindex.py, on libmauve_gb300.

Same names, arguments and in-place behaviour as the reference module:

  fixZeroIdx(idx_lut, genome, ref_genome)        indexutils.pyx:27-44
  fillGaps(idx_lut, max_gap_width=300)           indexutils.pyx:47-75
  smoothEdges(idx_lut, smoothing_radius=20)      indexutils.pyx:78-108
  findGaps(idx_lut) -> int32 array               indexutils.pyx:111-139
  findEdges(idx_lut) -> bool mask                indexutils.pyx:142-156
  findMismatches(idx_lut, genome, ref) -> mask   indexutils.pyx:159-175
  findDuplicateMappings(idx_lut) -> int          indexutils.pyx:178-186
  lookupSubAlignment(seq_num, group)             indexutils.pyx:17-24
  buildIndexFromGroups(groups, genome_length, …) buildindex.py:111-138

idx_lut is a contiguous 1-D int32 numpy array (updated in place through
the host C ABI) or a CUDA int32 torch tensor (updated in place on the
device, no host copies).  findEdges / findMismatches return the per-index
0/1 mask that the reference packs into a bitarray.  Errors raise what the
reference raises: IndexError where the Cython code's bounds checks fire,
OverflowError for a value outside int32.  Every call runs on the GPU.
"""
import ctypes

import numpy as np

import mvg

IDX_ARRAY_DTYPE = np.int32
MASK_ARRAY_DTYPE = np.uint8

_default_ctx = None


def _ctx(ctx):
    global _default_ctx
    if ctx is not None:
        return ctx
    if _default_ctx is None:
        _default_ctx = mvg.Context(0)
    return _default_ctx


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _lut_host(lut):
    if not (isinstance(lut, np.ndarray) and lut.dtype == np.int32 and lut.ndim == 1 and lut.flags.c_contiguous):
        raise TypeError("idx_lut must be a contiguous 1-D int32 array")
    return lut


def _lut_dev(lut):
    import torch
    if lut.dtype != torch.int32 or lut.dim() != 1 or not lut.is_contiguous() or not lut.is_cuda:
        raise TypeError("idx_lut must be a contiguous 1-D CUDA int32 tensor")
    return lut


def _seq_dev(seq, dev):
    import torch
    if _is_torch(seq):
        return seq.contiguous().to(dev, torch.uint8)
    return torch.from_numpy(mvg._u8(seq).copy()).to(dev)


def lookupSubAlignment(seq_num, sub_alignment_group):
    """The group's sub-alignment of sequence seq_num, or None."""
    for a in sub_alignment_group.alignments:
        if a.seq_num == seq_num:
            return a
    return None


def fixZeroIdx(idx_lut, genome, ref_genome, ctx=None):
    c = _ctx(ctx)
    L = mvg.load_library()
    if _is_torch(idx_lut):
        lut = _lut_dev(idx_lut)
        g, r = _seq_dev(genome, lut.device), _seq_dev(ref_genome, lut.device)
        mvg.wait_producers()
        mvg._check(L.mvg_lut_fix_zero_idx_dev(c.handle, lut.data_ptr(), lut.numel(), g.data_ptr(), g.numel(),
                                              r.data_ptr(), r.numel()))
        return
    lut = _lut_host(idx_lut)
    g, r = mvg._u8(genome), mvg._u8(ref_genome)
    mvg._check(L.mvg_lut_fix_zero_idx(c.handle, mvg._ptr(lut), len(lut), mvg._ptr(g), len(g), mvg._ptr(r), len(r)))


def _fill(fn_host, fn_dev, idx_lut, width, ctx):
    c = _ctx(ctx)
    L = mvg.load_library()
    if _is_torch(idx_lut):
        lut = _lut_dev(idx_lut)
        mvg.wait_producers()
        mvg._check(getattr(L, fn_dev)(c.handle, lut.data_ptr(), lut.numel(), int(width)))
        return
    lut = _lut_host(idx_lut)
    mvg._check(getattr(L, fn_host)(c.handle, mvg._ptr(lut), len(lut), int(width)))


def fillGaps(idx_lut, max_gap_width=300, ctx=None):
    _fill("mvg_lut_fill_gaps", "mvg_lut_fill_gaps_dev", idx_lut, max_gap_width, ctx)


def smoothEdges(idx_lut, smoothing_radius=20, ctx=None):
    _fill("mvg_lut_smooth_edges", "mvg_lut_smooth_edges_dev", idx_lut, smoothing_radius, ctx)


def findGaps(idx_lut, ctx=None):
    c = _ctx(ctx)
    L = mvg.load_library()
    if _is_torch(idx_lut):
        import torch
        lut = _lut_dev(idx_lut)
        gaps = torch.zeros(lut.numel(), dtype=torch.int32, device=lut.device)
        mvg.wait_producers()
        mvg._check(L.mvg_lut_find_gaps_dev(c.handle, lut.data_ptr(), lut.numel(), gaps.data_ptr()))
        return gaps
    lut = _lut_host(idx_lut)
    gaps = np.zeros(len(lut), np.int32)
    mvg._check(L.mvg_lut_find_gaps(c.handle, mvg._ptr(lut), len(lut), mvg._ptr(gaps)))
    return gaps


def findEdges(idx_lut, ctx=None):
    c = _ctx(ctx)
    lut = _lut_host(np.ascontiguousarray(idx_lut.cpu().numpy() if _is_torch(idx_lut) else idx_lut))
    out = np.zeros(len(lut), np.uint8)
    mvg._check(mvg.load_library().mvg_lut_find_edges(c.handle, mvg._ptr(lut), len(lut), mvg._ptr(out)))
    return out.astype(bool)


def findMismatches(idx_lut, genome, ref_genome, ctx=None):
    c = _ctx(ctx)
    lut = _lut_host(np.ascontiguousarray(idx_lut.cpu().numpy() if _is_torch(idx_lut) else idx_lut))
    g, r = mvg._u8(genome), mvg._u8(ref_genome)
    out = np.zeros(len(lut), np.uint8)
    mvg._check(mvg.load_library().mvg_lut_find_mismatches(c.handle, mvg._ptr(lut), len(lut), mvg._ptr(g), len(g),
                                                          mvg._ptr(r), len(r), mvg._ptr(out)))
    return out.astype(bool)


def findDuplicateMappings(idx_lut, ctx=None):
    c = _ctx(ctx)
    lut = _lut_host(np.ascontiguousarray(idx_lut.cpu().numpy() if _is_torch(idx_lut) else idx_lut))
    res = ctypes.c_int64()
    mvg._check(mvg.load_library().mvg_lut_find_duplicate_mappings(c.handle, mvg._ptr(lut), len(lut),
                                                                  ctypes.byref(res)))
    return int(res.value)


class Blocks:
    """Aligned blocks flattened for the C ABI: block b is columns
    [col_off[b], col_off[b+1]) of genome_rows / ref_rows."""

    def __init__(self, genome_start, ref_start, col_off, genome_rows, ref_rows):
        self.genome_start = np.ascontiguousarray(genome_start, np.int64)
        self.ref_start = np.ascontiguousarray(ref_start, np.int64)
        self.col_off = np.ascontiguousarray(col_off, np.uint64)
        self.genome_rows = np.ascontiguousarray(genome_rows, np.uint8)
        self.ref_rows = np.ascontiguousarray(ref_rows, np.uint8)
        if len(self.col_off) != len(self.genome_start) + 1 or len(self.ref_start) != len(self.genome_start):
            raise ValueError("block arrays disagree in length")
        if len(self.genome_rows) != len(self.ref_rows):
            raise ValueError("rows differ in length")

    @property
    def n(self):
        return len(self.genome_start)

    @classmethod
    def from_groups(cls, sub_alignment_groups):
        """Blocks of the groups where both sequence 1 (genome) and sequence
        2 (reference) are present, in group order (buildindex.py:116-120)."""
        gs, rs, rows_g, rows_r = [], [], [], []
        for grp in sub_alignment_groups:
            a, b = lookupSubAlignment(1, grp), lookupSubAlignment(2, grp)
            if a is None or b is None:
                continue
            sa, sb = _as_bytes(a.seq), _as_bytes(b.seq)
            # the reference walks the genome row and indexes the reference
            # row by column: extra reference columns are never read, a
            # shorter reference row raises IndexError
            if len(sb) < len(sa):
                raise IndexError("reference row shorter than the genome row")
            sb = sb[:len(sa)]
            gs.append(a.start_idx)
            rs.append(b.start_idx)
            rows_g.append(sa)
            rows_r.append(sb)
        off = np.zeros(len(gs) + 1, np.uint64)
        off[1:] = np.cumsum([len(x) for x in rows_g], dtype=np.uint64)
        g = np.frombuffer(b"".join(rows_g), np.uint8) if rows_g else np.zeros(0, np.uint8)
        r = np.frombuffer(b"".join(rows_r), np.uint8) if rows_r else np.zeros(0, np.uint8)
        return cls(gs, rs, off, g, r)

    def ptrs(self):
        return [mvg._ptr(x) for x in (self.genome_start, self.ref_start, self.col_off, self.genome_rows,
                                      self.ref_rows)]


def _as_bytes(seq):
    if isinstance(seq, str):
        return seq.encode("latin-1")
    return bytes(seq)


def lutFromBlocks(blocks, genome_length, ctx=None):
    """The unfilled LUT (buildindex.py:112-130)."""
    c = _ctx(ctx)
    lut = np.empty(int(genome_length), IDX_ARRAY_DTYPE)
    mvg._check(mvg.load_library().mvg_lut_from_blocks(c.handle, *blocks.ptrs(), blocks.n, mvg._ptr(lut), len(lut)))
    return lut


def buildIndexFromGroups(sub_alignment_groups, genome_length, genome_seq=None, ref_genome_seq=None, fill_gaps=True,
                         max_gap_width=300, smooth_edges=True, smoothing_radius=20, ctx=None):
    """buildIndex (buildindex.py:90-138) from already parsed XMFA
    sub-alignment groups: the LUT, then fixZeroIdx + fillGaps and
    smoothEdges as flagged.  Sequences are needed only with fill_gaps."""
    blocks = sub_alignment_groups if isinstance(sub_alignment_groups, Blocks) else \
        Blocks.from_groups(sub_alignment_groups)
    c = _ctx(ctx)
    lut = np.empty(int(genome_length), IDX_ARRAY_DTYPE)
    g = mvg._u8(genome_seq) if genome_seq is not None else np.zeros(0, np.uint8)
    r = mvg._u8(ref_genome_seq) if ref_genome_seq is not None else np.zeros(0, np.uint8)
    if fill_gaps and (genome_seq is None or ref_genome_seq is None):
        raise ValueError("fill_gaps needs genome_seq and ref_genome_seq")
    mvg._check(mvg.load_library().mvg_build_index_lut(
        c.handle, *blocks.ptrs(), blocks.n, mvg._ptr(g), len(g), mvg._ptr(r), len(r), int(bool(fill_gaps)),
        int(max_gap_width), int(bool(smooth_edges)), int(smoothing_radius), mvg._ptr(lut), len(lut)))
    return lut


def buildIndexLutDev(d_genome_start, d_ref_start, d_col_off, d_genome_rows, d_ref_rows, nblocks, d_genome,
                     genome_len, d_ref, ref_len, d_lut, n, fill_gaps=True, max_gap_width=300, smooth_edges=True,
                     smoothing_radius=20, ctx=None):
    """buildIndexFromGroups on device buffers (raw pointers): inputs and the
    n-entry int32 LUT stay in device memory."""
    c = _ctx(ctx)
    mvg.wait_producers()
    mvg._check(mvg.load_library().mvg_build_index_lut_dev(
        c.handle, d_genome_start, d_ref_start, d_col_off, d_genome_rows, d_ref_rows, nblocks, d_genome, genome_len,
        d_ref, ref_len, int(bool(fill_gaps)), int(max_gap_width), int(bool(smooth_edges)), int(smoothing_radius),
        d_lut, n))
