"""Seeded synthetic genome pairs and gap-alignment batches.

The reference publishes no benchmark data; these generators produce inputs
with the sizes and mutation spectra of the five workloads the build is
measured on (numpy default_rng, fixed seeds, so every run sees the same
bytes).  Sequences are ASCII uint8 arrays ('A','C','G','T'); DP batches are
base codes 0..3.
"""
import numpy as np

ACGT = np.frombuffer(b"ACGT", np.uint8)
_COMP = np.zeros(256, np.uint8)
for _x, _y in zip(b"ACGT", b"TGCA"):
    _COMP[_x] = _y


def random_bases(rng, n, gc=0.5):
    p = [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]
    return ACGT[rng.choice(4, size=n, p=p)].astype(np.uint8)


def revcomp(s):
    return _COMP[s[::-1]]


def _substitute(rng, s, mask):
    """Replace the masked bases with a different base (uniform over the other three)."""
    idx = np.nonzero(mask)[0]
    if len(idx) == 0:
        return s
    code = np.searchsorted(ACGT, s[idx])
    code = np.where(code > 3, 0, code)
    s = s.copy()
    s[idx] = ACGT[(code + rng.integers(1, 4, len(idx))) % 4]
    return s


def _indels(rng, s, nindel, mean_len):
    if nindel <= 0:
        return s
    pos = np.sort(rng.integers(0, len(s), nindel))
    lens = rng.geometric(1.0 / mean_len, nindel)
    ins = rng.random(nindel) < 0.5
    parts, prev = [], 0
    for p, l, i in zip(pos, lens, ins):
        if p < prev:
            continue
        parts.append(s[prev:p])
        if i:
            parts.append(random_bases(rng, int(l)))
            prev = p
        else:
            prev = min(len(s), p + int(l))
    parts.append(s[prev:])
    return np.concatenate(parts)


def _rearrange(rng, s, n, len_range):
    """n inversions or translocations of segments with lengths in len_range."""
    s = s.copy()
    for _ in range(n):
        l = int(rng.integers(len_range[0], len_range[1] + 1))
        if l >= len(s) // 2:
            continue
        p = int(rng.integers(0, len(s) - l))
        if rng.random() < 0.5:
            s[p:p + l] = revcomp(s[p:p + l])
        else:
            seg = s[p:p + l].copy()
            rest = np.concatenate([s[:p], s[p + l:]])
            q = int(rng.integers(0, len(rest)))
            s = np.concatenate([rest[:q], seg, rest[q:]])
    return s


def mutate(rng, b, sub, nindel, mean_len, nrearr, rearr_len):
    a = _substitute(rng, b, rng.random(len(b)) < sub)
    a = _indels(rng, a, nindel, mean_len)
    return _rearrange(rng, a, nrearr, rearr_len)


def insert_repeats(rng, b, family_len, copies, families=1):
    fams = [random_bases(rng, family_len) for _ in range(families)]
    pos = np.sort(rng.integers(0, len(b), copies))
    parts, prev = [], 0
    for k, p in enumerate(pos):
        parts.append(b[prev:p])
        parts.append(fams[k % families])
        prev = p
    parts.append(b[prev:])
    return np.concatenate(parts)


def mutate_codes(rng, a, sub, nindel, mean_len):
    """Mutate a base-code (0..3) sequence; never returns an empty sequence."""
    s = ACGT[a]
    s = _indels(rng, _substitute(rng, s, rng.random(len(s)) < sub), nindel, mean_len)
    if len(s) == 0:
        s = ACGT[rng.integers(0, 4, 1)]
    return np.searchsorted(ACGT, s).astype(np.uint8)


# ---------------------------------------------------------------- workloads

def genome_pair_small(seed=0, n=1_000_000):
    """Plain-method pair: B i.i.d. at GC 0.50; A = B + 0.5% substitutions,
    50 indels (geometric mean 5, half insertions) and 2 inversions of 10 kbp."""
    rng = np.random.default_rng(seed)
    b = random_bases(rng, n, 0.50)
    a = _substitute(rng, b, rng.random(n) < 0.005)
    a = _indels(rng, a, 50, 5.0)
    for _ in range(2):
        p = int(rng.integers(0, len(a) - 10_000))
        a[p:p + 10_000] = revcomp(a[p:p + 10_000])
    return a, b


def genome_pair_recoded(seed=1, n=4_600_000):
    """Recoded-genome stand-in: B at GC 0.508 with 40 copies of one 1.3 kbp
    repeat and 4,300 non-overlapping ORFs (mean 950 bp, multiple of 3);
    A = B with 3% of ORF codon third positions substituted, 0.05% elsewhere,
    200 indels (geometric mean 4) and 5 rearrangements of 5-50 kbp."""
    rng = np.random.default_rng(seed)
    core = random_bases(rng, n - 40 * 1300, 0.508)
    b = insert_repeats(rng, core, 1300, 40)
    norf = int(4300 * len(b) / 4_600_000)
    lens = (np.maximum(rng.normal(950, 250, norf), 90) // 3 * 3).astype(np.int64)
    total = int(lens.sum())
    if total > 0.95 * len(b):
        lens = (lens * (0.95 * len(b) / total) // 3 * 3).astype(np.int64)
        total = int(lens.sum())
    gaps = rng.multinomial(len(b) - total, np.ones(norf + 1) / (norf + 1))
    in_orf3 = np.zeros(len(b), bool)
    p = 0
    for g, l in zip(gaps[:-1], lens):
        p += int(g)
        in_orf3[p + 2:p + l:3] = True
        p += int(l)
    in_orf = np.zeros(len(b), bool)
    u = rng.random(len(b))
    mask = np.where(in_orf3, u < 0.03, u < 0.0005)
    del in_orf
    a = _substitute(rng, b, mask)
    a = _indels(rng, a, 200, 4.0)
    a = _rearrange(rng, a, 5, (5_000, 50_000))
    return a, b


def genome_pair_large(seed=5, n=12_000_000, ncontig=16):
    """Large pair: B = 12 Mbp in 16 contigs (0.2-1.5 Mbp) at GC 0.38 with
    300 copies of 5 repeat families (0.3-6 kbp); A = B with 8%
    substitutions, 2,000 indels (mean 6) and 1,000 rearrangements of
    1-100 kbp.  Contigs are concatenated (the seed path sees one sequence)."""
    rng = np.random.default_rng(seed)
    fam_lens = rng.integers(300, 6001, 5)
    rep_total = int(sum(fam_lens[k % 5] for k in range(300)))
    core = random_bases(rng, n - rep_total, 0.38)
    fams = [random_bases(rng, int(l), 0.38) for l in fam_lens]
    pos = np.sort(rng.integers(0, len(core), 300))
    parts, prev = [], 0
    for k, p in enumerate(pos):
        parts.append(core[prev:p])
        parts.append(fams[k % 5])
        prev = p
    parts.append(core[prev:])
    b = np.concatenate(parts)
    a = _substitute(rng, b, rng.random(len(b)) < 0.08)
    a = _indels(rng, a, 2000, 6.0)
    a = _rearrange(rng, a, 1000, (1_000, 100_000))
    return a, b


def gap_batch(seed=3, nprob=200_000, lmin=10, lmax=20_000, max_div=0.30):
    """Independent DP problems: lengths log-uniform on [lmin, lmax], the
    second sequence derived from the first at divergence U(0, max_div)
    (substitutions:indels 9:1, indel length geometric mean 3).
    Returns concatenated base codes and offsets (nprob+1)."""
    rng = np.random.default_rng(seed)
    la = np.exp(rng.uniform(np.log(lmin), np.log(lmax), nprob)).astype(np.int64)
    div = rng.uniform(0, max_div, nprob)
    seq_a = rng.integers(0, 4, int(la.sum())).astype(np.uint8)
    off_a = np.zeros(nprob + 1, np.int64)
    off_a[1:] = np.cumsum(la)
    pieces = []
    for k in range(nprob):
        a = seq_a[off_a[k]:off_a[k + 1]]
        sub = 0.9 * div[k]
        nind = rng.poisson(0.1 * div[k] * len(a) / 3.0)
        pieces.append(_mutate_codes_fast(rng, a, sub, nind))
    seq_b = np.concatenate(pieces)
    off_b = np.zeros(nprob + 1, np.int64)
    off_b[1:] = np.cumsum([len(x) for x in pieces])
    return seq_a, off_a, seq_b, off_b


def gap_batch_recoded(seed=4, nprob=1_000_000, lmin=20, lmax=5000, unrelated=0.1):
    """Inter-anchor gaps drawn like the recoded-genome pair's: lengths
    log-uniform on [lmin, lmax]; 90% homologous with substitutions U(0.5%, 3%)
    and Poisson(0.0005 L) indels (geometric mean 4); 10% divergent gap
    content (divergence U(25%, 40%), indel share 10%).  Vectorised over the
    whole batch.  Returns concatenated base codes and offsets."""
    rng = np.random.default_rng(seed)
    la = np.exp(rng.uniform(np.log(lmin), np.log(lmax), nprob)).astype(np.int64)
    off_a = np.zeros(nprob + 1, np.int64)
    off_a[1:] = np.cumsum(la)
    total = int(off_a[-1])
    seq_a = rng.integers(0, 4, total).astype(np.uint8)
    far = rng.random(nprob) < unrelated
    sub = np.where(far, rng.uniform(0.25, 0.40, nprob) * 0.9, rng.uniform(0.005, 0.03, nprob))
    ind_rate = np.where(far, rng.uniform(0.25, 0.40, nprob) * 0.1 / 3.0, 0.0005)
    gid = np.repeat(np.arange(nprob), la)
    b = seq_a.copy()
    m = rng.random(total) < sub[gid]
    b[m] = (b[m] + rng.integers(1, 4, int(m.sum()))) % 4
    nind = rng.poisson(ind_rate * la)
    eg = np.repeat(np.arange(nprob), nind)  # gap of each indel event
    pos = off_a[eg] + (rng.random(len(eg)) * la[eg]).astype(np.int64)
    lens = rng.geometric(0.25, len(eg))
    ins = rng.random(len(eg)) < 0.5
    order = np.argsort(pos, kind="stable")
    pos, lens, ins, eg = pos[order], lens[order], ins[order], eg[order]
    keep = np.ones(total, bool)
    add_at, add_len = [], []
    delta_len = np.zeros(nprob, np.int64)
    for p, l, i, g in zip(pos, lens, ins, eg):
        if i:
            add_at.append(p)
            add_len.append(int(l))
            delta_len[g] += l
        else:
            e = min(p + int(l), int(off_a[g + 1]))
            delta_len[g] -= int(keep[p:e].sum())
            keep[p:e] = False
    lb = la + delta_len
    empty = lb <= 0
    if empty.any():  # never return an empty sequence: keep the gap's first base
        for g in np.nonzero(empty)[0]:
            keep[off_a[g]] = True
            delta_len[g] += 1
        lb = la + delta_len
    pieces, prev = [], 0
    inserts = sorted(zip(add_at, add_len))
    for p, l in inserts:
        pieces.append(b[prev:p][keep[prev:p]])
        pieces.append(rng.integers(0, 4, l).astype(np.uint8))
        prev = p
    pieces.append(b[prev:][keep[prev:]])
    seq_b = np.concatenate(pieces)
    off_b = np.zeros(nprob + 1, np.int64)
    off_b[1:] = np.cumsum(lb)
    assert off_b[-1] == len(seq_b)
    return seq_a, off_a, seq_b, off_b


def _mutate_codes_fast(rng, a, sub, nind):
    m = rng.random(len(a)) < sub
    b = a.copy()
    b[m] = (b[m] + rng.integers(1, 4, int(m.sum()))) % 4
    if nind:
        pos = np.sort(rng.integers(0, len(b), nind))
        lens = rng.geometric(1 / 3.0, nind)
        ins = rng.random(nind) < 0.5
        parts, prev = [], 0
        for p, l, i in zip(pos, lens, ins):
            if p < prev:
                continue
            parts.append(b[prev:p])
            if i:
                parts.append(rng.integers(0, 4, int(l)).astype(np.uint8))
                prev = p
            else:
                prev = min(len(b), p + int(l))
        parts.append(b[prev:])
        b = np.concatenate(parts)
    if len(b) == 0:
        b = rng.integers(0, 4, 1).astype(np.uint8)
    return b


# ---------------------------------------------------------------- index LUT


def lut_alignment(seed, n_ref=20000, sub=0.01, indel=0.002, nblocks=8, shuffle=True, extras=True):
    """A pairwise alignment of a genome against a reference, cut into XMFA-
    like sub-alignment groups.  Returns (groups, genome, ref): each group is
    a list of (seq_num, start_idx, row) with seq_num 1 = genome, 2 =
    reference and start_idx the 1-based position of the row's first base.
    Columns come from a walk over the reference with substitutions, indels
    (geometric lengths), occasional N and lowercase bases; extras adds a
    genome-only group, a repeated (overwriting) block, a column gapped on
    both sides, and a block whose genome row is all gaps with start 0."""
    rng = np.random.default_rng(seed)
    ref = rng.choice(np.frombuffer(b"ACGT", np.uint8), n_ref)
    if extras:
        ref[rng.random(n_ref) < 0.001] = ord("N")
    cols_g, cols_r = [], []
    i = 0
    while i < n_ref:
        u = rng.random()
        if u < indel / 2:
            k = int(rng.geometric(0.3))
            for _ in range(k):
                cols_g.append(int(rng.choice(np.frombuffer(b"ACGT", np.uint8))))
                cols_r.append(ord("-"))
        elif u < indel:
            k = min(int(rng.geometric(0.3)), n_ref - i)
            for _ in range(k):
                cols_g.append(ord("-"))
                cols_r.append(int(ref[i]))
                i += 1
        else:
            b = int(ref[i])
            if rng.random() < sub:
                b = int(rng.choice([c for c in b"ACGT" if c != b]))
            if extras and rng.random() < 0.0005:
                b = b | 0x20 if 65 <= b <= 90 else b  # lowercase: compares unequal
            cols_g.append(b)
            cols_r.append(int(ref[i]))
            i += 1
    G = np.array(cols_g, np.uint8)
    R = np.array(cols_r, np.uint8)
    gpos = np.cumsum(G != ord("-"))  # 1-based genome position after each column
    rpos = np.cumsum(R != ord("-"))
    genome = G[G != ord("-")].tobytes()
    cuts = np.sort(rng.choice(np.arange(1, len(G)), nblocks - 1, replace=False)) if nblocks > 1 else []
    bounds = [0, *cuts.tolist(), len(G)] if nblocks > 1 else [0, len(G)]
    groups = []
    for a, e in zip(bounds[:-1], bounds[1:]):
        g0 = int(gpos[a - 1]) + 1 if a > 0 else 1
        r0 = int(rpos[a - 1]) + 1 if a > 0 else 1
        groups.append([(1, g0, G[a:e].tobytes()), (2, r0, R[a:e].tobytes())])
    if shuffle:
        order = rng.permutation(len(groups))
        groups = [groups[k] for k in order]
    if extras:
        groups.insert(int(rng.integers(0, len(groups) + 1)), [(1, 5, genome[4:200])])
        k = int(rng.integers(0, len(groups)))
        if len(groups[k]) == 2:
            (s1, g0, rg), (s2, r0, rr) = groups[k]
            # a copy shifted by one reference base, later in the list: it
            # overwrites the first copy's entries
            groups.append([(1, g0, rg), (2, r0 + 1, rr)])
            # a column gapped on both sides inside the block
            m = len(rg) // 2
            groups[k] = [(1, g0, rg[:m] + b"-" + rg[m:]), (2, r0, rr[:m] + b"-" + rr[m:])]
        groups.append([(1, 0, b"---"), (2, 7, b"A-C")])
    return groups, genome, ref.tobytes()


def lut_random(seed, n=5000, run_mean=60, p_gap=0.3, p_noise=0.05, p_island=0.2):
    """A LUT made of consecutive runs separated by -1 gaps, shifted runs,
    noisy single entries and mapped islands inside gaps (starts that a
    neighbouring fill covers)."""
    rng = np.random.default_rng(seed)
    lut = np.empty(n, np.int32)
    i, v = 0, int(rng.integers(0, 1000))
    while i < n:
        L = min(int(rng.geometric(1.0 / run_mean)), n - i)
        lut[i:i + L] = v + np.arange(L)
        i += L
        v += L
        r = rng.random()
        if r < p_gap:
            g = min(int(rng.geometric(1.0 / 12)), n - i)
            lut[i:i + g] = -1
            if g > 4 and rng.random() < p_island:
                k = int(rng.integers(1, g - 1))
                lut[i + k] = int(rng.integers(0, v + 100))
            i += g
            v += g + int(rng.integers(-3, 4)) * (rng.random() < 0.5)
        elif r < p_gap + 0.2:
            v += int(rng.integers(-50, 50))
        v = max(v, 0)
    noise = rng.random(n) < p_noise
    lut[noise] = rng.integers(-1, max(2, int(lut.max()) + 10), int(noise.sum()))
    return lut


def lut_alignment_fast(seed, n_ref=4_600_000, sub=0.01, indel=0.0005, nblocks=64, shuffle=True):
    """Vectorised lut_alignment without the extras, for genome-sized cases:
    returns (gs, rs, col_off, genome_rows, ref_rows, genome, ref) with the
    blocks already flattened (every block has both sequences)."""
    rng = np.random.default_rng(seed)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    R = rng.choice(acgt, n_ref)
    Gc = R.copy()
    m = rng.random(n_ref) < sub
    Gc[m] = acgt[(np.searchsorted(acgt, Gc[m]) + rng.integers(1, 4, int(m.sum()))) % 4]
    nev = rng.poisson(indel * n_ref)
    pos = rng.integers(0, n_ref, nev)
    lens = rng.geometric(0.3, nev)
    ins = rng.random(nev) < 0.5
    dele = np.zeros(n_ref + 1, np.int32)
    np.add.at(dele, pos[~ins], 1)
    np.add.at(dele, np.minimum(pos[~ins] + lens[~ins], n_ref), -1)
    Gc[np.cumsum(dele[:-1]) > 0] = ord("-")
    at = np.repeat(pos[ins], lens[ins])
    G = np.insert(Gc, at, rng.choice(acgt, len(at)))
    Rr = np.insert(R, at, np.full(len(at), ord("-"), np.uint8))
    gpos = np.cumsum(G != ord("-"))
    rpos = np.cumsum(Rr != ord("-"))
    genome = G[G != ord("-")]
    cuts = np.sort(rng.choice(np.arange(1, len(G)), nblocks - 1, replace=False))
    bounds = np.concatenate([[0], cuts, [len(G)]])
    order = rng.permutation(nblocks) if shuffle else np.arange(nblocks)
    gs, rs, rows_g, rows_r = [], [], [], []
    for b in order:
        a, e = int(bounds[b]), int(bounds[b + 1])
        gs.append(int(gpos[a - 1]) + 1 if a > 0 else 1)
        rs.append(int(rpos[a - 1]) + 1 if a > 0 else 1)
        rows_g.append(G[a:e])
        rows_r.append(Rr[a:e])
    off = np.zeros(nblocks + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in rows_g])
    return (np.array(gs, np.int64), np.array(rs, np.int64), off, np.concatenate(rows_g), np.concatenate(rows_r),
            genome, R)


def xmfa_text(groups, width=80, crlf=False, seed=0):
    """XMFA text of sub-alignment groups [(seq_num, start, row bytes)]:
    '#' header lines, one '>' header per sub-alignment with an end
    coordinate, strand and file name, rows wrapped at `width`, and an '='
    line (with a score note on some) closing each group."""
    rng = np.random.default_rng(seed)
    nl = "\r\n" if crlf else "\n"
    out = ["#FormatVersion Mauve1", "#Sequence1File\tgenome.fa", "#Sequence2File\tref.fa"]
    for grp in groups:
        for s, st, row in grp:
            n = sum(1 for c in row if c != ord("-"))
            end = st + n - 1 if n else 0
            strand = "+" if rng.random() < 0.8 else "-"
            out.append("> %d:%d-%d %s %s" % (s, st, end, strand, "genome.fa" if s == 1 else "ref.fa"))
            txt = row.decode("latin-1")
            out.extend(txt[k:k + width] for k in range(0, len(txt), width))
        out.append("=" if rng.random() < 0.5 else "= score=%d" % int(rng.integers(0, 10 ** 6)))
    return (nl.join(out) + nl).encode("latin-1")
