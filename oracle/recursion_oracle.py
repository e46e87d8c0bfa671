"""CPU restatement of the recursive anchor search's gap finding and of the
gapped-alignment pass's windows.

TEST INFRASTRUCTURE ONLY: the checker that tests/ compare the library's
mvg_recursion_gaps and mvg_refine_windows against.  The product package
never imports this module.

Follows ProgressiveAligner::recurseOnPairs (LM/ProgressiveAligner.cpp:682-924)
for one LCB of two genomes, as libMems' Match objects behave
(LM/HybridAbstractMatch.h:151-265: signed starts, Invert negates them;
LM/AbstractMatch.h:209-214: End = Start + Length - 1 for a forward start,
Start itself for a reverse one; LM/UngappedLocalAlignment.h:48-56: Length),
and getInterveningCoordinates (LM/ProgressiveAligner.cpp:566-588) with the
sequence cut of pairwiseAnchorSearch (:598-613); refine_windows follows
refineAlignment's windowing (:1015-1165).  Pinned through the reference's
own recurseOnPairs and refineAlignment (compiled here by
oracle/ref_progressive_driver.cpp; fixtures tests/golden/recursion.npz and
refine.npz): the library equals those fixtures, and equals this restatement
on random LCBs.
"""


class _Match:
    """A two-sequence libMems Match reduced to what recurseOnPairs uses."""

    def __init__(self):
        self.start = [0, 0]  # signed 1-based starts; 0 = NO_MATCH
        self.length = 0

    def set_left_end(self, seq, pos):
        # SetLeftEnd keeps the orientation of a defined start
        o = -1 if self.start[seq] < 0 else 1
        self.start[seq] = abs(pos) * (o if self.start[seq] != 0 else 1)

    def set_orientation(self, seq, reverse):
        self.start[seq] = abs(self.start[seq]) * (-1 if reverse else 1)

    def invert(self):
        self.start = [-s for s in self.start]

    def end(self, seq):
        s = self.start[seq]
        return s + self.length - 1 if s > 0 else s

    def len_of(self, seq):
        return 0 if self.start[seq] == 0 else self.length


def intervening(iv_left, iv_right, r_begin, r_end, seq):
    """getInterveningCoordinates for sequence `seq` of the pair."""
    if (r_end is not None and r_end.start[seq] == 0) or (r_begin is not None and r_begin.start[seq] == 0):
        return 0, 0
    gap_rend = r_end.start[seq] if r_end is not None else iv_right + 1
    gap_lend = r_begin.end(seq) + 1 if r_begin is not None else iv_left
    if gap_rend < 0 or gap_lend < 0:
        gap_rend = -r_begin.start[seq] if r_begin is not None else iv_right + 1
        gap_lend = -r_end.start[seq] + r_end.len_of(seq) if r_end is not None else 1
    return gap_lend, gap_rend


def recursion_gaps(row_a, row_b, left_a, rev_a, left_b, rev_b, glen_a, glen_b, min_gap=200):
    """Gaps (0-based start A, length A, 0-based start B, length B) in search
    order, and the LCB's unaligned flanks per genome [(start, end), ...]
    (1-based, end exclusive)."""
    ncol = len(row_a)
    ra = [bool(c != ord("-")) for c in row_a]
    rb = [bool(c != ord("-")) for c in row_b]
    right_a = left_a + sum(ra) - 1
    right_b = left_b + sum(rb) - 1
    # outer aligned boundaries (:738-782)
    p1l, p1r, p2l, p2r = (0, 0), (0, 0), (0, 0), (0, 0)
    ci = cj = 0
    for col in range(ncol + 1):
        if col == ncol or (ra[col] and rb[col]):
            if col == 0:
                break
            if not rev_a:
                p1l = (left_a, left_a + ci)
            else:
                p1r = (right_a - ci + 1, right_a + 1)
            if not rev_b:
                p2l = (left_b, left_b + cj)
            else:
                p2r = (right_b - cj + 1, right_b + 1)
            break
        if col < ncol and ra[col]:
            ci += 1
        if col < ncol and rb[col]:
            cj += 1
    ci = cj = 0
    for col in range(ncol, 0, -1):
        if ra[col - 1] and rb[col - 1]:
            if col == ncol:
                break
            if not rev_a:
                p1r = (right_a - ci + 1, right_a + 1)
            else:
                p1l = (left_a, left_a + ci)
            if not rev_b:
                p2r = (right_b - cj + 1, right_b + 1)
            else:
                p2l = (left_b, left_b + cj)
            break
        if ra[col - 1]:
            ci += 1
        if rb[col - 1]:
            cj += 1
    flanks = []
    for pl, pr in ((p1l, p1r), (p2l, p2r)):  # (:784-834)
        reg = []
        if pl[0] < pl[1]:
            reg.append([pl[0], pl[1]])
        if pr[0] < pr[1]:
            if pl[0] < pl[1] and pr[0] == pl[1]:
                reg[-1][1] = pr[1]
            else:
                reg.append([pr[0], pr[1]])
        flanks.append([tuple(x) for x in reg])
    # inter-anchor gaps (:836-921)
    gaps = []
    ci = cj = pi = pj = 0
    in_gap = False
    for col in range(ncol + 1):
        if col == ncol or (ra[col] and rb[col]):
            if in_gap and ci - pi > min_gap and cj - pj > min_gap:
                lm = _Match()
                if not rev_a:
                    lm.set_left_end(0, left_a + pi)
                else:
                    lm.set_left_end(0, right_a - pi)
                    lm.set_orientation(0, True)
                if not rev_b:
                    lm.set_left_end(1, left_b + pj)
                else:
                    lm.set_left_end(1, right_b - pj)
                    lm.set_orientation(1, True)
                rm = None
                if cj != right_b and ci != right_a:
                    rm = _Match()
                    if not rev_a:
                        rm.set_left_end(0, left_a + ci)
                    else:
                        rm.set_left_end(0, right_a - ci)
                        rm.set_orientation(0, True)
                    if not rev_b:
                        rm.set_left_end(1, left_b + cj)
                    else:
                        rm.set_left_end(1, right_b - cj)
                        rm.set_orientation(1, True)
                if rev_a:
                    lm, rm = rm, lm
                    if lm is not None:
                        lm.invert()
                    if rm is not None:
                        rm.invert()
                row = []
                for seq, (lft, rgt, glen) in enumerate(((left_a, right_a, glen_a), (left_b, right_b, glen_b))):
                    g0, g1 = intervening(lft, rgt, lm, rm, seq)
                    diff = g1 - g0
                    diff = diff - 1 if diff > 0 else 0
                    if not (diff > 0 and g0 + diff - 1 <= glen):
                        diff = 0
                    row += [g0 - 1 if diff > 0 else 0, diff]
                gaps.append(tuple(row))
            pi, pj = ci, cj
            in_gap = False
        else:
            in_gap = True
        if col < ncol:
            if ra[col]:
                ci += 1
            if rb[col]:
                cj += 1
    return gaps, flanks


def refine_windows(row_a, row_b, max_window_size=20000.0):
    """refineAlignment's windows of one LCB of two genomes
    (LM/ProgressiveAligner.cpp:1119-1165): removeLargeGapsPP (:1051-1117,
    max_gap_length 5000, lcb_hangover 300) then halving by IsDenseEnough
    (:1015-1038, window sizes 200 .. max_window_size, densities .5 .. .9).
    Returns [(first column, end column, gap window)]."""
    ra = [bool(c != ord("-")) for c in row_a]
    rb = [bool(c != ord("-")) for c in row_b]
    ncol = len(ra)
    wins = []
    gap_cols, last, base = 0, None, 0
    for c in range(ncol):
        if ra[c] and rb[c]:
            if gap_cols > 5000:
                if last is not None:
                    k = last + 300 - base
                    wins.append([base, base + k, False])
                    base += k
                k = c - 300 - base
                wins.append([base, base + k, True])
                base += k
            last = c
            gap_cols = 0
        else:
            gap_cols += 1
    if gap_cols > 5000:
        if last is not None:
            k = last + 300 - base
            wins.append([base, base + k, False])
            base += k
        wins.append([base, ncol, True])
    else:
        wins.append([base, ncol, False])

    def dclass(w):
        n = w[1] - w[0]
        na, nb = int(sum(ra[w[0]:w[1]])), int(sum(rb[w[0]:w[1]]))
        total = float(na + nb)
        mult = int(na > 0) + int(nb > 0)
        den = n * float(mult)
        density = total / den if den else float("nan")
        thr = ((0.9 - 0.5) / (200.0 - max_window_size)) * (n - max_window_size) + 0.5
        if density > 0.9:
            return 2
        if density > thr:
            return 1
        return 0

    i = 0
    while i < len(wins):
        w = wins[i]
        n = w[1] - w[0]
        d = dclass(w)
        if (d == 0 and n > max_window_size / 3) or (d == 1 and n > max_window_size) or \
                (d == 2 and n > max_window_size * 3):
            half = n // 2
            right = [w[1] - half, w[1], w[2]]
            w[1] -= half
            wins.insert(i + 1, right)
            continue
        i += 1
    return [tuple(w) for w in wins]
