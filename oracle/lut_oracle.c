/* CPU oracle for the genome -> reference index LUT and its clean-up passes.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference's
 * sequential loops, the checker for the CUDA LUT kernels.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * Parity is pinned against the reference's own code: its compiled
 * mauve/indexutils.pyx (built into oracle/_ref by
 * oracle/build_ref_indexutils.sh) and its buildIndex() loop executed from
 * mauve/buildindex.py with the XMFA parse replaced by in-memory blocks
 * (tests/golden/make_golden_lut.py writes tests/golden/lut.npz).
 *
 * Error returns mirror the Python exceptions the reference raises:
 * -2 = IndexError (an index outside the LUT or a sequence), -3 = a value
 * that does not fit the int32 LUT (numpy's OverflowError).
 */
#include <stdint.h>
#include <string.h>

#include "mauve_oracle.h"

/* mauve/buildindex.py:112-130.  The LUT starts all -1; every block walks its
 * columns, advancing each side's index on a non-gap character, and a column
 * whose two characters are equal writes lut[genome_idx] = ref_idx when
 * genome_idx < n.  genome_idx is start-1 before the first column, so -1 can
 * reach the write (both characters '-'); numpy then writes lut[n-1]. */
int64_t mo_lut_from_blocks(const int64_t* g_start, const int64_t* r_start, const uint64_t* col_off,
                           const uint8_t* g_rows, const uint8_t* r_rows, uint64_t nblocks,
                           int32_t* lut, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) lut[i] = -1;
  for (uint64_t b = 0; b < nblocks; ++b) {
    int64_t gi = g_start[b] - 1, ri = r_start[b] - 1;
    for (uint64_t c = col_off[b]; c < col_off[b + 1]; ++c) {
      uint8_t g = g_rows[c], r = r_rows[c];
      if (g != '-') ++gi;
      if (r != '-') ++ri;
      if (g == r && gi < (int64_t)n) {
        int64_t t = gi < 0 ? gi + (int64_t)n : gi;
        if (t < 0) return -2;
        if (ri < INT32_MIN || ri > INT32_MAX) return -3;
        lut[t] = (int32_t)ri;
      }
    }
  }
  return 0;
}

/* mauve/indexutils.pyx:27-44 (fixZeroIdx).  Bounds-checked like the
 * Cython function: a scan that runs off the LUT, an empty genome or a
 * reference index past the reference sequence is an IndexError. */
int mo_fix_zero_idx(int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t glen,
                    const uint8_t* ref, uint64_t rlen) {
  if (n == 0) return -2;
  if (lut[0] != -1) return 0;
  uint64_t nx = 1;
  for (;;) {
    if (nx >= n) return -2;
    if (lut[nx] == -1 || nx < 10) { ++nx; continue; }
    break;
  }
  int32_t ref_idx = (int32_t)((int64_t)lut[nx] - (int64_t)nx);
  if (ref_idx > -1) {
    if (glen == 0 || (uint64_t)ref_idx >= rlen) return -2;
    if (genome[0] == ref[ref_idx]) lut[0] = ref_idx;
  }
  return 0;
}

/* Shared body of fillGaps (mauve/indexutils.pyx:47-75), smoothEdges
 * (:78-108) and findGaps (:111-139): scan idx = 1..n-1; at a gap start
 * (fill: lut[idx] == -1, smooth: lut[idx] != lut[idx-1] + 1; both with
 * lut[idx-1] != -1) look for the first upper in idx+1 .. idx+width with
 * lut[upper] - lut[idx-1] == upper - (idx-1) and overwrite lut[idx-1..upper]
 * with the consecutive run.  gaps (findGaps only) records upper-(idx-1) at
 * a filled gap start and -1 at one that found no partner. */
static void run_fill(int32_t* lut, uint64_t n, int width, int smooth, int32_t* gaps) {
  for (uint64_t idx = 1; idx < n; ++idx) {
    int32_t m = lut[idx], lo = lut[idx - 1];
    int start = smooth ? (m != (int32_t)((uint32_t)lo + 1u)) : (m == -1);
    if (!start || lo == -1) continue;
    uint64_t lower = idx - 1;
    int ok = 0;
    for (uint64_t up = idx + 1; up < n; ++up) {
      if ((int64_t)(up - idx) > (int64_t)width) break;
      if ((int32_t)((uint32_t)lut[up] - (uint32_t)lo) == (int32_t)(up - lower)) {
        for (uint64_t k = lower; k <= up; ++k) lut[k] = lo + (int32_t)(k - lower);
        if (gaps) gaps[idx] = (int32_t)(up - lower);
        ok = 1;
        break;
      }
    }
    if (gaps && !ok) gaps[idx] = -1;
  }
}

void mo_fill_gaps(int32_t* lut, uint64_t n, int max_gap_width) { run_fill(lut, n, max_gap_width, 0, 0); }

void mo_smooth_edges(int32_t* lut, uint64_t n, int smoothing_radius) { run_fill(lut, n, smoothing_radius, 1, 0); }

/* mauve/indexutils.pyx:111-139: fillGaps with width 300 that also returns
 * the per-gap-start record (zero elsewhere). */
void mo_find_gaps(int32_t* lut, uint64_t n, int32_t* gaps) {
  memset(gaps, 0, n * sizeof(int32_t));
  run_fill(lut, n, 300, 0, gaps);
}

/* mauve/indexutils.pyx:142-156 (findEdges), as the per-index 0/1 mask
 * before it is packed: index 0, and every i with lut[i] - lut[i-1] != 1 in
 * wrapping int32 arithmetic. */
void mo_find_edges(const int32_t* lut, uint64_t n, uint8_t* edges) {
  if (n == 0) return;
  edges[0] = 1;
  for (uint64_t i = 1; i < n; ++i) edges[i] = (uint32_t)lut[i] - (uint32_t)lut[i - 1] != 1u;
}

/* mauve/indexutils.pyx:159-175 (findMismatches): for idx < glen with a
 * mapped index, 1 when the genome base differs from the reference base it
 * maps to.  -2 when a mapped index lies outside the reference or glen > n. */
int mo_find_mismatches(const int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t glen,
                       const uint8_t* ref, uint64_t rlen, uint8_t* mism) {
  memset(mism, 0, n);
  if (glen > n) return -2;
  for (uint64_t i = 0; i < glen; ++i) {
    int32_t m = lut[i];
    if (m == -1) continue;
    if (m < 0 || (uint64_t)m >= rlen) return -2;
    mism[i] = genome[i] != ref[m];
  }
  return 0;
}

/* mauve/indexutils.pyx:178-186 (findDuplicateMappings): values are clipped
 * to [0, 2^31-1] (so -1 counts as 0), counted, and the number of values
 * seen more than once, minus one, is returned. */
int64_t mo_find_duplicate_mappings(const int32_t* lut, uint64_t n, uint32_t* counts, uint64_t ncounts) {
  memset(counts, 0, ncounts * sizeof(uint32_t));
  if (n == 0) return -1;
  for (uint64_t i = 0; i < n; ++i) {
    int32_t v = lut[i] < 0 ? 0 : lut[i];
    if ((uint64_t)v >= ncounts) return -2;
    counts[v]++;
  }
  int64_t dup = 0;
  for (uint64_t v = 0; v < ncounts; ++v) dup += counts[v] > 1;
  return dup - 1;
}
