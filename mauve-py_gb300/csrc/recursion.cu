// The recursive anchor search's gap finding for one LCB of two genomes:
// ProgressiveAligner::recurseOnPairs (LM/ProgressiveAligner.cpp:682-924)
// with getInterveningCoordinates (:566-588) and pairwiseAnchorSearch's cut
// of the gap sequences (:598-613).  Host code: a column scan of the LCB's
// two gapped rows.  Its output is the gap list mvg_gap_anchor_search takes.
//
// The bounding anchors recurseOnPairs builds are zero-length libMems
// Matches; their coordinates follow libMems' conventions
// (LM/HybridAbstractMatch.h:151-265, LM/AbstractMatch.h:209-214): a signed
// 1-based start per sequence (negative = reverse strand), End = Start - 1
// for a forward zero-length match and Start for a reverse one, Invert()
// negating every start.  The cut keeps the reference's arithmetic exactly:
// the gap sequence starts at the left anchor's end + 1 and is one base
// shorter than the distance to the right anchor's start.
#include <stdint.h>
#include <stdlib.h>

#include "mvg_internal.h"

namespace mvg {
namespace {

// A zero-length bounding anchor of two sequences (0 start = undefined).
struct Bound {
  int64_t start[2] = {0, 0};
  bool set = false;
  int64_t end(int q) const { return start[q] > 0 ? start[q] - 1 : start[q]; }
  int64_t length(int) const { return 0; }  // zero-length in every sequence
};

// The anchor at `consumed` characters into the LCB from its left end (or,
// on a reverse strand, from its right end).
Bound bound_at(const int64_t lend[2], const int64_t rend[2], const bool rev[2], const int64_t consumed[2]) {
  Bound b;
  b.set = true;
  for (int q = 0; q < 2; ++q) b.start[q] = rev[q] ? -(rend[q] - consumed[q]) : lend[q] + consumed[q];
  return b;
}

// getInterveningCoordinates for sequence q between r_begin and r_end.
void intervening(const int64_t lend[2], const int64_t rend[2], const Bound& rb, const Bound& re, int q, int64_t* gl,
                 int64_t* gr) {
  if ((re.set && re.start[q] == 0) || (rb.set && rb.start[q] == 0)) {
    *gl = 0;
    *gr = 0;
    return;
  }
  int64_t r = re.set ? re.start[q] : rend[q] + 1;
  int64_t l = rb.set ? rb.end(q) + 1 : lend[q];
  if (r < 0 || l < 0) {
    r = rb.set ? -rb.start[q] : rend[q] + 1;
    l = re.set ? -re.start[q] + re.length(q) : 1;
  }
  *gl = l;
  *gr = r;
}

}  // namespace
}  // namespace mvg

using namespace mvg;

extern "C" int mvg_recursion_gaps(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, int64_t left_end_a,
                                  int reverse_a, int64_t left_end_b, int reverse_b, uint64_t genome_len_a,
                                  uint64_t genome_len_b, int64_t min_gap, int64_t* gaps, uint64_t cap,
                                  uint64_t* ngaps, int64_t* flanks) {
  if (!ngaps || (ncols && (!row_a || !row_b)) || (cap && !gaps) || left_end_a < 1 || left_end_b < 1 || min_gap < 0)
    return report_error(MVG_ERR_ARG, "bad argument");
  *ngaps = 0;
  const int64_t lend[2] = {left_end_a, left_end_b};
  const bool rev[2] = {reverse_a != 0, reverse_b != 0};
  const uint64_t glen[2] = {genome_len_a, genome_len_b};
  const uint8_t* rows[2] = {row_a, row_b};
  int64_t nchar[2] = {0, 0};
  for (uint64_t c = 0; c < ncols; ++c)
    for (int q = 0; q < 2; ++q) nchar[q] += rows[q][c] != '-';
  const int64_t rend[2] = {lend[0] + nchar[0] - 1, lend[1] + nchar[1] - 1};
  if ((uint64_t)rend[0] > genome_len_a || (uint64_t)rend[1] > genome_len_b)
    return report_error(MVG_ERR_RANGE, "LCB reaches past its genome");
  auto both = [&](uint64_t c) { return rows[0][c] != '-' && rows[1][c] != '-'; };

  if (flanks) {
    // the unaligned stretches before the first and after the last column
    // where both sequences are aligned (iv_regions, :738-834)
    int64_t left[2][2] = {{0, 0}, {0, 0}}, right[2][2] = {{0, 0}, {0, 0}};  // per genome: [start, end)
    int64_t run[2] = {0, 0};
    for (uint64_t c = 0; c <= ncols; ++c) {
      if (c == ncols || both(c)) {
        if (c == 0) break;
        for (int q = 0; q < 2; ++q) {
          if (!rev[q]) {
            left[q][0] = lend[q];
            left[q][1] = lend[q] + run[q];
          } else {
            right[q][0] = rend[q] - run[q] + 1;
            right[q][1] = rend[q] + 1;
          }
        }
        break;
      }
      for (int q = 0; q < 2; ++q) run[q] += c < ncols && rows[q][c] != '-';
    }
    run[0] = run[1] = 0;
    for (uint64_t c = ncols; c > 0; --c) {
      if (both(c - 1)) {
        if (c == ncols) break;
        for (int q = 0; q < 2; ++q) {
          if (!rev[q]) {
            right[q][0] = rend[q] - run[q] + 1;
            right[q][1] = rend[q] + 1;
          } else {
            left[q][0] = lend[q];
            left[q][1] = lend[q] + run[q];
          }
        }
        break;
      }
      for (int q = 0; q < 2; ++q) run[q] += rows[q][c - 1] != '-';
    }
    for (int q = 0; q < 2; ++q) {
      int64_t* f = flanks + 4 * q;
      f[0] = f[1] = f[2] = f[3] = 0;
      int k = 0;
      if (left[q][0] < left[q][1]) {
        f[0] = left[q][0];
        f[1] = left[q][1];
        k = 1;
      }
      if (right[q][0] < right[q][1]) {
        if (k == 1 && right[q][0] == left[q][1]) {
          f[1] = right[q][1];  // adjacent: one interval
        } else {
          f[2 * k] = right[q][0];
          f[2 * k + 1] = right[q][1];
        }
      }
    }
  }

  // inter-anchor gaps: both sequences more than min_gap characters between
  // two columns where both are aligned (or the LCB's end) (:836-921)
  int64_t consumed[2] = {0, 0}, prev[2] = {0, 0};
  bool in_gap = false;
  uint64_t n = 0;
  for (uint64_t c = 0; c <= ncols; ++c) {
    if (c == ncols || both(c)) {
      if (in_gap && consumed[0] - prev[0] > min_gap && consumed[1] - prev[1] > min_gap) {
        Bound lb = bound_at(lend, rend, rev, prev);
        Bound rb;
        // (the reference compares the counts with the right ends' coordinates)
        if (consumed[1] != rend[1] && consumed[0] != rend[0]) rb = bound_at(lend, rend, rev, consumed);
        if (rev[0]) {  // anchors are kept with sequence A forward
          Bound t = lb;
          lb = rb;
          rb = t;
          for (Bound* b : {&lb, &rb})
            if (b->set)
              for (int q = 0; q < 2; ++q) b->start[q] = -b->start[q];
        }
        if (n < cap) {
          for (int q = 0; q < 2; ++q) {
            int64_t gl = 0, gr = 0;
            intervening(lend, rend, lb, rb, q, &gl, &gr);
            int64_t diff = gr - gl;
            diff = diff > 0 ? diff - 1 : 0;
            if (!(diff > 0 && (uint64_t)(gl + diff - 1) <= glen[q])) diff = 0;
            gaps[4 * n + 2 * q] = diff > 0 ? gl - 1 : 0;
            gaps[4 * n + 2 * q + 1] = diff;
          }
        }
        ++n;
      }
      prev[0] = consumed[0];
      prev[1] = consumed[1];
      in_gap = false;
    } else {
      in_gap = true;
    }
    if (c < ncols)
      for (int q = 0; q < 2; ++q) consumed[q] += rows[q][c] != '-';
  }
  *ngaps = n;
  if (n > cap) return report_error(MVG_ERR_CAPACITY, "gap output buffer too small");
  return 0;
}
