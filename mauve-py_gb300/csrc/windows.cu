// Windows of the gapped-alignment pass over one LCB of two genomes:
// ProgressiveAligner::refineAlignment (LM/ProgressiveAligner.cpp:1119-1165)
// with removeLargeGapsPP (:1051-1117) and IsDenseEnough (:1015-1038).  Host
// code over the LCB's two gapped rows; every window is a column range of
// the LCB.  The windows that are not gap windows and hold bases of both
// genomes are what ProfileAlignFast(anchored) realigns
// (mvg_anchor_columns and the batched gap DP); the LCB's new rows are the
// windows' rows concatenated in order (:1215-1230).
//
// The same windows drive the final iterative-refinement pass
// (refineAlignment with profile_aln = false, :1199-1212): a window of
// density class 1 or 2 goes through MuscleInterface::RefineFast
// (LM/MuscleInterface.cpp:823-894) with RefineW's column windows of 500 or
// 200 columns (MU/refinew.cpp:75-184), each of which MUSCLE realigns from
// its bases alone -- for two sequences one NWSmall problem, the first
// genome as profile A; a class-0 window goes through RefineVert, which
// returns at once for fewer than three sequences (MU/refinevert.cpp:60-61).
// mvg_refine_fast_ranges lists those column windows.
//
// Cuts follow GappedAlignment::Split / CropStart / CropEnd
// (LM/GappedAlignment.h:123-229): Split(k) keeps columns [0, k) on the left;
// halving a window of L columns keeps L - L/2 columns on the left and L/2 on
// the right, and the left half is examined again first.  A genome with no
// base in a window is undefined there (Length 0 -> NO_MATCH), which changes
// the window's multiplicity in the density test.
#include <stdint.h>

#include <algorithm>
#include <list>
#include <vector>

#include "lcb_host.h"
#include "mvg_internal.h"

namespace mvg {
namespace {

constexpr uint64_t kMaxGapLength = 5000;  // max_gap_length (:62)
constexpr uint64_t kLcbHangover = 300;    // lcb_hangover (:63)
constexpr double kMinWindowSize = 200;    // min_window_size (:58)
constexpr double kMinDensity = .5;        // min_density (:60)
constexpr double kMaxDensity = .9;        // max_density (:61)

using Window = LcbWindow;

// RefineW's window widths by density class (refineAlignment with
// profile_aln = false, :1201-1212: RefineFast(w), RefineFast(w, 500),
// RefineFast(w, 200)); 0 = no change (RefineVert needs three sequences,
// MU/refinevert.cpp:60-61).
constexpr uint64_t kRefineWidth[3] = {0, 500, 200};

}  // namespace

// refineAlignment's windows of one LCB (removeLargeGapsPP, then halving by
// IsDenseEnough), each with its density class.
std::vector<Window> lcb_windows(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, double max_window_size) {
  const uint8_t* rows[2] = {row_a, row_b};
  // prefix base counts, for the bases of any column range
  std::vector<uint64_t> pre[2];
  for (int q = 0; q < 2; ++q) {
    pre[q].assign(ncols + 1, 0);
    for (uint64_t c = 0; c < ncols; ++c) pre[q][c + 1] = pre[q][c] + (rows[q][c] != '-');
  }
  // removeLargeGapsPP: cut out every stretch of more than max_gap_length
  // columns in which the genomes are never aligned to each other, keeping
  // lcb_hangover columns on either side with the aligned parts
  std::list<Window> wins;
  const uint64_t kNone = ~0ull;
  uint64_t gap_cols = 0, last_aln = kNone, base = 0;
  for (uint64_t c = 0; c < ncols; ++c) {
    if (rows[0][c] != '-' && rows[1][c] != '-') {
      if (gap_cols > kMaxGapLength) {
        if (last_aln != kNone) {
          const uint64_t k = last_aln + kLcbHangover - base;
          wins.push_back({base, base + k, false, 0});
          base += k;
        }
        const uint64_t k = c - kLcbHangover - base;
        wins.push_back({base, base + k, true, 0});
        base += k;
      }
      last_aln = c;
      gap_cols = 0;
    } else {
      ++gap_cols;
    }
  }
  if (gap_cols > kMaxGapLength) {
    if (last_aln != kNone) {
      const uint64_t k = last_aln + kLcbHangover - base;
      wins.push_back({base, base + k, false, 0});
      base += k;
    }
    wins.push_back({base, ncols, true, 0});
  } else {
    wins.push_back({base, ncols, false, 0});
  }
  // halve windows too long for their density (IsDenseEnough)
  auto density_class = [&](const Window& w) {
    const uint64_t len = w.hi - w.lo;
    double total = 0;
    unsigned mult = 0;
    for (int q = 0; q < 2; ++q) {
      const uint64_t n = pre[q][w.hi] - pre[q][w.lo];
      if (n == 0) continue;  // undefined in this window
      total += (double)n;
      ++mult;
    }
    const double density = total / ((double)len * (double)mult);
    const double threshold = ((kMaxDensity - kMinDensity) / (kMinWindowSize - max_window_size)) *
                                 ((double)len - max_window_size) +
                             kMinDensity;
    if (density > kMaxDensity) return 2;
    if (density > threshold) return 1;
    return 0;
  };
  for (auto it = wins.begin(); it != wins.end();) {
    const uint64_t len = it->hi - it->lo;
    const int d = density_class(*it);
    if ((d == 0 && (double)len > max_window_size / 3) || (d == 1 && (double)len > max_window_size) ||
        (d == 2 && (double)len > max_window_size * 3)) {
      const uint64_t half = len / 2;  // CropEnd(half) on the left, CropStart(len - half) on the right
      Window right{it->hi - half, it->hi, it->gap, 0};
      it->hi -= half;
      wins.insert(std::next(it), right);
      continue;
    }
    it->density = d;
    ++it;
  }
  return std::vector<Window>(wins.begin(), wins.end());
}

uint64_t refine_width(int density) { return kRefineWidth[density]; }

}  // namespace mvg

using namespace mvg;

extern "C" int mvg_refine_windows(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols,
                                  double max_window_size, int64_t* windows, uint64_t cap, uint64_t* nwindows) {
  if (!nwindows || (ncols && (!row_a || !row_b)) || (cap && !windows) || !(max_window_size > kMinWindowSize))
    return report_error(MVG_ERR_ARG, "bad argument");
  *nwindows = 0;
  const std::vector<Window> wins = lcb_windows(row_a, row_b, ncols, max_window_size);
  uint64_t n = 0;
  for (const Window& w : wins) {
    if (n < cap) {
      windows[3 * n] = (int64_t)w.lo;
      windows[3 * n + 1] = (int64_t)w.hi;
      windows[3 * n + 2] = w.gap ? 1 : 0;
    }
    ++n;
  }
  *nwindows = n;
  if (n > cap) return report_error(MVG_ERR_CAPACITY, "window buffer too small");
  return 0;
}

extern "C" int mvg_refine_fast_ranges(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols,
                                      double max_window_size, int64_t* ranges, uint64_t cap, uint64_t* nranges) {
  if (!nranges || (ncols && (!row_a || !row_b)) || (cap && !ranges) || !(max_window_size > kMinWindowSize))
    return report_error(MVG_ERR_ARG, "bad argument");
  *nranges = 0;
  uint64_t n = 0;
  for (const Window& w : lcb_windows(row_a, row_b, ncols, max_window_size)) {
    const uint64_t width = kRefineWidth[w.density];
    if (w.gap || width == 0) continue;
    for (uint64_t lo = w.lo; lo < w.hi; lo += width) {  // RefineW's column windows (MU/refinew.cpp:113-118)
      if (n < cap) {
        ranges[2 * n] = (int64_t)lo;
        ranges[2 * n + 1] = (int64_t)std::min(w.hi, lo + width);
      }
      ++n;
    }
  }
  *nranges = n;
  if (n > cap) return report_error(MVG_ERR_CAPACITY, "range buffer too small");
  return 0;
}
