// Anchor columns of a window of a two-genome alignment, which cut it into
// the ranges the gap DP aligns: MUSCLE's AnchoredProfileProfile
// (muscle/libMUSCLE/anchoredpp.cpp:429-458) as MuscleInterface::
// ProfileAlignFast calls it for two single-sequence profiles
// (libMems/MuscleInterface.cpp:1053-1109: DNA, PPSCORE_SPN).  Host code.
//
// Per column the score is LetterObjScoreXP's (anchoredpp.cpp:256-329) for one
// pair of sequences of weight 1: the NUC_SP letter score (with its +60
// centre, muscle/libMUSCLE/nucmx.cpp:8-25) where both rows hold a base
// between the first and last column not gapped in both, and the pair's gap
// penalties (open -400, extend 0, a terminal gap half an open) spread evenly
// over each gap run's columns (ScoreSeqPairGaps, anchoredpp.cpp:96-247).  It
// is smoothed over 21 columns with a ceiling of 999 (WindowSmooth,
// muscle/libMUSCLE/anchors.cpp:9-47); columns scoring at least 90 raw and
// smoothed are candidates (FindBestColsComboPP, anchoredpp.cpp:334-351),
// merged within windows of 96 columns (MergeBestCols, anchors.cpp:137-186).
// All arithmetic is the reference's single-precision arithmetic in its
// order, so every threshold decision is the same.
#include <stdint.h>

#include <vector>

#include "lcb_host.h"
#include "mvg_internal.h"

namespace mvg {
namespace {

constexpr float kCenter = 60.0f;  // NUC_SP_CENTER = 2 * NUC_EXTEND
constexpr float kNucSp[4][4] = {{91, -114, -31, -123}, {-114, 100, -125, -31}, {-31, -125, 100, -114},
                                {-123, -31, -114, 91}};
constexpr float kGapOpen = -400.0f;
constexpr float kGapExtend = 0.0f;
constexpr float kTermGap = kGapOpen / 2;  // TERMGAPS_Half
constexpr unsigned kSmoothWindow = 21;
constexpr double kSmoothCeil = 999.0;
constexpr double kMinBestColScore = 90.0;
constexpr double kMinSmoothScore = 90.0;
constexpr unsigned kAnchorSpacing = 96;
constexpr unsigned kInsane = 0xffffffffu;

bool is_gap(uint8_t c) { return c == '-' || c == '.'; }

// DNA letter of a column character; 4 (the wildcard) for anything else.
unsigned letter(uint8_t c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': case 'U': case 'u': return 3;
    default: return 4;
  }
}

// The per-column score of LetterObjScoreXP for the pair (one sequence each).
void column_scores(const uint8_t* a, const uint8_t* b, unsigned n, std::vector<float>& score) {
  std::vector<float> mm(n, 0.0f), gg(n, 0.0f);
  unsigned start = 0, end = n - 1;
  for (unsigned c = 0; c < n; ++c)
    if (!is_gap(a[c]) || !is_gap(b[c])) {
      start = c;
      break;
    }
  for (int c = (int)n - 1; c >= 0; --c)
    if (!is_gap(a[c]) || !is_gap(b[c])) {
      end = (unsigned)c;
      break;
    }
  for (unsigned c = start; c <= end; ++c) {
    const unsigned l1 = letter(a[c]), l2 = letter(b[c]);
    if (l1 >= 4 || l2 >= 4) continue;
    mm[c] = (float)kNucSp[l1][l2] + kCenter;
  }
  bool gapping[2] = {false, false};
  unsigned gap_left = 0;
  float cur = 0.0f;
  for (unsigned c = start; c <= end; ++c) {
    const bool g[2] = {is_gap(a[c]), is_gap(b[c])};
    if (g[0] && g[1]) continue;
    if (g[0] || g[1]) {
      const int q = g[0] ? 0 : 1;
      if (!gapping[q]) {
        gap_left = c;
        cur += c == start ? kTermGap : kGapOpen;
        gapping[q] = true;
      } else {
        cur += kGapExtend;
      }
      continue;
    }
    if (gapping[0] || gapping[1]) {  // spread the run's penalty over its columns
      const float per_site = cur / (float)(c - gap_left);
      for (unsigned k = gap_left; k < c; ++k) gg[k] = per_site;
      gap_left = kInsane;
      cur = 0.0f;
    }
    gapping[0] = gapping[1] = false;
  }
  if (gapping[0] || gapping[1]) {  // a terminal gap pays half an open
    cur -= kGapOpen;
    cur += kTermGap;
    const float per_site = cur / (float)(n - gap_left);
    for (unsigned k = gap_left; k < n; ++k) gg[k] = per_site;
  }
  score.assign(n, 0.0f);
  const float w = 1.0f;  // sequence weight product of two one-sequence profiles
  for (unsigned c = 0; c < n; ++c) score[c] += w * (mm[c] + gg[c]);
}

float ceil_score(float x) { return (float)(x > kSmoothCeil ? kSmoothCeil : x); }

}  // namespace
}  // namespace mvg

using namespace mvg;

void mvg::anchor_columns(const uint8_t* row_a, const uint8_t* row_b, unsigned n, std::vector<unsigned>& out) {
  out.clear();
  if (n == 0) return;
  std::vector<float> score, smooth(n, 0.0f);
  column_scores(row_a, row_b, n, score);
  // WindowSmooth
  if (n > kSmoothWindow) {
    const unsigned w2 = kSmoothWindow / 2;
    float total = 0.0f;
    for (unsigned i = 0; i < kSmoothWindow; ++i) total += ceil_score(score[i]);
    for (unsigned i = w2;; ++i) {
      smooth[i] = total / (float)kSmoothWindow;
      if (i == n - w2 - 1) break;
      total -= ceil_score(score[i - w2]);
      total += ceil_score(score[i + w2 + 1]);
    }
  }
  // FindBestColsComboPP
  std::vector<unsigned> best;
  for (unsigned c = 0; c < n; ++c) {
    if (score[c] < kMinBestColScore) continue;
    if (smooth[c] < kMinSmoothScore) continue;
    best.push_back(c);
  }
  // MergeBestCols: two candidates within a window keep the better scoring;
  // more keep the one nearest the first, among all but the window's last
  for (size_t k = 0; k < best.size();) {
    const unsigned first = best[k];
    unsigned within = 0;
    for (size_t i = k + 1; i < best.size(); ++i) {
      if (best[i] - first >= kAnchorSpacing) break;
      ++within;
    }
    unsigned anchor = first;
    if (within == 1) {
      const unsigned second = best[k + 1];
      anchor = score[first] > score[second] ? first : second;
    } else if (within > 1) {
      int closest_dist = (int)kAnchorSpacing;
      unsigned closest = first;
      for (size_t i = k + 1; i < k + within; ++i) {
        int d = (int)best[i] - (int)first;
        if (d < 0) d = -d;
        if (d < closest_dist) {
          closest = best[i];
          closest_dist = d;
        }
      }
      anchor = closest;
    }
    out.push_back(anchor);
    k += within + 1;
  }
}

extern "C" int mvg_anchor_columns(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, uint32_t* cols,
                                  uint64_t cap, uint64_t* ncols_out) {
  if (!ncols_out || (ncols && (!row_a || !row_b)) || (cap && !cols)) return report_error(MVG_ERR_ARG, "null argument");
  if (ncols >= (1ull << 31)) return report_error(MVG_ERR_ARG, "window longer than 2^31 columns");
  std::vector<unsigned> found;
  anchor_columns(row_a, row_b, (unsigned)ncols, found);
  const uint64_t m = found.size();
  for (uint64_t k = 0; k < m && k < cap; ++k) cols[k] = found[k];
  *ncols_out = m;
  if (m > cap) return report_error(MVG_ERR_CAPACITY, "anchor column buffer too small");
  return 0;
}
