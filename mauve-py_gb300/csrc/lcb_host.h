// Host steps over one LCB of two genomes shared by the window, anchor and
// whole-pass entry points (windows.cu, anchors.cu, gapped.cu).
#pragma once
#include <stdint.h>

#include <vector>

namespace mvg {

// A window of refineAlignment: columns [lo, hi), whether it is a gap window
// (removeLargeGapsPP) and IsDenseEnough's class (0, 1, 2) of the window.
struct LcbWindow {
  uint64_t lo, hi;
  bool gap;
  int density;
};

// refineAlignment's windows of one LCB (LM/ProgressiveAligner.cpp:1119-1165).
std::vector<LcbWindow> lcb_windows(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols,
                                   double max_window_size);

// RefineW's column-window width for a density class in the final refinement
// pass (0 = the window is left as it is).
uint64_t refine_width(int density);

// MUSCLE's anchor columns of a window (FindAnchorColsPP for two sequences),
// ascending.
void anchor_columns(const uint8_t* row_a, const uint8_t* row_b, unsigned n, std::vector<unsigned>& cols);

}  // namespace mvg
