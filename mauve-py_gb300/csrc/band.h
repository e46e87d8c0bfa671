// Diagonal band geometry for the banded gap DP, shared by host and device.
//
// A problem (LA, LB) with band (delta, half) keeps, for every row i, the
// columns within `half` of the line j = i*LB/LA + delta.  The kernel works in
// strips of `srows` rows, so the kept region is a staircase: strip k spans
// [lo_k, hi_k], the union over its rows, with strip 0 starting at column 1
// and the last strip ending at column LB (the path's two end cells).  Both
// bounds are non-decreasing in k.  The full DP is the same geometry with
// lo_k = 1 and hi_k = LB for every strip.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define MVG_HD __host__ __device__ __forceinline__
#else
#define MVG_HD inline
#endif

namespace mvg {

struct Band {
  int LA, LB, delta, half, srows, nstrips;
  bool full;
};

MVG_HD Band make_band(int LA, int LB, int delta, int half, int srows) {
  Band b;
  b.LA = LA;
  b.LB = LB;
  b.delta = delta;
  b.half = half < 0 ? 0 : half;
  b.srows = srows;
  b.nstrips = (LA + srows - 1) / srows;
  b.full = false;
  return b;
}

MVG_HD Band make_full(int LA, int LB, int srows) {
  Band b = make_band(LA, LB, 0, 0, srows);
  b.full = true;
  return b;
}

MVG_HD int64_t band_center(const Band& b, int i) { return (int64_t)i * b.LB / b.LA + b.delta; }

MVG_HD int band_lo(const Band& b, int k) {
  if (k == 0 || b.full) return 1;
  int64_t lo = band_center(b, k * b.srows + 1) - b.half;
  if (lo < 1) lo = 1;
  if (lo > b.LB) lo = b.LB;
  return (int)lo;
}

MVG_HD int band_hi(const Band& b, int k) {
  if (k == b.nstrips - 1 || b.full) return b.LB;
  int last = (k + 1) * b.srows;
  if (last > b.LA) last = b.LA;
  int64_t hi = band_center(b, last) + b.half + 1;
  if (hi < 1) hi = 1;
  if (hi > b.LB) hi = b.LB;
  return (int)hi;
}

// Last row whose strip starts at column 1 (so column 0 is its left boundary).
MVG_HD int band_last_row_at_col1(const Band& b, int LA) {
  int k = 0;
  while (k + 1 < b.nstrips && band_lo(b, k + 1) == 1) ++k;
  int last = (k + 1) * b.srows;
  return last > LA ? LA : last;
}

// Traceback words of one lane for a strip of width W: R nibbles per step,
// W + 31 steps.
MVG_HD int band_words_per_lane(int W, int rows_per_lane) { return ((W + 31) * 4 * rows_per_lane + 31) / 32; }

MVG_HD uint64_t band_tb_words(const Band& b, int rows_per_lane) {
  uint64_t words = 0;
  for (int k = 0; k < b.nstrips; ++k)
    words += (uint64_t)band_words_per_lane(band_hi(b, k) - band_lo(b, k) + 1, rows_per_lane) * 32;
  return words;
}

MVG_HD uint64_t band_cells(const Band& b) {
  uint64_t cells = 0;
  for (int k = 0; k < b.nstrips; ++k) {
    int rows = b.LA - k * b.srows;
    if (rows > b.srows) rows = b.srows;
    cells += (uint64_t)rows * (band_hi(b, k) - band_lo(b, k) + 1);
  }
  return cells;
}

}  // namespace mvg
