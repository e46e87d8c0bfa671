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

// Ring-schedule geometry of the banded kernel (gapdp_ring.cuh).
//
// Rows are cut into groups of R; group g (rows gR+1 .. gR+R) keeps columns
// [lo_g, lo_g + W) with lo_g = floor((gR+1)*LB/LA) + delta - half and the
// same width W for every group, W = 2*half + 2 + ceil((R-1)*LB/LA): the
// columns within `half` of the band centre of each of its rows, like Band.
// lo_g is not clamped: column 0 is the matrix's left boundary, columns below
// it and above LB lie outside the matrix.  Lane g mod 32 of a warp runs group
// g on wavefront steps [start_g, start_g + W) with start_g = g + lo_g - lo_0,
// so group g reaches column j (step j + g - lo_0) exactly one step after
// group g-1 did, and the cell above comes from the previous lane of the ring.
struct RingBand {
  int LA, LB, R, G, delta, half, W, lo0, lo_last;
  int64_t steps;  // wavefront steps of the whole problem
};

MVG_HD int ring_lo(const RingBand& b, int g) {
  return (int)(((int64_t)g * b.R + 1) * b.LB / b.LA + b.delta - b.half);
}

MVG_HD RingBand make_ring_band(int LA, int LB, int delta, int half, int R) {
  RingBand b;
  b.LA = LA;
  b.LB = LB;
  b.R = R;
  b.delta = delta;
  b.half = half < 0 ? 0 : half;
  b.G = (LA + R - 1) / R;
  const int64_t span = ((int64_t)(R - 1) * LB + LA - 1) / LA;
  const int64_t W = 2 * (int64_t)b.half + 2 + span;
  b.W = W > (1 << 30) ? (1 << 30) : (int)W;
  b.lo0 = ring_lo(b, 0);
  b.lo_last = ring_lo(b, b.G - 1);
  b.steps = (int64_t)(b.G - 1) + b.lo_last - b.lo0 + b.W;
  return b;
}

// Whether the ring schedule is valid for this band: group 0 reaches column 1
// and the last group column LB (the path's end cells); lo_g <= LB and
// lo_g + W > 1 for every group (lo is non-decreasing); each group's first
// column lies inside its predecessor's range (lo_g - lo_{g-1} <=
// ceil(R*LB/LA) <= W - 1); and a lane finishes group g before it starts
// group g+32: W <= 32 + lo_{g+32} - lo_g, where lo_{g+32} - lo_g >=
// floor(32*R*LB/LA).
MVG_HD bool ring_eligible(const RingBand& b) {
  if (b.half > (1 << 20) || b.delta > (1 << 24) || b.delta < -(1 << 24)) return false;
  if (b.lo0 > 1 || b.lo0 + b.W - 1 < 1) return false;
  if (b.lo_last > b.LB || b.lo_last + b.W - 1 < b.LB) return false;
  const int64_t step = ((int64_t)b.R * b.LB + b.LA - 1) / b.LA;
  if (step > b.W - 1) return false;
  if (b.G > 32 && (int64_t)b.W > 32 + (int64_t)32 * b.R * b.LB / b.LA) return false;
  return true;
}

// Traceback layout of a ring-scheduled problem: each lane stores its R
// nibbles per step as one stream.  When R divides 8, 8 / R steps share a
// word (nibble r of step s at nibble R*(s mod 8/R) + r of word s / (8/R));
// otherwise a step takes ceil(R / 8) words (nibble r in word s*NW + r/8 at
// nibble r mod 8).  Word x of lane t sits at x*32 + t.
MVG_HD int ring_steps_per_word(int R) { return (R < 8 && 8 % R == 0) ? 8 / R : 1; }
MVG_HD int ring_words_per_step(int R) { return (R + 7) / 8; }
MVG_HD void ring_tb_at(int R, int64_t s, int r, int64_t& word, int& shift) {
  const int per = ring_steps_per_word(R);
  if (per > 1) {
    word = s / per;
    shift = 4 * (R * (int)(s % per) + r);
  } else {
    word = s * ring_words_per_step(R) + (r >> 3);
    shift = 4 * (r & 7);
  }
}
MVG_HD uint64_t ring_tb_words(const RingBand& b) {
  const int per = ring_steps_per_word(b.R);
  const uint64_t w = per > 1 ? (uint64_t)((b.steps + per - 1) / per) : (uint64_t)b.steps * ring_words_per_step(b.R);
  return w * 32;
}

// Matrix cells inside the kept region (rows 1..LA, columns 1..LB).
MVG_HD uint64_t ring_cells(const RingBand& b) {
  uint64_t cells = 0;
  for (int g = 0; g < b.G; ++g) {
    int rows = b.LA - g * b.R;
    if (rows > b.R) rows = b.R;
    int lo = ring_lo(b, g), hi = lo + b.W - 1;
    if (lo < 1) lo = 1;
    if (hi > b.LB) hi = b.LB;
    if (hi >= lo) cells += (uint64_t)rows * (uint64_t)(hi - lo + 1);
  }
  return cells;
}

}  // namespace mvg
