// CPU restatement of the reference's gap anchor search (the part after the
// seed matching).  TEST INFRASTRUCTURE ONLY: the checker for the CUDA path,
// loaded by tests/ and bench.py's CPU legs through oracle.py; the product
// library never links it.  Pinned against the reference's own code through
// tests/golden/gapsearch.npz.
//
// ProgressiveAligner::pairwiseAnchorSearch (libMems/ProgressiveAligner.cpp:590-679)
// on two gap sequences: seed weight getDefaultSeedWeight of the mean gap
// length, return if below MIN_DNA_SEED_WEIGHT = 5 (libMems/SeedMasks.h:375),
// MemHash matches with the rank-0 seed (the pairwise matcher's list, pinned
// equal), EliminateOverlaps_v2 (libMems/ProgressiveAligner.h:302-392),
// LengthFilter(MIN_ANCHOR_LENGTH + 3 = 12) (libMems/MatchList.h:680-692,
// libMems/Aligner.h:266).  C++ because EliminateOverlaps_v2 orders the list
// with std::sort, whose order among equal left ends is the library's: the
// same call on the same input gives the same order.
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "mauve_oracle.h"

namespace {

struct Anchor {
  int64_t s[2];  // 1-based starts, negative = reverse strand
  int64_t len;
};

int64_t left_end(const Anchor& m, int q) { return m.s[q] < 0 ? -m.s[q] : m.s[q]; }

// UngappedLocalAlignment::CropStart / CropEnd over HybridAbstractMatch's
// MoveStart / MoveEnd (libMems/UngappedLocalAlignment.h:137-152,
// libMems/HybridAbstractMatch.h:271-290): forward starts move with the
// alignment's first column, reverse starts with its last.
void crop_start(Anchor& m, int64_t n) {
  m.len -= n;
  for (int q = 0; q < 2; ++q)
    if (m.s[q] > 0) m.s[q] += n;
}
void crop_end(Anchor& m, int64_t n) {
  m.len -= n;
  for (int q = 0; q < 2; ++q)
    if (m.s[q] < 0) m.s[q] -= n;
}
// CropLeft / CropRight in sequence q's coordinates (:169-184)
void crop_left(Anchor& m, int64_t n, int q) { m.s[q] > 0 ? crop_start(m, n) : crop_end(m, n); }
void crop_right(Anchor& m, int64_t n, int q) { m.s[q] > 0 ? crop_end(m, n) : crop_start(m, n); }

// EliminateOverlaps_v2 with eliminate_both = false for two-sequence
// matches: every match is defined in both sequences (multiplicity 2), so the
// cropped-off copies processNewMatch receives have multiplicity 1 and are
// dropped; only the crops and deletions remain.
void eliminate_overlaps(std::vector<Anchor*>& ml) {
  if (ml.size() < 2) return;
  for (int q = 0; q < 2; ++q) {
    std::sort(ml.begin(), ml.end(), [q](const Anchor* a, const Anchor* b) { return left_end(*a, q) < left_end(*b, q); });
    int64_t deleted = 0;
    const int64_t n = (int64_t)ml.size();
    for (int64_t i = 0; i < n; ++i) {
      if (!ml[i]) continue;
      for (int64_t j = i + 1; j < n; ++j) {
        if (!ml[j]) continue;
        const int64_t len_i = ml[i]->len;
        int64_t diff = left_end(*ml[j], q) - left_end(*ml[i], q) - len_i;
        if (diff >= 0) break;  // no more overlaps with match i
        diff = -diff;
        bool deleted_i = false;
        if (ml[j]->len > len_i) {  // match i is the smaller one: crop or delete it
          if (diff >= len_i) {
            ml[i] = nullptr;
            --i;
            deleted_i = true;
            ++deleted;
          } else {
            crop_right(*ml[i], diff, q);
          }
        } else {  // match j is: crop or delete it
          if (diff >= ml[j]->len) {
            ml[j] = nullptr;
            ++deleted;
          } else {
            crop_left(*ml[j], diff, q);
          }
        }
        if (deleted_i) break;
      }
    }
    if (deleted) {
      size_t cur = 0;
      for (size_t k = 0; k < ml.size(); ++k)
        if (ml[k]) ml[cur++] = ml[k];
      ml.resize(cur);
    }
  }
}

}  // namespace

extern "C" {

// In place on n (start0, start1, length) rows in list order: the overlap
// elimination and the length filter.  Returns the surviving count.
int64_t mo_gap_anchor_filter(int64_t* rows, int64_t n) {
  std::vector<Anchor> store((size_t)n);
  std::vector<Anchor*> ml((size_t)n);
  for (int64_t k = 0; k < n; ++k) {
    store[k] = Anchor{{rows[3 * k], rows[3 * k + 1]}, rows[3 * k + 2]};
    ml[k] = &store[k];
  }
  eliminate_overlaps(ml);
  int64_t out = 0;
  for (const Anchor* m : ml) {
    if (m->len < 12) continue;
    rows[3 * out + 0] = m->s[0];
    rows[3 * out + 1] = m->s[1];
    rows[3 * out + 2] = m->len;
    ++out;
  }
  return out;
}

// The whole gap anchor search on two gap sequences (ASCII).  Returns the
// anchor count, -1 if cap is too small, -2 if the gap's seed weight is below
// the minimum (no search).  *weight gets the weight used.
int64_t mo_gap_anchor_search(const uint8_t* a, uint64_t la, const uint8_t* b, uint64_t lb, int64_t* out,
                             uint64_t cap, uint32_t* weight) {
  const unsigned w = mo_default_seed_weight((la + lb) / 2);
  if (weight) *weight = w;
  if (w < 5) return -2;
  const uint64_t mcap = (la < lb ? la : lb) + 16;
  std::vector<int64_t> m(3 * mcap);
  const int64_t n = mo_pairwise_matches(a, la, b, lb, mo_get_seed((int)w, 0), m.data(), mcap);
  if (n < 0) return n;
  const int64_t k = mo_gap_anchor_filter(m.data(), n);
  if ((uint64_t)k > cap) return -1;
  std::copy(m.begin(), m.begin() + 3 * k, out);
  return k;
}
}
