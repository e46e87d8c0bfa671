// Test-only C entry points over the reference's own ProgressiveAligner for
// one LCB of two genomes.
//
// Compiled with the reference sources (read in place, never copied) by
// oracle/Makefile.ref into oracle/_ref/libmauveref.so; used only to write the
// golden fixtures under tests/golden/.  Nothing shipped links it.
//
// The aligner gets a three-node guide tree (genome A, genome B, their
// ancestor, both edges aligned) and the LCB as a GappedAlignment of two rows.
//
//   ref_recurse_on_pairs -> ProgressiveAligner::recurseOnPairs
//       (libMems/ProgressiveAligner.cpp:682-924) on the LCB, as alignPP calls
//       it (:2450-2466) with an empty search cache: the anchors every
//       searched gap gives (pairwiseAnchorSearch, :590-679, appended gap by
//       gap) and the regions outside the LCB (iv_regions, :784-834).
//   ref_refine_alignment -> ProgressiveAligner::refineAlignment
//       (:1119-1230) as doGappedAlignment calls it: mode 0 = the
//       gapped-alignment pass (profile_aln = true, step 8 of
//       alignProfileToProfile, :2560-2565), 1 = the final iterative
//       refinement pass (profile_aln = false, :3750-3755), 2 = the first then
//       the second, as a two-genome progressiveMauve run does them.
//   ref_refine_fast -> MuscleInterface::RefineFast
//       (libMems/MuscleInterface.cpp:823-894) on one window.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "libGenome/gnSequence.h"
#include "libMems/CompactGappedAlignment.h"
#include "libMems/GappedAlignment.h"
#include "libMems/MuscleInterface.h"
#include "libMems/ProgressiveAligner.h"

using namespace mems;
using namespace genome;

namespace {

class TwoGenomeAligner : public ProgressiveAligner {
 public:
  TwoGenomeAligner(gnSequence* a, gnSequence* b) : ProgressiveAligner(2) {
    alignment_tree.nodes.resize(3);
    for (int k = 0; k < 3; ++k) {
      alignment_tree.nodes[k].sequence = NULL;
      alignment_tree.nodes[k].refined = false;
    }
    alignment_tree.nodes[0].sequence = a;
    alignment_tree.nodes[1].sequence = b;
    for (int k = 0; k < 2; ++k) {
      alignment_tree.nodes[k].parents.push_back(2);
      alignment_tree.nodes[k].parents_aligned.push_back(true);
      alignment_tree.nodes[2].children.push_back(k);
      alignment_tree.nodes[2].children_aligned.push_back(true);
    }
    alignment_tree.root = 2;
    node_sequence_map.assign(3, (uint)-1);
    node_sequence_map[0] = 0;
    node_sequence_map[1] = 1;
  }
};

// The LCB: rows of ncols columns, signed 1-based starts (negative = reverse).
GappedAlignment lcb(const char* row_a, const char* row_b, uint64_t ncols, int64_t start_a, int64_t start_b) {
  std::vector<std::string> rows(2);
  rows[0] = std::string(row_a, ncols);
  rows[1] = std::string(row_b, ncols);
  GappedAlignment ga(2, ncols);
  ga.SetAlignment(rows);
  const int64_t starts[2] = {start_a, start_b};
  for (int q = 0; q < 2; ++q) {
    int64_t n = 0;
    for (char ch : rows[q]) n += ch != '-';
    ga.SetStart(q, starts[q]);
    ga.SetLength(n, q);
  }
  return ga;
}

}  // namespace

extern "C" {

// out: anchors as (start 0, start 1, length); regions: the two iv_regions
// boundary lists, A's then B's, with their sizes in nregions[0..1].  Returns
// the anchor count, -1 when a buffer is too small.
int64_t ref_recurse_on_pairs(const char* seq_a, uint64_t la, const char* seq_b, uint64_t lb, const char* row_a,
                             const char* row_b, uint64_t ncols, int64_t start_a, int64_t start_b, uint64_t min_gap,
                             int64_t* out, uint64_t cap, int64_t* regions, uint64_t rcap, uint64_t* nregions) {
  gnSequence sa(std::string(seq_a, la)), sb(std::string(seq_b, lb));
  TwoGenomeAligner p(&sa, &sb);
  p.SetMinRecursionGapLength(min_gap);
  GappedAlignment ga = lcb(row_a, row_b, ncols, start_a, start_b);
  CompactGappedAlignment<> cga(ga);
  std::vector<node_id_t> n1(1, 0), n2(1, 1);
  Matrix<MatchList> matches;
  Matrix<std::vector<search_cache_t> > cache(1, 1), new_cache(1, 1);
  boost::multi_array<std::vector<std::vector<int64> >, 2> ivr(boost::extents[1][1]);
  ivr[0][0].resize(2);
  p.recurseOnPairs(n1, n2, cga, matches, cache, new_cache, ivr);
  MatchList& ml = matches(0, 0);
  int64_t r = (int64_t)ml.size();
  const std::vector<int64>& ra = ivr[0][0][0];
  const std::vector<int64>& rb = ivr[0][0][1];
  if ((uint64_t)r > cap || ra.size() + rb.size() > rcap) r = -1;
  for (size_t i = 0; r >= 0 && i < ml.size(); ++i) {
    out[3 * i] = ml[i]->Start(0);
    out[3 * i + 1] = ml[i]->Start(1);
    out[3 * i + 2] = (int64_t)ml[i]->Length();
  }
  if (r >= 0) {
    for (size_t i = 0; i < ra.size(); ++i) regions[i] = ra[i];
    for (size_t i = 0; i < rb.size(); ++i) regions[ra.size() + i] = rb[i];
    nregions[0] = ra.size();
    nregions[1] = rb.size();
  }
  for (size_t i = 0; i < ml.size(); ++i) ml[i]->Free();
  for (size_t i = 0; i < new_cache(0, 0).size(); ++i) {
    if (new_cache(0, 0)[i].first) new_cache(0, 0)[i].first->Free();
    if (new_cache(0, 0)[i].second) new_cache(0, 0)[i].second->Free();
  }
  return r;
}

static int64_t rows_out(GappedAlignment& gal, char* out_a, char* out_b, uint64_t cap) {
  const std::vector<std::string> rows = GetAlignment(gal, std::vector<gnSequence*>(2));
  const uint64_t n = rows[0].size();
  if (n > cap || rows[1].size() != n) return -1;
  std::memcpy(out_a, rows[0].data(), n);
  std::memcpy(out_b, rows[1].data(), n);
  return (int64_t)n;
}

// out_a / out_b: the refined rows; returns their length, -1 when cap is too
// small.
int64_t ref_refine_alignment(const char* row_a, const char* row_b, uint64_t ncols, int64_t start_a, int64_t start_b,
                             uint64_t max_window_size, int mode, char* out_a, char* out_b, uint64_t cap) {
  gnSequence sa, sb;  // leaves need a sequence; refineAlignment reads the rows only
  TwoGenomeAligner p(&sa, &sb);
  p.SetMaxGappedAlignmentLength(max_window_size);
  GappedAlignment gal = lcb(row_a, row_b, ncols, start_a, start_b);
  AlnProgressTracker apt;
  apt.total_len = ncols ? ncols : 1;
  apt.cur_leftend = 0;
  apt.prev_progress = 0;
  if (mode == 0 || mode == 2) p.refineAlignment(gal, 2, true, apt);
  if (mode == 1 || mode == 2) {
    apt.cur_leftend = 0;
    apt.prev_progress = 0;
    p.refineAlignment(gal, 2, false, apt);
  }
  return rows_out(gal, out_a, out_b, cap);
}

int64_t ref_refine_fast(const char* row_a, const char* row_b, uint64_t ncols, uint64_t windowsize, char* out_a,
                        char* out_b, uint64_t cap) {
  GappedAlignment gal = lcb(row_a, row_b, ncols, 1, 1);
  MuscleInterface::getMuscleInterface().RefineFast(gal, windowsize);
  return rows_out(gal, out_a, out_b, cap);
}
}
