// Test-only C entry point over the reference's own LCB computation with
// greedy breakpoint elimination for collinear genomes.
//
// Compiled with the reference sources (read in place, never copied) by
// oracle/Makefile.ref into oracle/_ref/libmauveref.so; used only to write the
// golden fixtures under tests/golden/.  Nothing shipped links it.
//
//   ref_collinear_lcbs -> the collinear branch of
//       ProgressiveAligner::alignProfileToProfile
//       (libMems/ProgressiveAligner.cpp:2281-2303): IdentifyBreakpoints,
//       ComputeLCBs_v2, SimpleGetLCBCoverage weights, the breakpoint penalty
//       100 + their sum, computeLCBAdjacencies_v3, a collinear
//       SimpleBreakpointScorer, greedyBreakpointElimination_v4 and
//       filterMatches_v2.
// Match lists cross this interface as (start 0, start 1, length) int64
// triples: libMems' signed 1-based starts.  The LCBs come back concatenated
// with their offsets, then the matches the elimination deleted.
#include <cstdint>
#include <vector>

#include "libMems/GreedyBreakpointElimination.h"
#include "libMems/Match.h"
#include "libMems/ProgressiveAligner.h"

using namespace mems;
using namespace genome;

extern "C" int ref_collinear_lcbs(const int64_t* m, uint64_t n, int64_t* out, uint64_t* lcb_off, uint64_t lcb_cap,
                                  uint64_t* nlcb, int64_t* deleted, uint64_t* ndeleted) {
  std::vector<AbstractMatch*> ancestral_matches;
  for (uint64_t i = 0; i < n; ++i) {
    Match x(2);
    x.SetStart(0, m[3 * i]);
    x.SetStart(1, m[3 * i + 1]);
    x.SetLength((gnSeqI)m[3 * i + 2]);
    ancestral_matches.push_back(x.Copy());
  }
  std::vector<gnSeqI> breakpoints;
  std::vector<std::vector<AbstractMatch*> > LCB_list;
  std::vector<LCB> adjacencies;
  IdentifyBreakpoints(ancestral_matches, breakpoints);
  ComputeLCBs_v2(ancestral_matches, breakpoints, LCB_list);
  std::vector<double> lcb_scores(LCB_list.size());
  double score_sum = 100;
  for (size_t lcbI = 0; lcbI < LCB_list.size(); ++lcbI) {
    lcb_scores[lcbI] = SimpleGetLCBCoverage(LCB_list[lcbI]);
    score_sum += lcb_scores[lcbI];
  }
  computeLCBAdjacencies_v3(LCB_list, lcb_scores, adjacencies);
  SimpleBreakpointScorer wbs(adjacencies, score_sum, true);
  greedyBreakpointElimination_v4(adjacencies, lcb_scores, wbs, NULL, false);
  std::vector<AbstractMatch*> deleted_matches;
  filterMatches_v2(adjacencies, LCB_list, lcb_scores, deleted_matches);

  int rc = 0;
  *nlcb = LCB_list.size();
  if (LCB_list.size() + 1 > lcb_cap) rc = -1;
  uint64_t at = 0;
  if (rc == 0) lcb_off[0] = 0;
  for (size_t k = 0; k < LCB_list.size(); ++k) {
    for (AbstractMatch* x : LCB_list[k]) {
      if (rc == 0) {
        out[3 * at] = x->Start(0);
        out[3 * at + 1] = x->Start(1);
        out[3 * at + 2] = (int64_t)x->Length(0);
      }
      ++at;
      x->Free();
    }
    if (rc == 0) lcb_off[k + 1] = at;
  }
  *ndeleted = deleted_matches.size();
  for (size_t i = 0; i < deleted_matches.size(); ++i) {
    deleted[3 * i] = deleted_matches[i]->Start(0);
    deleted[3 * i + 1] = deleted_matches[i]->Start(1);
    deleted[3 * i + 2] = (int64_t)deleted_matches[i]->Length(0);
    deleted_matches[i]->Free();
  }
  return rc;
}
