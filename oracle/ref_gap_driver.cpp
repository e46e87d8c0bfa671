// Test-only C entry point over the reference's own gap anchor search.
//
// Compiled with the reference sources (read in place, never copied) by
// oracle/Makefile.ref into oracle/_ref/libmauveref.so; used only to write the
// golden fixtures under tests/golden/.  Nothing shipped links it.
//
//   ref_gap_anchor_search -> the body of ProgressiveAligner::pairwiseAnchorSearch
//       (libMems/ProgressiveAligner.cpp:590-679) on two gap sequences that the
//       caller has already cut out of the genomes: seed weight
//       getDefaultSeedWeight of the mean gap length (return if below
//       MIN_DNA_SEED_WEIGHT), the rank-0 spaced seed, a DNAMemorySML per
//       sequence, MemHash::FindMatches, EliminateOverlaps_v2
//       (libMems/ProgressiveAligner.h:302-392) and LengthFilter(MIN_ANCHOR_LENGTH
//       + 3) (libMems/MatchList.h:680-692).  Coordinates stay those of the gap
//       sequences (1-based); the reference then adds the gap's left end - 1.
#include <cstdint>
#include <string>

#include "libGenome/gnSequence.h"
#include "libMems/DNAMemorySML.h"
#include "libMems/MatchList.h"
#include "libMems/MemHash.h"
#include "libMems/ProgressiveAligner.h"
#include "libMems/SeedMasks.h"

using namespace mems;
using namespace genome;

extern "C" {

// out: (start0, start1, length) per anchor in list order; returns the count,
// -1 if cap is too small, or -2 when the seed weight is below the minimum
// (the reference returns without searching).
int64_t ref_gap_anchor_search(const char* a, uint64_t la, const char* b, uint64_t lb, int64_t* out, uint64_t cap,
                              uint32_t* weight_out) {
  const gnSeqI avg_len = (la + lb) / 2;
  const uint w = getDefaultSeedWeight(avg_len);
  if (weight_out) *weight_out = w;
  if (w < MIN_DNA_SEED_WEIGHT) return -2;
  MatchList gap_list;
  gap_list.seq_table.push_back(la ? new gnSequence(std::string(a, la)) : new gnSequence());
  gap_list.seq_table.push_back(lb ? new gnSequence(std::string(b, lb)) : new gnSequence());
  for (int i = 0; i < 2; ++i) {
    DNAMemorySML* s = new DNAMemorySML();
    s->Create(*gap_list.seq_table[i], getSeed(w, 0));
    gap_list.sml_table.push_back(s);
  }
  MemHash mh;
  mh.Clear();
  mh.ClearSequences();
  mh.FindMatches(gap_list);
  EliminateOverlaps_v2(gap_list);
  gap_list.LengthFilter(MIN_ANCHOR_LENGTH + 3);
  int64_t r = (int64_t)gap_list.size();
  if ((uint64_t)r > cap) r = -1;
  for (size_t i = 0; r >= 0 && i < gap_list.size(); ++i) {
    out[3 * i + 0] = gap_list[i]->Start(0);
    out[3 * i + 1] = gap_list[i]->Start(1);
    out[3 * i + 2] = (int64_t)gap_list[i]->Length();
  }
  for (size_t i = 0; i < gap_list.size(); ++i) gap_list[i]->Free();
  mh.Clear();
  for (int i = 0; i < 2; ++i) {
    delete gap_list.sml_table[i];
    delete gap_list.seq_table[i];
  }
  return r;
}
}
