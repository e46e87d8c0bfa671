// Test-only C entry points over the reference's own search outside LCBs.
//
// Compiled with the reference sources (read in place, never copied) by
// oracle/Makefile.ref into oracle/_ref/libmauveref.so; used only to write the
// golden fixtures under tests/golden/.  Nothing shipped links it.
//
//   ref_search_lcb_gaps -> SearchLCBGaps (libMems/Aligner.cpp:784-928) for
//       two genomes, as ProgressiveAligner::alignPP calls it
//       (libMems/ProgressiveAligner.cpp:2474-2488) with a fresh MaskedMemHash:
//       the regions are concatenated, searched with the rank-0 seed of
//       getDefaultSeedWeight of their mean length, and the matches are
//       transposed back, overlap-eliminated and filtered.
//   ref_gap_concat_matches -> the match list SearchLCBGaps builds before
//       transposing (MaskedMemHash::FindMatches over the concatenations,
//       MultiplicityFilter(2)), in the concatenations' coordinates.
//   ref_transpose_matches -> transposeMatches (libMems/Aligner.cpp:973-1045)
//       for one sequence of a two-genome match list.
//   ref_eliminate_overlaps -> EliminateOverlaps (libMems/Aligner.cpp:62-176).
//   ref_lcb_gap_finish -> the steps after the search: transposeMatches for
//       both genomes, EliminateOverlaps, MultiplicityFilter(2),
//       LengthFilter(MIN_ANCHOR_LENGTH) (libMems/Aligner.cpp:910-923).
// Match lists cross this interface as (start 0, start 1, length) int64
// triples: libMems' signed 1-based starts, 0 for a sequence without the match.
#include <cstdint>
#include <string>
#include <vector>

#include "libGenome/gnSequence.h"
#include "libMems/Aligner.h"
#include "libMems/DNAMemorySML.h"
#include "libMems/MaskedMemHash.h"
#include "libMems/MatchList.h"
#include "libMems/SeedMasks.h"

using namespace mems;
using namespace genome;

namespace {

void load(MatchList& ml, const int64_t* m, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    Match x(2);
    if (m[3 * i]) x.SetStart(0, m[3 * i]);
    if (m[3 * i + 1]) x.SetStart(1, m[3 * i + 1]);
    x.SetLength((gnSeqI)m[3 * i + 2]);
    ml.push_back(x.Copy());
  }
}

int64_t store(MatchList& ml, int64_t* out, uint64_t cap) {
  int64_t r = (int64_t)ml.size();
  if ((uint64_t)r > cap) r = -1;
  for (size_t i = 0; r >= 0 && i < ml.size(); ++i) {
    out[3 * i + 0] = ml[i]->Start(0);
    out[3 * i + 1] = ml[i]->Start(1);
    out[3 * i + 2] = (int64_t)ml[i]->Length();
  }
  for (size_t i = 0; i < ml.size(); ++i) ml[i]->Free();
  ml.clear();
  return r;
}

std::vector<int64> regions(const int64_t* r, uint64_t n) { return std::vector<int64>(r, r + n); }

}  // namespace

extern "C" {

// The external-sort fallback SearchLCBGaps takes only when a memory SML
// cannot be built; it is not compiled here, and this stand-in reports
// failure if it were ever reached.
int dmSML(const char*, const char*, const char* const*, unsigned long long) { return -1; }

int64_t ref_search_lcb_gaps(const char* a, uint64_t la, const char* b, uint64_t lb, const int64_t* ra, uint64_t nra,
                            const int64_t* rb, uint64_t nrb, int64_t* out, uint64_t cap) {
  gnSequence* sa = la ? new gnSequence(std::string(a, la)) : new gnSequence();
  gnSequence* sb = lb ? new gnSequence(std::string(b, lb)) : new gnSequence();
  MatchList ml;
  ml.seq_table.push_back(sa);
  ml.seq_table.push_back(sb);
  std::vector<std::vector<int64> > iv(2);
  iv[0] = regions(ra, nra);
  iv[1] = regions(rb, nrb);
  MaskedMemHash nway_mh;
  SearchLCBGaps(ml, iv, nway_mh);
  const int64_t r = store(ml, out, cap);
  delete sa;
  delete sb;
  return r;
}

int64_t ref_gap_concat_matches(const char* a, uint64_t la, const char* b, uint64_t lb, int64_t* out, uint64_t cap,
                               uint32_t* weight_out) {
  const gnSeqI total = (la + lb) / 2;
  const uint w = getDefaultSeedWeight(total);
  if (weight_out) *weight_out = w;
  if (w < MIN_DNA_SEED_WEIGHT) return -2;
  MatchList gl;
  gl.seq_table.push_back(la ? new gnSequence(std::string(a, la)) : new gnSequence());
  gl.seq_table.push_back(lb ? new gnSequence(std::string(b, lb)) : new gnSequence());
  for (int i = 0; i < 2; ++i) {
    DNAMemorySML* s = new DNAMemorySML();
    s->Create(*gl.seq_table[i], getSeed(w));
    gl.sml_table.push_back(s);
  }
  MaskedMemHash mh;
  mh.Clear();
  mh.FindMatches(gl);
  gl.MultiplicityFilter(2);
  for (int i = 0; i < 2; ++i) {
    gl.sml_table[i]->Clear();
    delete gl.sml_table[i];
    delete gl.seq_table[i];
  }
  return store(gl, out, cap);
}

int64_t ref_transpose_matches(const int64_t* m, uint64_t n, unsigned seq, const int64_t* reg, uint64_t nreg, int64_t* out,
                              uint64_t cap) {
  MatchList ml;
  load(ml, m, n);
  transposeMatches(ml, seq, regions(reg, nreg));
  return store(ml, out, cap);
}

int64_t ref_eliminate_overlaps(const int64_t* m, uint64_t n, int64_t* out, uint64_t cap) {
  MatchList ml;
  load(ml, m, n);
  EliminateOverlaps(ml);
  return store(ml, out, cap);
}

int64_t ref_lcb_gap_finish(const int64_t* m, uint64_t n, const int64_t* ra, uint64_t nra, const int64_t* rb,
                           uint64_t nrb, int64_t* out, uint64_t cap) {
  MatchList ml;
  load(ml, m, n);
  transposeMatches(ml, 0, regions(ra, nra));
  transposeMatches(ml, 1, regions(rb, nrb));
  EliminateOverlaps(ml);
  ml.MultiplicityFilter(2);
  ml.LengthFilter(MIN_ANCHOR_LENGTH);
  return store(ml, out, cap);
}
}
