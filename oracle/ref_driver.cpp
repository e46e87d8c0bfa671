// Test-only C entry points over the reference's own C++ classes.
//
// Compiled together with the reference sources (read in place, never copied)
// by oracle/Makefile.ref into oracle/_ref/libmauveref.so.  Used only to pin
// the CPU restatement in oracle/mauve_oracle.c and to generate the golden
// fixtures under tests/golden/; nothing shipped links it.
//
//   ref_sml_build        -> mems::DNAMemorySML::Create + Read
//                           (libMems/MemorySML.cpp:45-60, 62-84)
//   ref_pairwise_matches -> mems::PairwiseMatchFinder::FindMatches, as called
//                           by progressiveMauve (mauveAligner/src/progressiveMauve.cpp:500-503)
//   ref_profile_align    -> muscle::ProfileProfile with the DNA settings that
//                           MuscleInterface::ProfileAlignFast installs
//                           (libMems/MuscleInterface.cpp:1053-1112)
//   ref_sml_header_layout, ref_sml_file_image
//                        -> the SMLHeader struct (libMems/SortedMerList.h:48-63)
//                           and the header and packed sequence an SML holds
//                           after Create, which FileSML::Create writes
//                           (libMems/FileSML.cpp:401-459)
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <sstream>

#include "libGenome/gnSequence.h"
#include "libMems/SeedMasks.h"
#include "libMems/DNAMemorySML.h"
#include "libMems/MatchList.h"
#include "libMems/PairwiseMatchFinder.h"
#include "libMems/MemHash.h"
#include "libMUSCLE/muscle.h"
#include "libMUSCLE/msa.h"
#include "libMUSCLE/profile.h"
#include "libMUSCLE/params.h"

using namespace mems;
using namespace genome;

namespace muscle {
void ProfileProfile(MSA &msa1, MSA &msa2, MSA &msaOut);
void SetPPScore(PPSCORE p);
}

extern "C" {

unsigned ref_default_seed_weight(uint64_t avg_len) { return getDefaultSeedWeight(avg_len); }

uint64_t ref_get_seed(int weight, int rank) { return (uint64_t)getSeed(weight, rank); }

int ref_seed_length(uint64_t seed) { return getSeedLength((int64)seed); }
int ref_seed_weight(uint64_t seed) { return getSeedWeight((int64)seed); }

// Builds a DNAMemorySML over seq[0..len) with the given seed pattern and
// writes the sorted positions and the canonical seed mers that Read()
// recomputes for them.  Returns the SML length, or -1 if cap is too small.
int64_t ref_sml_build(const char* seq, uint64_t len, uint64_t seed,
                      uint32_t* pos_out, uint64_t* mer_out, uint64_t cap) {
  gnSequence gs(std::string(seq, len));
  DNAMemorySML sml;
  sml.Create(gs, seed);
  uint64_t n = sml.SMLLength();
  if (n > cap) return -1;
  std::vector<bmer> buf;
  uint64_t off = 0;
  while (off < n) {
    uint64_t want = std::min<uint64_t>(100000, n - off);
    sml.Read(buf, want, off);
    for (size_t i = 0; i < buf.size(); ++i) {
      pos_out[off + i] = buf[i].position;
      mer_out[off + i] = buf[i].mer;
    }
    off += buf.size();
    if (buf.empty()) break;
  }
  return (int64_t)n;
}

// sizeof(SMLHeader) then the offset of each member in declaration order
// (15 values).
int ref_sml_header_layout(int64_t* out) {
  out[0] = (int64_t)sizeof(SMLHeader);
  out[1] = (int64_t)offsetof(SMLHeader, version);
  out[2] = (int64_t)offsetof(SMLHeader, alphabet_bits);
  out[3] = (int64_t)offsetof(SMLHeader, seed);
  out[4] = (int64_t)offsetof(SMLHeader, seed_length);
  out[5] = (int64_t)offsetof(SMLHeader, seed_weight);
  out[6] = (int64_t)offsetof(SMLHeader, length);
  out[7] = (int64_t)offsetof(SMLHeader, unique_mers);
  out[8] = (int64_t)offsetof(SMLHeader, word_size);
  out[9] = (int64_t)offsetof(SMLHeader, little_endian);
  out[10] = (int64_t)offsetof(SMLHeader, id);
  out[11] = (int64_t)offsetof(SMLHeader, circular);
  out[12] = (int64_t)offsetof(SMLHeader, translation_table);
  out[13] = (int64_t)offsetof(SMLHeader, description);
  out[14] = (int64_t)(sizeof(((SMLHeader*)0)->translation_table));
  return 0;
}

namespace {
// Exposes the header and packed words an SML holds after Create.
struct SmlImage : public DNAMemorySML {
  const SMLHeader& hdr() const { return header; }
  const uint32* words() const { return sequence; }
  uint64_t nwords() const { return binary_seq_len; }
};
}  // namespace

// After DNAMemorySML::Create: the header (sizeof(SMLHeader) bytes; members
// the reference never sets are zeroed here) and the packed sequence words.
// Returns the number of words, or -1 if cap_words is too small.
int64_t ref_sml_file_image(const char* seq, uint64_t len, uint64_t seed, uint8_t* header_out, uint32_t* words_out,
                           uint64_t cap_words) {
  gnSequence gs(std::string(seq, len));
  SmlImage sml;
  sml.Create(gs, seed);
  SMLHeader h;
  memset(&h, 0, sizeof(h));
  const SMLHeader& r = sml.hdr();
  h.alphabet_bits = r.alphabet_bits;
  h.seed = r.seed;
  h.seed_length = r.seed_length;
  h.seed_weight = r.seed_weight;
  h.length = r.length;
  h.unique_mers = r.unique_mers;
  h.id = r.id;
  h.circular = r.circular;
  memcpy(h.translation_table, r.translation_table, sizeof(h.translation_table));
  h.description[0] = r.description[0];
  memcpy(header_out, &h, sizeof(h));
  if (sml.nwords() > cap_words) return -1;
  memcpy(words_out, sml.words(), sml.nwords() * 4);
  return (int64_t)sml.nwords();
}

// Canonical seed mer at every position, in position order (the unsorted fill).
int64_t ref_seed_mers(const char* seq, uint64_t len, uint64_t seed, uint64_t* mer_out, uint64_t cap) {
  gnSequence gs(std::string(seq, len));
  DNAMemorySML sml;
  sml.Create(gs, seed);
  uint64_t n = sml.SMLLength();
  if (n > cap) return -1;
  for (uint64_t p = 0; p < n; ++p) mer_out[p] = sml.GetSeedMer(p);
  return (int64_t)n;
}

static int64_t emit_matches(MatchList& ml, int64_t* out, uint64_t cap) {
  uint64_t n = ml.size();
  if (n > cap) return -1;
  for (uint64_t i = 0; i < n; ++i) {
    Match* m = ml[i];
    out[3 * i + 0] = m->Start(0);
    out[3 * i + 1] = m->Start(1);
    out[3 * i + 2] = (int64_t)m->Length();
  }
  return (int64_t)n;
}

// Genome-pair seed matching exactly as progressiveMauve's pairwise path runs it.
// out holds (start0, start1, length) per match: 1-based starts, a negative
// start marks the reverse strand.  Order is the reference's MatchList order.
int64_t ref_pairwise_matches(const char* a, uint64_t la, const char* b, uint64_t lb,
                             uint64_t seed, int64_t* out, uint64_t cap) {
  MatchList ml;
  ml.seq_table.push_back(new gnSequence(std::string(a, la)));
  ml.seq_table.push_back(new gnSequence(std::string(b, lb)));
  for (int i = 0; i < 2; ++i) {
    DNAMemorySML* s = new DNAMemorySML();
    s->Create(*ml.seq_table[i], seed);
    ml.sml_table.push_back(s);
  }
  PairwiseMatchFinder pmf;
  pmf.FindMatches(ml);
  int64_t r = emit_matches(ml, out, cap);
  for (size_t i = 0; i < ml.size(); ++i) ml[i]->Free();
  pmf.Clear();
  for (int i = 0; i < 2; ++i) { delete ml.sml_table[i]; delete ml.seq_table[i]; }
  return r;
}

// Gap-search seed matching: a plain MemHash over two in-memory SMLs, the
// way pairwiseAnchorSearch runs it (libMems/ProgressiveAligner.cpp:590-679)
// before its overlap and length filters.
int64_t ref_memhash_matches(const char* a, uint64_t la, const char* b, uint64_t lb,
                            uint64_t seed, int64_t* out, uint64_t cap) {
  MatchList ml;
  ml.seq_table.push_back(new gnSequence(std::string(a, la)));
  ml.seq_table.push_back(new gnSequence(std::string(b, lb)));
  for (int i = 0; i < 2; ++i) {
    DNAMemorySML* s = new DNAMemorySML();
    s->Create(*ml.seq_table[i], seed);
    ml.sml_table.push_back(s);
  }
  MemHash mh;
  mh.FindMatches(ml);
  int64_t r = emit_matches(ml, out, cap);
  for (size_t i = 0; i < ml.size(); ++i) ml[i]->Free();
  mh.Clear();
  for (int i = 0; i < 2; ++i) { delete ml.sml_table[i]; delete ml.seq_table[i]; }
  return r;
}

static void msa_from(muscle::MSA& msa, const char* s, int n, unsigned id) {
  msa.SetSize(1, n);
  msa.SetSeqName(0, id ? "seq1" : "seq0");
  msa.SetSeqId(0, id);
  for (int i = 0; i < n; ++i) msa.SetChar(0, i, s[i]);
}

// Profile-profile alignment of two single DNA sequences (no gap characters)
// through MUSCLE's NWSmall.  Writes the two aligned rows (with '-') and
// returns the column count, or -1 if cap is too small.
int ref_profile_align(const char* a, int la, const char* b, int lb,
                      char* outA, char* outB, int cap) {
  using namespace muscle;
  g_SeqType.get() = SEQTYPE_DNA;
  g_uMaxIters.get() = 1;
  g_bStable.get() = true;
  g_bQuiet.get() = true;
  g_SeqWeight1.get() = SEQWEIGHT_ClustalW;
  SetMaxIters(g_uMaxIters.get());
  SetSeqWeightMethod(g_SeqWeight1.get());
  MSA::SetIdCount(2);
  MSA m1, m2, mo;
  msa_from(m1, a, la, 0);
  msa_from(m2, b, lb, 1);
  SetAlpha(ALPHA_DNA);
  m1.FixAlpha();
  m2.FixAlpha();
  SetPPScore(PPSCORE_SPN);
  ProfileProfile(m1, m2, mo);
  int ncol = (int)mo.GetColCount();
  if (ncol > cap) return -1;
  // Rows are identified by the names given above, not by position.
  for (unsigned r = 0; r < mo.GetSeqCount(); ++r) {
    const char* buf = mo.GetSeqBuffer(r);
    char* dst = (strcmp(mo.GetSeqName(r), "seq0") == 0) ? outA : outB;
    memcpy(dst, buf, ncol);
  }
  return ncol;
}

}  // extern "C"
