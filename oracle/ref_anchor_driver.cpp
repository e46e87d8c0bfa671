// Test-only driver of the reference's own MUSCLE anchor-column search, for
// golden fixtures of mvg_anchor_ranges.  It sets MUSCLE up exactly as
// MuscleInterface::ProfileAlignFast does before AnchoredProfileProfile
// (libMems/MuscleInterface.cpp:1053-1109: DNA, one iteration, stable order,
// ClustalW weights, ALPHA_DNA, PPSCORE_SPN), builds one MSA per gapped row,
// and runs AnchoredProfileProfile's scoring preparation and anchor search
// (muscle/libMUSCLE/anchoredpp.cpp:429-458: PrepareMSAforScoring,
// FindAnchorColsPP).  Built only into oracle/_ref/libmauveref.so.
#include <string.h>

#include "libMUSCLE/muscle.h"
#include "libMUSCLE/msa.h"

namespace muscle {
void SetPPScore(PPSCORE p);
void PrepareMSAforScoring(MSA& msa);
void FindAnchorColsPP(const MSA& msa1, const MSA& msa2, unsigned AnchorCols[], unsigned* ptruAnchorColCount);
void AnchoredProfileProfile(MSA& msa1, MSA& msa2, MSA& msaOut);
}  // namespace muscle

static void row_msa(muscle::MSA& msa, const char* s, int n, unsigned id) {
  msa.SetSize(1, n);
  msa.SetSeqName(0, id ? "seq1" : "seq0");
  msa.SetSeqId(0, id);
  for (int i = 0; i < n; ++i) msa.SetChar(0, i, s[i]);
}

extern "C" {

static void setup_dna() {
  using namespace muscle;
  g_SeqType.get() = SEQTYPE_DNA;
  g_uMaxIters.get() = 1;
  g_bStable.get() = true;
  g_bQuiet.get() = true;
  g_SeqWeight1.get() = SEQWEIGHT_ClustalW;
  SetMaxIters(g_uMaxIters.get());
  SetSeqWeightMethod(g_SeqWeight1.get());
  MSA::SetIdCount(2);
}

// Anchor columns of two gapped rows of ncols columns (ascending); returns
// their number, or -1 if cap is too small.
int ref_anchor_cols(const char* row_a, const char* row_b, int ncols, unsigned* out, int cap) {
  using namespace muscle;
  setup_dna();
  MSA m1, m2;
  row_msa(m1, row_a, ncols, 0);
  row_msa(m2, row_b, ncols, 1);
  SetAlpha(ALPHA_DNA);
  m1.FixAlpha();
  m2.FixAlpha();
  SetPPScore(PPSCORE_SPN);
  PrepareMSAforScoring(m1);
  PrepareMSAforScoring(m2);
  unsigned* cols = new unsigned[ncols > 0 ? ncols : 1];
  unsigned n = 0;
  FindAnchorColsPP(m1, m2, cols, &n);
  int r = (int)n;
  if (r > cap) r = -1;
  else memcpy(out, cols, n * sizeof(unsigned));
  delete[] cols;
  return r;
}

// The whole anchored realignment of the window (ProfileAlignFast with
// anchored = true): writes the two output rows and returns their column
// count, or -1 if cap is too small.
int ref_anchored_align(const char* row_a, const char* row_b, int ncols, char* out_a, char* out_b, int cap) {
  using namespace muscle;
  setup_dna();
  MSA m1, m2, mo;
  row_msa(m1, row_a, ncols, 0);
  row_msa(m2, row_b, ncols, 1);
  SetAlpha(ALPHA_DNA);
  m1.FixAlpha();
  m2.FixAlpha();
  SetPPScore(PPSCORE_SPN);
  AnchoredProfileProfile(m1, m2, mo);
  const int n = (int)mo.GetColCount();
  if (n > cap) return -1;
  for (unsigned r = 0; r < mo.GetSeqCount(); ++r) {
    const char* buf = mo.GetSeqBuffer(r);
    memcpy(strcmp(mo.GetSeqName(r), "seq0") == 0 ? out_a : out_b, buf, n);
  }
  return n;
}

}  // extern "C"
