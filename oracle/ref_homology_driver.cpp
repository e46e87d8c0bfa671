// Test-only C entry points over the reference's own backbone-detection HMM.
//
// Compiled with the reference sources (read in place, never copied) by
// oracle/Makefile.ref into oracle/_ref/libmauveref.so; used only to write the
// golden fixtures under tests/golden/.  Nothing shipped links it.
//
//   ref_hmm_params -> the parameters applyBackbone sets up
//       (mauveAligner/src/progressiveMauve.cpp:226-238):
//       getAdaptedHoxdMatrixParameters(gc) (libMems/HomologyHMM/parameters.h),
//       the two transition overrides, adaptToPercentIdentity; out: the Params
//       members in declaration order (21 doubles).
//   ref_homologous_segments -> findHssHomologyHMM for one pairwise alignment
//       (libMems/Islands.h:122-196): column states, the HMM's forward and
//       backward passes and the posterior >= 0.9 decision
//       (libMems/HomologyHMM/homologymain.cc), and the homologous column
//       ranges; out: (left column, right column) pairs.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "libMems/HomologyHMM/parameters.h"
#include "libMems/Islands.h"

using namespace mems;

namespace {

void to_array(const Params& p, double* out) {
  out[0] = p.iStartHomologous;
  out[1] = p.iGoHomologous;
  out[2] = p.iGoUnrelated;
  out[3] = p.iGoStopFromUnrelated;
  out[4] = p.iGoStopFromHomologous;
  for (int k = 0; k < 8; ++k) out[5 + k] = p.aEmitHomologous[k];
  for (int k = 0; k < 8; ++k) out[13 + k] = p.aEmitUnrelated[k];
}

Params from_array(const double* in) {
  Params p;
  p.iStartHomologous = in[0];
  p.iGoHomologous = in[1];
  p.iGoUnrelated = in[2];
  p.iGoStopFromUnrelated = in[3];
  p.iGoStopFromHomologous = in[4];
  for (int k = 0; k < 8; ++k) p.aEmitHomologous[k] = in[5 + k];
  for (int k = 0; k < 8; ++k) p.aEmitUnrelated[k] = in[13 + k];
  return p;
}

}  // namespace

extern "C" {

void ref_hmm_params(double gc_content, double go_homologous, double go_unrelated, double pct_identity, double* out) {
  Params p = getAdaptedHoxdMatrixParameters(gc_content);
  p.iGoHomologous = go_homologous;
  p.iGoUnrelated = go_unrelated;
  adaptToPercentIdentity(p, pct_identity);
  to_array(p, out);
}

int64_t ref_homologous_segments(const char* row_a, const char* row_b, uint64_t ncols, const double* params,
                                int left_homologous, int right_homologous, int64_t* out, uint64_t cap) {
  std::vector<std::string> aln(2);
  aln[0] = std::string(row_a, ncols);
  aln[1] = std::string(row_b, ncols);
  hss_list_t hss;
  findHssHomologyHMM(aln, hss, 0, 1, from_array(params), left_homologous != 0, right_homologous != 0);
  if (hss.size() > cap) return -1;
  for (size_t i = 0; i < hss.size(); ++i) {
    out[2 * i] = (int64_t)hss[i].left_col;
    out[2 * i + 1] = (int64_t)hss[i].right_col;
  }
  return (int64_t)hss.size();
}
}
