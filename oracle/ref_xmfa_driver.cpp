// Test-only C entry point over the reference's own XMFA writer.
//
// Compiled with the reference sources (read in place, never copied) by
// oracle/Makefile.ref into oracle/_ref/libmauveref.so; used only to write the
// golden fixtures under tests/golden/.  Nothing shipped links it.
//
//   ref_xmfa_write -> GenericIntervalList::WriteStandardAlignment
//       (libMems/IntervalList.h:353-440) over two sequences and a list of
//       pairwise gapped blocks.  Each block is a GappedAlignment built from two
//       gap-patterned rows (any character = a base, '-' = a gap) and its two
//       signed starts (negative = reverse strand, 0 = absent); the writer
//       fills the rows from the sequences itself (GetAlignment,
//       libMems/AbstractGappedAlignment.h:84-103, reverse complement for the
//       reverse strand).
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "libGenome/gnSequence.h"
#include "libMems/GappedAlignment.h"
#include "libMems/IntervalList.h"

using namespace mems;
using namespace genome;

extern "C" {

// Returns the text length, or -1 if cap is too small (nothing written).
int64_t ref_xmfa_write(const char* seq_a, uint64_t la, const char* seq_b, uint64_t lb, const char* file_a,
                       const char* file_b, const char* backbone, int64_t nblocks, const int64_t* starts,
                       const uint64_t* col_off, const char* rows_a, const char* rows_b, char* out, uint64_t cap) {
  GenericIntervalList<GappedAlignment> iv_list;
  gnSequence sa(std::string(seq_a, la)), sb(std::string(seq_b, lb));
  iv_list.seq_table.push_back(&sa);
  iv_list.seq_table.push_back(&sb);
  iv_list.seq_filename.push_back(file_a);
  iv_list.seq_filename.push_back(file_b);
  iv_list.backbone_filename = backbone ? backbone : "";
  for (int64_t b = 0; b < nblocks; ++b) {
    const uint64_t c0 = col_off[b], c1 = col_off[b + 1];
    std::vector<std::string> rows(2);
    rows[0] = std::string(rows_a + c0, c1 - c0);
    rows[1] = std::string(rows_b + c0, c1 - c0);
    GappedAlignment ga(2, c1 - c0);
    ga.SetAlignment(rows);
    for (int q = 0; q < 2; ++q) {
      int64_t n = 0;
      for (char ch : rows[q]) n += ch != '-';
      ga.SetStart(q, starts[2 * b + q]);
      ga.SetLength(n, q);
    }
    iv_list.push_back(ga);
  }
  std::ostringstream os;
  iv_list.WriteStandardAlignment(os);
  const std::string text = os.str();
  iv_list.seq_table.clear();
  if (text.size() > cap) return -1;
  std::memcpy(out, text.data(), text.size());
  return (int64_t)text.size();
}
}
