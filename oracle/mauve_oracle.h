/* CPU oracle for the pairwise anchoring and gap-alignment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (each function cites the reference file:line it follows, paths
 * relative to the mauve-py source tree).  It is the checker for the CUDA
 * path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  The product library never links or calls it.
 *
 * Parity of this restatement is pinned against the reference's own C++ code
 * (compiled from its sources into oracle/_ref by oracle/Makefile.ref) through
 * the golden fixtures in tests/golden/.
 */
#ifndef MAUVE_ORACLE_H
#define MAUVE_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Seed patterns and default weights (libMems/SeedMasks.h). */
uint64_t mo_get_seed(int weight, int rank);
int mo_seed_length(uint64_t seed);
int mo_seed_weight(uint64_t seed);
unsigned mo_default_seed_weight(uint64_t avg_len);

/* 2-bit MSB-first packing into uint32 words, plus two zero pad words
 * (SortedMerList::translate32 / SetSequence).  out needs n/16 + 3 words.
 * Returns the word count written, or -1 on a '-' gap character. */
int64_t mo_pack(const uint8_t* seq, uint64_t n, uint32_t* out);

/* Canonical seed mer at every position p in [0, n-L] (GetDnaSeedMer).  */
int64_t mo_seed_mers(const uint8_t* seq, uint64_t n, uint64_t seed, uint64_t* mer_out);

/* Sorted mer list: positions sorted by canonical mer, ties by position. */
int64_t mo_sml_build(const uint8_t* seq, uint64_t n, uint64_t seed, uint32_t* pos_out, uint64_t* mer_out);

/* Genome-pair match finding (PairwiseMatchFinder::FindMatches).  out holds
 * (start0, start1, length) per match in the reference's MatchList order,
 * 1-based starts, negative start1 = reverse strand.  Returns the match count,
 * -1 if cap is too small, -2 on bad input. */
int64_t mo_pairwise_matches(const uint8_t* a, uint64_t na, const uint8_t* b, uint64_t nb,
                            uint64_t seed, int64_t* out, uint64_t cap);

/* Gap anchor search (oracle/gap_oracle.cpp): pairwiseAnchorSearch
 * (libMems/ProgressiveAligner.cpp:590-679) on two gap sequences.
 * mo_gap_anchor_filter applies EliminateOverlaps_v2 and LengthFilter(12) in
 * place to (start0, start1, length) rows and returns the count kept;
 * mo_gap_anchor_search runs the seed matching first (-2: seed weight below
 * the minimum, no search; -1: cap too small). */
int64_t mo_gap_anchor_filter(int64_t* rows, int64_t n);
int64_t mo_gap_anchor_search(const uint8_t* a, uint64_t la, const uint8_t* b, uint64_t lb, int64_t* out,
                             uint64_t cap, uint32_t* weight);

/* Same, stopping after the join: the unique seed pairs in processing order
 * (posA, posB, canonical-mer parity bits), for checking the join kernel. */
int64_t mo_unique_pairs(const uint8_t* a, uint64_t na, const uint8_t* b, uint64_t nb,
                        uint64_t seed, uint32_t* pa, uint32_t* pb, uint64_t cap);

/* Gap DP (muscle NWSmall + BitTraceBack for two single DNA sequences with
 * MUSCLE's DNA defaults).  a, b are base codes 0..3 (A,C,G,T).  Writes the
 * path as edge letters 'M','D','I' from the first column to the last and
 * returns its length; *score gets max(M,D,I) at (LA,LB).  -1 on bad input. */
int64_t mo_nw_align(const uint8_t* a, int la, const uint8_t* b, int lb, char* path, int32_t* score);

/* Score only (no traceback), same recurrences. */
int32_t mo_nw_score(const uint8_t* a, int la, const uint8_t* b, int lb);

/* Batch of independent problems, parallel over problems with nthreads
 * host threads (0 = all).  Sequences are concatenated; off_a/off_b hold
 * nprob+1 offsets.  Paths are written at path_off[p] (sum of la+lb bound).
 * Used as the CPU baseline. */
int64_t mo_nw_batch(const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                    const uint64_t* off_b, int64_t nprob, char* paths, const uint64_t* path_off,
                    int64_t* path_len, int32_t* scores, int nthreads);

/* Index LUT (oracle/lut_oracle.c).  Genome -> reference LUT built from
 * aligned blocks (buildindex.py:112-130) and the indexutils.pyx passes.
 * Blocks: columns [col_off[b], col_off[b+1]) of the two gapped rows, start
 * indices as the XMFA parse gives them.  -2 = IndexError, -3 = overflow. */
int64_t mo_lut_from_blocks(const int64_t* g_start, const int64_t* r_start, const uint64_t* col_off,
                           const uint8_t* g_rows, const uint8_t* r_rows, uint64_t nblocks,
                           int32_t* lut, uint64_t n);
int mo_fix_zero_idx(int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t glen,
                    const uint8_t* ref, uint64_t rlen);
void mo_fill_gaps(int32_t* lut, uint64_t n, int max_gap_width);
void mo_smooth_edges(int32_t* lut, uint64_t n, int smoothing_radius);
void mo_find_gaps(int32_t* lut, uint64_t n, int32_t* gaps);
void mo_find_edges(const int32_t* lut, uint64_t n, uint8_t* edges);
int mo_find_mismatches(const int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t glen,
                       const uint8_t* ref, uint64_t rlen, uint8_t* mism);
int64_t mo_find_duplicate_mappings(const int32_t* lut, uint64_t n, uint32_t* counts, uint64_t ncounts);

#ifdef __cplusplus
}
#endif
#endif
