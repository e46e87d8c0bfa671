/* mauve_gb300.h -- C ABI of the GB300 (sm_103a) pairwise anchoring and
 * gap-alignment path of progressiveMauve.
 *
 * Plain C: POD pointers and sizes, an explicit CUDA stream passed as void*,
 * integer status returns (0 = ok), no exceptions across the boundary.  The
 * caller owns every input and output buffer; the library owns its device
 * workspaces through an opaque handle.  Functions whose name ends in _dev
 * take device pointers; the others take host pointers and do their own
 * host<->device copies on the handle's stream.
 *
 * Reference citations are file:line within the mauve-py tree
 * (LM/ = mauve/src/libMems/libMems/, MU/ = mauve/src/muscle/libMUSCLE/).
 */
#ifndef MAUVE_GB300_H
#define MAUVE_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define MVG_OK 0
#define MVG_ERR_ARG 1        /* invalid argument (null pointer, bad length, bad seed) */
#define MVG_ERR_CUDA 2       /* a CUDA runtime call failed; see mvg_last_error() */
#define MVG_ERR_GAP_CHAR 3   /* '-' in a genome sequence (LM/SortedMerList.cpp:433-437 throws) */
#define MVG_ERR_BAD_BASE 4   /* gap-DP input code outside 0..3 */
#define MVG_ERR_CAPACITY 5   /* caller's output buffer or a size limit is too small */
#define MVG_ERR_NOMEM 6      /* device allocation failed */
#define MVG_ERR_DEVICE 7     /* a kernel reported an internal error (watchdog, bound) */
#define MVG_ERR_RANGE 8      /* index outside the LUT or a sequence (the reference raises IndexError) */
#define MVG_ERR_OVERFLOW 9   /* a LUT value does not fit int32 (numpy raises OverflowError) */

typedef struct mvg_context* mvg_handle;

/* Creates a handle bound to CUDA device `device` with its own stream.
 * Replaces nothing in the reference (which keeps no device state). */
int mvg_create(mvg_handle* out, int device);
int mvg_destroy(mvg_handle h);
/* Human-readable description of the last error on this thread. */
const char* mvg_last_error(void);
/* The handle's CUDA stream (cudaStream_t as void*). */
void* mvg_stream(mvg_handle h);
/* Number of this library's kernels launched through the handle so far. */
uint64_t mvg_kernel_launches(mvg_handle h);

/* ---------------------------------------------------------------- seeds */

/* getSeed(weight, rank) -- LM/SeedMasks.h:298-321 (pattern tables 44-260). */
uint64_t mvg_get_seed(int weight, int rank);
/* getDefaultSeedWeight -- LM/SeedMasks.h:389-401. */
unsigned mvg_default_seed_weight(uint64_t avg_len);
/* getSeedLength / getSeedWeight -- LM/SeedMasks.h:334-371. */
int mvg_seed_length(uint64_t seed);
int mvg_seed_weight(uint64_t seed);

/* Sorted mer list construction: 2-bit packing (translate32,
 * LM/SortedMerList.cpp:425-459), canonical spaced-seed mer per position
 * (GetDnaSeedMer, :726-769; FillDnaSeedSML :771-784 / FillDnaSML :617-724)
 * and the sort by mer (std::sort(bmer_lessthan), LM/MemorySML.cpp:45-60,
 * LM/FileSML.cpp:429).  Replaces SortedMerList::Create (LM/SortedMerList.h:89).
 * seq: n ASCII bases.  Writes n-L+1 positions sorted by canonical mer (ties
 * by ascending position) and, if mer_out is not NULL, the canonical mers in
 * the same order.  *count gets n-L+1 (0 if n < L). */
int mvg_sml_build(mvg_handle h, const uint8_t* seq, uint64_t n, uint64_t seed,
                  uint32_t* pos_out, uint64_t* mer_out, uint64_t cap, uint64_t* count);
int mvg_sml_build_dev(mvg_handle h, const uint8_t* d_seq, uint64_t n, uint64_t seed,
                      uint32_t* d_pos_out, uint64_t* d_mer_out, uint64_t cap, uint64_t* count);

/* Sorted mer list build that allocates no device memory.  No counterpart in
 * the reference.  Some callers cannot call cudaMalloc when they need a sorted
 * mer list.  One example is a process whose other runtime reserved the
 * device's memory for its own pool up front.  Another is a latency-bound
 * loop that cannot take cudaMalloc's implicit device-wide synchronisation.
 * This call needs no handle.  It takes device input/output pointers like
 * mvg_sml_build_dev and a CUDA stream (void*, NULL = default stream).  It
 * produces the same output.  Its scratch is one static device array of
 * about 6.3 MB that every GPU loading the library holds until exit, which
 * limits n to 262,144 bases; longer input returns MVG_ERR_CAPACITY.  The first
 * call on a device looks up that array's device address (with the device
 * current) and uploads the base table, so make it before any stream capture;
 * a call with n = 0 does only that set-up.  Under CUDA's default lazy module
 * loading that first look-up is also when the array's device memory is
 * committed, so a caller about to give the rest of the device to another
 * allocator makes its first call before doing so.  The set-up is repeated
 * when the current context changes (after cudaDeviceReset).  All calls share
 * the array: calls whose GPU work overlaps (other streams or host threads)
 * race and must be serialised by the caller. */
int mvg_sml_build_noalloc(const uint8_t* d_seq, uint64_t n, uint64_t seed, uint32_t* d_pos_out,
                          uint64_t* d_mer_out, uint64_t cap, uint64_t* count, void* stream);

/* --------------------------------------------------------------- matches */

/* Pairwise seed matching and maximal-match extension for two genomes:
 * PairwiseMatchFinder::FindMatches as progressiveMauve calls it
 * (MA/progressiveMauve.cpp:500-503): SearchRange (LM/MatchFinder.cpp:172-340),
 * unique-seed enumeration (LM/PairwiseMatchFinder.cpp:37-71), HashMatch /
 * SetDirection / CalculateOffset / AddHashEntry (LM/MemHash.cpp:167-251),
 * ExtendMatch (LM/MatchFinder.h:218-374) and GetMatchList order
 * (LM/MemHash.h:182-203).  Replaces MemHash::FindMatches(MatchList&)
 * (LM/MemHash.h:55).
 * out receives 3 int64 per match: start in A, start in B (1-based; a
 * negative B start means the reverse strand) and length, in the reference's
 * MatchList order.  *count gets the number of matches; MVG_ERR_CAPACITY if
 * it exceeds cap (then *count still holds the needed size). */
int mvg_pairwise_matches(mvg_handle h, const uint8_t* seq_a, uint64_t na, const uint8_t* seq_b,
                         uint64_t nb, uint64_t seed, int64_t* out, uint64_t cap, uint64_t* count);
int mvg_pairwise_matches_dev(mvg_handle h, const uint8_t* d_seq_a, uint64_t na, const uint8_t* d_seq_b,
                             uint64_t nb, uint64_t seed, int64_t* d_out, uint64_t cap, uint64_t* count);

/* Match-finding statistics of the last mvg_pairwise_matches* call on h:
 * stats[0] = unique seed pairs hashed, [1] = collisions (contained seeds),
 * [2] = matches, [3] = non-empty hash buckets. */
int mvg_pairwise_stats(mvg_handle h, uint64_t stats[4]);

/* Batched gap anchor search: ProgressiveAligner::pairwiseAnchorSearch
 * (LM/ProgressiveAligner.cpp:590-679) for many inter-anchor gaps in one call,
 * as recurseOnPairs (:682-924) issues it for every gap of a recursion round.
 * gaps holds 4 int64 per gap: start in A (0-based), length in A, start in
 * B, length in B -- the subsequences the reference cuts out (ToString(diff,
 * gap_start), :600-611).  Per gap: seed weight getDefaultSeedWeight of the
 * mean length (LM/SeedMasks.h:389-401; below 5 the gap is not searched),
 * the rank-0 seed, MemHash::FindMatches over the two gap sequences,
 * EliminateOverlaps_v2 (LM/ProgressiveAligner.h:302-392) and
 * LengthFilter(12) (LM/MatchList.h:680-692), coordinates shifted to the
 * genomes (:657-665).  out receives 3 int64 per anchor (start in A, start
 * in B, 1-based genome coordinates, negative = reverse strand; length), the
 * anchors of gap g at rows gap_off[g] .. gap_off[g+1]-1 (gap_off has
 * ngaps+1 entries) in the reference's list order.  *count gets the total;
 * MVG_ERR_CAPACITY if it exceeds cap (gap_off and *count are still set),
 * MVG_ERR_RANGE for a gap outside its genome, MVG_ERR_ARG for a gap whose
 * mean length needs a seed weight above 15 (above about 5.9 Mbp: search
 * such a gap with mvg_pairwise_matches and the rank-0 seed). */
int mvg_gap_anchor_search(mvg_handle h, const uint8_t* seq_a, uint64_t na, const uint8_t* seq_b, uint64_t nb,
                          const int64_t* gaps, uint64_t ngaps, int64_t* out, uint64_t cap, uint64_t* gap_off,
                          uint64_t* count);
/* The same with the genomes in device memory (gaps and outputs on the host). */
int mvg_gap_anchor_search_dev(mvg_handle h, const uint8_t* d_seq_a, uint64_t na, const uint8_t* d_seq_b,
                              uint64_t nb, const int64_t* gaps, uint64_t ngaps, int64_t* out, uint64_t cap,
                              uint64_t* gap_off, uint64_t* count);

/* The seed join groups both genomes' seeds into buckets by the mer's top
 * bits and sorts each bucket in shared memory when it holds at most cap
 * seeds, else in chunks through global memory.  cap in 32..3072 (default
 * 3072); the matches do not depend on it. */
int mvg_set_pair_bucket_cap(mvg_handle h, int cap);

/* ---------------------------------------------------------------- gap DP */

/* Batched global gap alignment: for each problem p, muscle NWSmall
 * (MU/nwsmall.cpp:500-670) on two single-sequence DNA profiles built with
 * MUSCLE's DNA defaults (NUC_SP + 60, MU/nucmx.cpp:8-25; gap open -400 split
 * into -200 open / -200 close, MU/profilefrommsa.cpp:291-292; extend 0;
 * TERMGAPS_Half, MU/termgaps.cpp:6-38), then BitTraceBack
 * (MU/bittraceback.cpp:138-210).  Replaces muscle::GlobalAlign
 * (MU/glbalign.cpp:69) per range.
 * seq_a / seq_b: concatenated base codes 0..3 (A,C,G,T); off_a / off_b:
 * nprob+1 offsets; every length must be >= 1.  scores[p] gets
 * max(M,D,I) at (LA,LB).  If paths is not NULL, path p is written as edge
 * letters 'M' (both), 'D' (A only), 'I' (B only) in column order at
 * paths + path_off[p] (path_off[p+1]-path_off[p] >= LA+LB) and its length
 * in path_len[p]. */
int mvg_gapdp_batch(mvg_handle h, const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                    const uint64_t* off_b, int64_t nprob, int32_t* scores, char* paths,
                    const uint64_t* path_off, int64_t* path_len);
int mvg_gapdp_batch_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                        const uint64_t* d_off_b, int64_t nprob, int32_t* d_scores, char* d_paths,
                        const uint64_t* d_path_off, int64_t* d_path_len);

/* Banded gap DP with an exactness check and full-DP fallback.  Problem p is
 * first aligned inside the diagonal band of half-width band_half[p] around
 * j = i*LB/LA + band_delta[p] (host arrays).  The banded result is kept only
 * if its score is strictly above an upper bound on every path that leaves
 * the band (best exit-cell score + the sum of the best NUC_SP + 60 entry of
 * each base the path would still have to consume, taking the smaller of the
 * two sequences' sums); then its path equals the full NWSmall path.
 * Otherwise the problem is re-run through the full DP.  A band whose strips
 * cover at least half of the matrix (mvg_set_band_whole_fraction) is not
 * banded: that problem runs over the whole matrix.  Output is therefore always
 * identical to mvg_gapdp_batch.  used_band[p] (host, may be NULL) gets 1 when
 * the banded result was kept, 0 when the band was tried and rejected, 2 when
 * it was not tried; *cells (may be NULL) gets the DP cells actually computed.
 * No counterpart in the reference (a new method behind GlobalAlign,
 * MU/glbalign.cpp:69). */
int mvg_gapdp_banded(mvg_handle h, const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                     const uint64_t* off_b, int64_t nprob, const int32_t* band_delta, const int32_t* band_half,
                     int32_t* scores, char* paths, const uint64_t* path_off, int64_t* path_len,
                     uint8_t* used_band, uint64_t* cells);
int mvg_gapdp_banded_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                         const uint64_t* d_off_b, int64_t nprob, const int32_t* band_delta,
                         const int32_t* band_half, int32_t* d_scores, char* d_paths, const uint64_t* d_path_off,
                         int64_t* d_path_len, uint8_t* used_band, uint64_t* cells);

/* Full DP (as mvg_gapdp_batch_dev, scores into d_scores) that also writes each
 * optimal path's envelope: d_env[2p], d_env[2p+1] = min and max over the
 * path's cells (rows >= 1) of j - floor(i*LB/LA).  Training labels for the
 * band proposal; no counterpart in the reference. */
int mvg_gapdp_envelope_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                           const uint64_t* d_off_b, int64_t nprob, int32_t* d_scores, int32_t* d_env);

/* ------------------------------------------------ recursive anchor search */

/* The gaps one LCB of two genomes sends to the recursive anchor search:
 * ProgressiveAligner::recurseOnPairs (LM/ProgressiveAligner.cpp:682-924)
 * with getInterveningCoordinates (:566-588) and pairwiseAnchorSearch's cut
 * of the gap sequences (:598-613).  Host code, no GPU work.
 * row_a, row_b: the LCB's two gapped rows (ncols bytes each, '-' = gap);
 * left_end_a/b: 1-based left end of each genome's aligned range;
 * reverse_a/b: 1 if the genome is on the reverse strand in this LCB;
 * genome_len_a/b: the genomes' lengths; min_gap: the reference's
 * min_recursive_gap_length (200, LM/Aligner.cpp:183): a gap is searched when
 * both genomes leave more than min_gap characters between two columns where
 * both are aligned (or the LCB's end).
 * Out: gaps[4k .. 4k+3] = (0-based start in A, length in A, 0-based start
 * in B, length in B) in the reference's search order, ready for
 * mvg_gap_anchor_search (an empty cut has length 0); *ngaps = their number
 * (MVG_ERR_CAPACITY when above cap; nothing is written past cap);
 * flanks (optional, 8 values): per genome up to two unaligned stretches at
 * the LCB's ends (recurseOnPairs' iv_regions), 1-based [start, end), 0 where
 * absent. */
int mvg_recursion_gaps(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, int64_t left_end_a,
                       int reverse_a, int64_t left_end_b, int reverse_b, uint64_t genome_len_a,
                       uint64_t genome_len_b, int64_t min_gap, int64_t* gaps, uint64_t cap, uint64_t* ngaps,
                       int64_t* flanks);

/* ------------------------------------------------ anchored gap alignment */

/* Anchor columns of one window of a two-genome alignment: MUSCLE's
 * AnchoredProfileProfile as MuscleInterface::ProfileAlignFast calls it for
 * two single-sequence profiles (muscle/libMUSCLE/anchoredpp.cpp:256-458,
 * anchors.cpp:9-186; libMems/MuscleInterface.cpp:1053-1109), in the
 * reference's single-precision arithmetic.  Host code, no GPU work.
 * row_a, row_b: the window's two gapped rows (ncols bytes each, '-' or '.'
 * = gap).  Out: cols[0 .. *n) ascending (MVG_ERR_CAPACITY when above cap).
 * The n + 1 ranges [cols[i-1], cols[i]) (from column 0, to column ncols) are
 * what the reference realigns: each range's rows without their gaps are one
 * gap-DP problem (mvg_gapdp_batch), ranges of no column are skipped, and the
 * aligned ranges are concatenated in order (MSAAppend). */
int mvg_anchor_columns(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, uint32_t* cols, uint64_t cap,
                       uint64_t* n);

/* The windows of the gapped-alignment pass over one LCB of two genomes:
 * ProgressiveAligner::refineAlignment (LM/ProgressiveAligner.cpp:1119-1165)
 * with removeLargeGapsPP (:1051-1117: stretches of more than 5,000 columns
 * where the genomes are never aligned to each other become gap windows,
 * 300 columns kept on either side) and IsDenseEnough (:1015-1038: windows
 * halved while too long for their density; max_window_size is the
 * reference's 20,000 unless its option changes it).  Host code.
 * Out: windows[3k .. 3k+2] = (first column, end column, 1 for a gap window)
 * in column order; *n their number (MVG_ERR_CAPACITY when above cap).  Each
 * window that is not a gap window and holds bases of both genomes is
 * realigned with mvg_anchor_columns and the gap DP; the LCB's new rows are
 * the windows' rows in order. */
int mvg_refine_windows(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, double max_window_size,
                       int64_t* windows, uint64_t cap, uint64_t* n);

/* The column ranges the final iterative-refinement pass realigns in one LCB
 * of two genomes: refineAlignment with profile_aln = false
 * (LM/ProgressiveAligner.cpp:1199-1212) over the same windows as
 * mvg_refine_windows; every window that is not a gap window and has density
 * class 1 or 2 (IsDenseEnough, :1015-1038) goes through
 * MuscleInterface::RefineFast (LM/MuscleInterface.cpp:823-894) with RefineW
 * column windows of 500 or 200 columns (MU/refinew.cpp:75-184), each
 * realigned from its bases alone (for two sequences: one NWSmall problem,
 * genome A as profile A).  Class-0 windows stay as they are (RefineVert
 * returns at once for fewer than three sequences, MU/refinevert.cpp:60-61).
 * Host only.  Out: ranges[2k] = (first column, end column), in column order;
 * *n their number (MVG_ERR_CAPACITY when above cap). */
int mvg_refine_fast_ranges(const uint8_t* row_a, const uint8_t* row_b, uint64_t ncols, double max_window_size,
                           int64_t* ranges, uint64_t cap, uint64_t* n);

/* Both gapped-alignment passes of a two-genome progressiveMauve run over
 * many LCBs in one call: doGappedAlignment (LM/ProgressiveAligner.cpp:
 * 1242-1290) with refineAlignment (:1119-1230).  passes bit 0: the
 * gapped-alignment pass (profile_aln = true; every window that is not a gap
 * window and holds bases of both genomes realigned as ProfileAlignFast
 * (anchored) does, LM/MuscleInterface.cpp:1053-1109); bit 1: the final
 * iterative-refinement pass (profile_aln = false; mvg_refine_fast_ranges'
 * column windows realigned as RefineFast does).  Each pass plans on the
 * host, runs all problems of all LCBs in one batched gap-DP call and
 * rebuilds their rows on the GPU.  LCB k is columns col_off[k] ..
 * col_off[k+1]-1 of rows_a / rows_b ('-' gaps, bases A/C/G/T in either case
 * where a problem needs them, else MVG_ERR_BAD_BASE).  Out: the new rows in
 * out_a / out_b, LCB k at out_off[k] .. out_off[k+1]-1 (out_off has nlcb+1
 * entries and is set even when MVG_ERR_CAPACITY reports that the rows need
 * more than cap columns). */
int mvg_gapped_alignment(mvg_handle h, const uint8_t* rows_a, const uint8_t* rows_b, const uint64_t* col_off,
                         int64_t nlcb, double max_window_size, int passes, uint8_t* out_a, uint8_t* out_b,
                         uint64_t* out_off, uint64_t cap);

/* -------------------------------------------------- backbone detection */

/* Parameters of the backbone-detection HMM, the members of the reference's
 * Params (LM/HomologyHMM/homology.h:169-177) in order. */
typedef struct mvg_hmm_params {
  double start_homologous;
  double go_homologous;
  double go_unrelated;
  double go_stop_from_unrelated;
  double go_stop_from_homologous;
  double emit_homologous[8];
  double emit_unrelated[8];
} mvg_hmm_params;

/* The parameters applyBackbone uses (MA/progressiveMauve.cpp:226-238):
 * getAdaptedHoxdMatrixParameters(gc_content), then go_homologous and
 * go_unrelated set, then adaptToPercentIdentity(pct_identity)
 * (LM/HomologyHMM/parameters.h).  progressiveMauve's defaults: 1e-5, 1e-9,
 * 0.7.  MVG_ERR_ARG unless 0 < pct_identity <= 1 (the reference throws). */
int mvg_hmm_backbone_params(double gc_content, double go_homologous, double go_unrelated, double pct_identity,
                            mvg_hmm_params* out);

/* Homologous segments of two-genome alignments: findHssHomologyHMM
 * (LM/Islands.h:122-196) for every LCB, as detectAndApplyBackbone runs it
 * (LM/Backbone.cpp:1081-1088, left and right homologous both set): column
 * emission symbols, the HMM's forward and backward passes in HMMoC's
 * extended-exponent arithmetic, posterior >= 0.9, and the homologous column
 * ranges.  Host only (one LCB per host thread).  LCB k is columns
 * col_off[k] .. col_off[k+1]-1 of rows_a / rows_b.  Out: 2 int64 per
 * segment (first and last column, inclusive, relative to the LCB), LCB k's
 * segments at seg_off[k] .. seg_off[k+1]-1 (seg_off has nlcb+1 entries);
 * *nsegs the total, MVG_ERR_CAPACITY when above cap. */
int mvg_homologous_segments(const uint8_t* rows_a, const uint8_t* rows_b, const uint64_t* col_off, int64_t nlcb,
                            const mvg_hmm_params* params, int left_homologous, int right_homologous, int64_t* segs,
                            uint64_t cap, uint64_t* nsegs, uint64_t* seg_off);

/* ------------------------------------------------ search outside LCBs */

/* Match lists below are 3 int64 per match: libMems' signed 1-based start in
 * A, start in B (negative = reverse strand, 0 = not in that genome), length.
 * Regions are 1-based (left end, right end + 1) pairs, flattened, in
 * concatenation order -- the iv_regions vectors of the reference. */

/* SearchLCBGaps (LM/Aligner.cpp:784-928) for two genomes, as
 * ProgressiveAligner::alignPP calls it after a recursion round
 * (LM/ProgressiveAligner.cpp:2474-2488, regions sorted there).  The regions
 * of each genome are concatenated and the concatenations searched on the GPU
 * by the pairwise matcher with seed getSeed(getDefaultSeedWeight(mean
 * concatenation length), 0) (no search below weight 5: *count = 0); the
 * matches are then transposed back to genome coordinates, split at region
 * seams, overlap-eliminated and length-filtered as mvg_lcb_gap_finish.
 * *weight (optional) gets the seed weight.  MVG_ERR_RANGE for a region
 * outside its genome (the reference catches the cut's exception and searches
 * without that region), MVG_ERR_CAPACITY when the matches exceed cap
 * (*count holds the number). */
int mvg_search_lcb_gaps(mvg_handle h, const uint8_t* seq_a, uint64_t na, const uint8_t* seq_b, uint64_t nb,
                        const int64_t* regions_a, uint64_t nra, const int64_t* regions_b, uint64_t nrb, int64_t* out,
                        uint64_t cap, uint64_t* count, uint32_t* weight);
/* The same with the genomes in device memory (regions and output on the
 * host); the regions are gathered on the GPU. */
int mvg_search_lcb_gaps_dev(mvg_handle h, const uint8_t* d_seq_a, uint64_t na, const uint8_t* d_seq_b, uint64_t nb,
                            const int64_t* regions_a, uint64_t nra, const int64_t* regions_b, uint64_t nrb,
                            int64_t* out, uint64_t cap, uint64_t* count, uint32_t* weight);

/* The host steps after the search (LM/Aligner.cpp:891-923): matches of the
 * two concatenations (pairwise-matcher order) -> MultiplicityFilter(2),
 * transposeMatches for A then B, EliminateOverlaps, MultiplicityFilter(2),
 * LengthFilter(MIN_ANCHOR_LENGTH = 9).  Host only. */
int mvg_lcb_gap_finish(const int64_t* matches, uint64_t n, const int64_t* regions_a, uint64_t nra,
                       const int64_t* regions_b, uint64_t nrb, int64_t* out, uint64_t cap, uint64_t* count);
/* transposeMatches (LM/Aligner.cpp:973-1045) for genome seq (0 = A, 1 = B):
 * sorts by MatchLeftEndComparator(seq), maps concatenation starts to genome
 * starts and splits a match at each region seam it crosses (the pieces are
 * appended after the sorted list).  Host only. */
int mvg_transpose_matches(const int64_t* matches, uint64_t n, unsigned seq, const int64_t* regions,
                          uint64_t nregions, int64_t* out, uint64_t cap, uint64_t* count);
/* EliminateOverlaps (LM/Aligner.cpp:62-176) for two-genome matches.  Host
 * only. */
int mvg_eliminate_overlaps(const int64_t* matches, uint64_t n, int64_t* out, uint64_t cap, uint64_t* count);
/* LCBs of a two-genome match list for collinear genomes: the collinear
 * branch of alignProfileToProfile (LM/ProgressiveAligner.cpp:2281-2303) --
 * IdentifyBreakpoints, ComputeLCBs_v2, SimpleGetLCBCoverage weights,
 * breakpoint penalty 100 + their sum, computeLCBAdjacencies_v3, greedy
 * breakpoint elimination (greedyBreakpointElimination_v4 with a collinear
 * SimpleBreakpointScorer) and filterMatches_v2.  matches: n (start A, start
 * B, length) triples, both starts nonzero.  Out: the surviving LCBs' matches
 * concatenated into out (room for n triples), LCB k at
 * [lcb_off[k], lcb_off[k + 1]) (*nlcb LCBs; MVG_ERR_CAPACITY when
 * *nlcb + 1 > lcb_cap), and the deleted matches in deleted (room for n
 * triples, *ndeleted of them).  Host only. */
int mvg_collinear_lcbs(const int64_t* matches, uint64_t n, int64_t* out, uint64_t* lcb_off, uint64_t lcb_cap,
                       uint64_t* nlcb, int64_t* deleted, uint64_t* ndeleted);

/* ------------------------------------------------ band-proposal network */

/* The band proposal for mvg_gapdp_banded: a 528 -> 256 -> 256 -> 256 -> 2
 * MLP (GELU, BF16 weights and activations, FP32 accumulation on the tensor
 * cores: tcgen05 for the forward hidden layers, mma.sync for the backward
 * GEMMs; FP32 master weights and Adam state), one per handle.  Its input per
 * gap is the 4-mer spectra of both sequences (2 x 256) and their log lengths;
 * its outputs are the band's diagonal offset / 100 and log(1 + half-width).
 * No counterpart in the reference.
 * Parameters are a flat fp32 array of mvg_mlp_num_params() values:
 * W1[256x528], b1[256], W2[256x256], b2, W3[256x256], b3, W4[2x256], b4[2]. */
int64_t mvg_mlp_num_params(void);
int mvg_mlp_set_params(mvg_handle h, const float* params);
int mvg_mlp_get_params(mvg_handle h, float* params);
/* Features of nprob gaps (device inputs) into d_x_bf16 [nprob x 528] (bf16). */
int mvg_band_features_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                          const uint64_t* d_off_b, int64_t nprob, void* d_x_bf16);
/* Forward pass: d_out [n x 2] (fp32, device). */
int mvg_mlp_forward_dev(mvg_handle h, const void* d_x_bf16, int64_t n, float* d_out);
/* Mean-squared-error loss against d_target [n x 2] and its gradient with
 * respect to every parameter (host, flat layout; may be NULL). */
int mvg_mlp_grad_dev(mvg_handle h, const void* d_x_bf16, const float* d_target, int64_t n, float* grads,
                     float* loss);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on a minibatch; step counts from 1.
 * The gradient is scaled to global L2 norm <= 1; a minibatch whose gradient
 * is not finite changes nothing (its loss is still returned). */
int mvg_mlp_train_step_dev(mvg_handle h, const void* d_x_bf16, const float* d_target, int64_t n, float lr,
                           int step, float* loss);
/* Forward hidden layers on the tcgen05 tensor cores (on = 1, the default):
 * TMA loads the operand tiles, the accumulators live in tensor memory, and
 * bias, GELU and (last hidden layer) the 256 -> 2 output layer run in the
 * epilogue.  on = 0 runs them as mma.sync GEMMs plus elementwise kernels.
 * The tcgen05 path also needs every operand in TMA form (16-byte aligned,
 * rows a multiple of 8; inputs the library allocates are padded, an input
 * passed to mvg_mlp_forward_dev with n not a multiple of 8 is not), else
 * the pass runs on mma.sync.  The two paths differ only in the order of
 * fp32 sums.  mvg_mlp_tcgen05_passes counts the forward passes that ran on
 * tcgen05.  No counterpart in the reference. */
int mvg_set_mlp_tcgen05(mvg_handle h, int on);
int mvg_mlp_tcgen05_passes(mvg_handle h, uint64_t* passes);
/* Features + forward + mapping to integer bands: delta = round(100 * o0),
 * half = ceil(alpha * (exp(o1) - 1) + beta); host outputs. */
int mvg_band_propose_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                         const uint64_t* d_off_b, int64_t nprob, float alpha, float beta, int32_t* band_delta,
                         int32_t* band_half);
/* Divergence gate for mvg_band_propose_dev (min_match = 0, the default,
 * turns it off): up to 8 windows of 32 bases of A along the diagonal
 * j = i*LB/LA are matched against B at diagonal offsets -8..8; a gap where
 * fewer than half of its windows reach min_match matching bases (of 32) at
 * their best offset is proposed the whole matrix, since no narrow band can
 * pass the exactness check there.  Gaps shorter than 32 are not gated. */
int mvg_set_band_gate(mvg_handle h, int min_match);

/* ------------------------------------------------------ .sslist cache file */

/* The sorted mer list file progressiveMauve caches next to each FASTA
 * (FileSML::Create / LoadFile2, libMems/FileSML.cpp:401-459, 120-195):
 * the SMLHeader struct (libMems/SortedMerList.h:48-63, 2352 bytes, format
 * version 5), the 2-bit packed sequence (binary_seq_len uint32 words: the
 * sequence's words plus two pad words), then one uint32 position per SML
 * entry in sorted order.  mvg_sslist_write builds the SML on the GPU and
 * writes the file; entries with equal mers are in position order.
 * mvg_sslist_read parses a file (no GPU needed): with words / pos NULL it
 * only fills info; status gets LoadFile2's failure code (1 cannot open, 2
 * short header, 3 other format version, 4 truncated sequence, 5 positions
 * unreadable; 0 otherwise). */
typedef struct {
  uint64_t seed;
  uint32_t seed_length, seed_weight;
  uint64_t length;   /* bases */
  uint64_t words;    /* packed sequence words, pad words included */
  uint64_t entries;  /* positions after the sequence */
  int circular;
  int status;
} mvg_sslist_info;
int mvg_sslist_write(mvg_handle h, const uint8_t* seq, uint64_t n, uint64_t seed, const char* path);
int mvg_sslist_read(const char* path, mvg_sslist_info* info, uint32_t* words, uint64_t cap_words, uint32_t* pos,
                    uint64_t cap_pos);

/* ------------------------------------------------------------ index LUT */

/* Genome -> reference index LUT (int32, -1 = unmapped) as mauve.buildIndex
 * builds it after parsing progressiveMauve's XMFA output.  Aligned blocks
 * are passed flattened: block b's two gapped rows (genome = sequence 1,
 * reference = sequence 2) are columns [col_off[b], col_off[b+1]) of
 * genome_rows / ref_rows; genome_start / ref_start are the sub-alignments'
 * start_idx as the XMFA parse gives them.  Callers pass only groups where
 * both sequences are present (lookupSubAlignment, mauve/indexutils.pyx:17-24,
 * returned both).  Limits: n <= 2^31-1 entries, fewer than 2^32-1 columns.
 * The _dev forms take device pointers and run on the handle's stream; like
 * every entry point they return once their GPU work has finished. */

/* mauve/buildindex.py:112-130: LUT of n entries from the blocks (later
 * blocks and columns overwrite earlier ones; a write at genome index -1
 * lands in lut[n-1] as a numpy index does).  MVG_ERR_RANGE / MVG_ERR_OVERFLOW
 * where the reference raises IndexError / OverflowError; the LUT is then
 * unspecified. */
int mvg_lut_from_blocks(mvg_handle h, const int64_t* genome_start, const int64_t* ref_start, const uint64_t* col_off,
                        const uint8_t* genome_rows, const uint8_t* ref_rows, uint64_t nblocks, int32_t* lut,
                        uint64_t n);
int mvg_lut_from_blocks_dev(mvg_handle h, const int64_t* d_genome_start, const int64_t* d_ref_start,
                            const uint64_t* d_col_off, const uint8_t* d_genome_rows, const uint8_t* d_ref_rows,
                            uint64_t nblocks, int32_t* d_lut, uint64_t n);
/* mauve/indexutils.pyx:27-44 fixZeroIdx (in place).  MVG_ERR_RANGE where
 * the Cython function raises IndexError. */
int mvg_lut_fix_zero_idx(mvg_handle h, int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t genome_len,
                         const uint8_t* ref, uint64_t ref_len);
int mvg_lut_fix_zero_idx_dev(mvg_handle h, int32_t* d_lut, uint64_t n, const uint8_t* d_genome, uint64_t genome_len,
                             const uint8_t* d_ref, uint64_t ref_len);
/* mauve/indexutils.pyx:47-75 fillGaps and :78-108 smoothEdges (in place,
 * same result as the sequential passes). */
int mvg_lut_fill_gaps(mvg_handle h, int32_t* lut, uint64_t n, int max_gap_width);
int mvg_lut_fill_gaps_dev(mvg_handle h, int32_t* d_lut, uint64_t n, int max_gap_width);
int mvg_lut_smooth_edges(mvg_handle h, int32_t* lut, uint64_t n, int smoothing_radius);
int mvg_lut_smooth_edges_dev(mvg_handle h, int32_t* d_lut, uint64_t n, int smoothing_radius);
/* mauve/indexutils.pyx:111-139 findGaps: fills like fillGaps(300) and writes
 * gaps[n] (filled gap size at a gap start, -1 where none was found, else 0). */
int mvg_lut_find_gaps(mvg_handle h, int32_t* lut, uint64_t n, int32_t* gaps);
int mvg_lut_find_gaps_dev(mvg_handle h, int32_t* d_lut, uint64_t n, int32_t* d_gaps);
/* mauve/indexutils.pyx:142-156 findEdges as its 0/1 byte mask (before the
 * bit packing). */
int mvg_lut_find_edges(mvg_handle h, const int32_t* lut, uint64_t n, uint8_t* edges);
/* mauve/indexutils.pyx:159-175 findMismatches as a 0/1 byte mask of n
 * entries.  A mapped index outside the reference is MVG_ERR_RANGE (the
 * Cython function reads past its buffer there). */
int mvg_lut_find_mismatches(mvg_handle h, const int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t genome_len,
                            const uint8_t* ref, uint64_t ref_len, uint8_t* mismatches);
/* mauve/indexutils.pyx:178-186 findDuplicateMappings. */
int mvg_lut_find_duplicate_mappings(mvg_handle h, const int32_t* lut, uint64_t n, int64_t* result);
/* mauve/buildindex.py:111-138 after the XMFA parse: the LUT of n entries
 * (the genome's length) from the blocks, then fixZeroIdx +
 * fillGaps(max_gap_width) when fill_gaps, then smoothEdges(smoothing_radius)
 * when smooth_edges.  genome / ref are read only when fill_gaps. */
int mvg_build_index_lut(mvg_handle h, const int64_t* genome_start, const int64_t* ref_start, const uint64_t* col_off,
                        const uint8_t* genome_rows, const uint8_t* ref_rows, uint64_t nblocks, const uint8_t* genome,
                        uint64_t genome_len, const uint8_t* ref, uint64_t ref_len, int fill_gaps, int max_gap_width,
                        int smooth_edges, int smoothing_radius, int32_t* lut, uint64_t n);
int mvg_build_index_lut_dev(mvg_handle h, const int64_t* d_genome_start, const int64_t* d_ref_start,
                            const uint64_t* d_col_off, const uint8_t* d_genome_rows, const uint8_t* d_ref_rows,
                            uint64_t nblocks, const uint8_t* d_genome, uint64_t genome_len, const uint8_t* d_ref,
                            uint64_t ref_len, int fill_gaps, int max_gap_width, int smooth_edges,
                            int smoothing_radius, int32_t* d_lut, uint64_t n);

/* Aligned rows from gap-DP paths: AlignTwoMSAsGivenPath
 * (MU/aligngivenpath.cpp:256) for single-sequence profiles, for a batch.
 * Edge t of path p is column t: 'M' takes the next character of both
 * sequences, 'D' the next of A against '-', 'I' '-' against the next of B.
 * seq_a / seq_b / off_a / off_b as for mvg_gapdp_batch (the characters are
 * copied as given, so ASCII bases may be passed); paths / path_off /
 * path_len as mvg_gapdp_batch writes them.  rows_a and rows_b receive the
 * two gapped rows of problem p at [path_off[p], path_off[p] + path_len[p]).
 * MVG_ERR_ARG if a path does not consume exactly its two sequences. */
int mvg_path_rows(mvg_handle h, const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                  const uint64_t* off_b, int64_t nprob, const char* paths, const uint64_t* path_off,
                  const int64_t* path_len, uint8_t* rows_a, uint8_t* rows_b);
int mvg_path_rows_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                      const uint64_t* d_off_b, int64_t nprob, const char* d_paths, const uint64_t* d_path_off,
                      const int64_t* d_path_len, uint8_t* d_rows_a, uint8_t* d_rows_b);

/* XMFA writer: GenericIntervalList::WriteStandardAlignment
 * (LM/IntervalList.h:353-440) for pairwise blocks, as progressiveMauve
 * writes the file buildIndex parses (MA/progressiveMauve.cpp:727).
 * file_a / file_b: the two sequence file names (written as the sequence
 * names; the format line follows the name's extension as libGenome's
 * source factory does); backbone_file may be NULL or "".  Block b has
 * columns col_off[b] .. col_off[b+1]-1 of rows_a / rows_b (the gapped rows,
 * '-' for gaps, already reverse-complemented for a reverse-strand
 * sequence), signed starts starts[2b], starts[2b+1] (1-based left end,
 * negative = reverse strand, 0 = absent) and base counts lengths[2b],
 * lengths[2b+1].  out receives the text (not NUL-terminated); *out_len gets
 * its length, MVG_ERR_CAPACITY if it exceeds cap.  The text is assembled on
 * the device. */
int mvg_xmfa_write(mvg_handle h, const char* file_a, const char* file_b, const char* backbone_file,
                   int64_t nblocks, const int64_t* starts, const int64_t* lengths, const uint8_t* rows_a,
                   const uint8_t* rows_b, const uint64_t* col_off, char* out, uint64_t cap, uint64_t* out_len);
/* The same with the rows in device memory (the other arrays on the host). */
int mvg_xmfa_write_dev(mvg_handle h, const char* file_a, const char* file_b, const char* backbone_file,
                       int64_t nblocks, const int64_t* starts, const int64_t* lengths, const uint8_t* d_rows_a,
                       const uint8_t* d_rows_b, const uint64_t* col_off, char* out, uint64_t cap, uint64_t* out_len);

/* Upper bound on the device bytes the gap-DP traceback arena may use.  Each
 * call uses min(bound, 60% of free device memory); problems run in waves of
 * mixed sizes that fit it.  Default: no bound beyond the 60% cap. */
int mvg_set_tb_arena(mvg_handle h, uint64_t bytes);

/* Gap-DP kernel shape: rows per lane for the full DP (4 or 8) and for banded
 * passes (1, 2, 4 or 8); strips are 32*rows rows.  The Python binding applies
 * the tuned choice committed in mauve-py_gb300/dp_tuning.json. */
int mvg_set_dp_rows(mvg_handle h, int full_rows, int band_rows);

/* Banded passes: a proposed band that covers at least `fraction` of its
 * matrix (0 < fraction <= 1, default 0.5) is not banded; the problem runs
 * over the whole matrix in the strip kernel's launch (status 2).  With the
 * ring schedule on, the share is that of the columns a row keeps
 * (2*half + 2 + ceil(LB/LA)) in LB; otherwise that of the strips' cells. */
int mvg_set_band_whole_fraction(mvg_handle h, double fraction);

/* Banded passes on the ring schedule (on = 1, the default): one warp per
 * problem, groups of 4, 6, 8, 12, 16, 24 or 32 rows per lane chained lane to lane along
 * the band, the smallest group height whose schedule is valid for the band;
 * bands no height fits run in the strip kernel.  on = 0 runs every band in
 * the strip kernel.  Results are identical either way. */
int mvg_set_band_ring(mvg_handle h, int on);

/* Watchdog of the gap DP's whole-CTA mode: each wait of a warp for the
 * previous strip's warp polls at most `polls` times (default 2^26, about a
 * second) before it gives up; the kernel then stops that problem, the other
 * warps of the CTA stop at their next wait, and the call returns
 * MVG_ERR_DEVICE instead of hanging.  The handle stays usable.  A very small
 * limit makes the waits give up on purpose (a test of the watchdog).  No
 * counterpart in the reference (single-threaded). */
int mvg_set_dp_spin_limit(mvg_handle h, long long polls);

/* Full gap DP: problems of at least `strips` strips (of 32 * rows-per-lane
 * rows) are solved by a whole CTA whose 8 warps pipeline the strips, smaller
 * ones by one warp each (default 16; the Python binding applies the tuned
 * choice in mauve-py_gb300/dp_tuning.json).  Results do not depend on it. */
int mvg_set_dp_coop_strips(mvg_handle h, int strips);

/* mvg_gapdp_banded: the tallest group height (rows per lane) a band may use
 * on the ring schedule (0..32, default 32); bands no allowed height fits run
 * in the strip kernel.  Results do not depend on it. */
int mvg_set_ring_max_rows(mvg_handle h, int rows);

/* mvg_gapdp_banded: problems whose band covers so much of the matrix that
 * they run whole (see mvg_set_band_whole_fraction) go to the full DP when A
 * has at least `rows` rows, else into the strip kernel's launch with a band
 * covering the matrix (default 512, measured on 200,000 gaps drawn like the
 * recoded pair's).  Results do not depend on it. */
int mvg_set_band_whole_full_rows(mvg_handle h, int64_t rows);

/* Full gap-DP passes checkpointed (on = 1, the default): the forward pass
 * keeps every strip's bottom row and, every 128 columns, every strip's
 * column of cell states instead of traceback bits (about 0.19 instead of
 * 0.5 bytes per cell), and the traceback recomputes the bits of only the
 * blocks of the matrix its path crosses, with the same recurrence and tie
 * order.  on = 0 stores the bits.  Scores and paths are identical either
 * way; banded passes always store bits.  No counterpart in the reference. */
int mvg_set_dp_checkpoint(mvg_handle h, int on);

/* Gap-DP passes as one CUDA graph (on = 1, the default): the launches of a
 * call's waves (claim counters, the persistent DP kernel, both traceback
 * walkers, path compaction) are recorded into one graph and launched at
 * once; the handle keeps the executable graph per DP lane and updates it in
 * place from the next call's recording when its shape is the same.  on = 0
 * launches them one by one.  Results are identical either way.  No
 * counterpart in the reference. */
int mvg_set_dp_graph(mvg_handle h, int on);

/* Per-stage timing with CUDA events on the handle's stream (off by default;
 * no extra synchronisation).  After a call, mvg_stage_times gives the stage
 * names (comma separated into names, of capacity names_cap) and each stage's
 * milliseconds in ms[0..*n); the device stages come first, then the call's
 * host-side planning sections as "host_<name>" (wall time, summed per
 * name).  No counterpart in the reference (it prints progress only). */
int mvg_set_profiling(mvg_handle h, int on);
int mvg_stage_times(mvg_handle h, char* names, size_t names_cap, double* ms, int cap, int* n);

/* Microbenchmark: sustained INT32 add/max throughput of this GPU, in
 * operations per second, from a dependent-chain-free kernel timed with
 * CUDA events.  Used as the roofline denominator for the gap DP. */
int mvg_probe_int32_peak(mvg_handle h, double* ops_per_s);

#ifdef __cplusplus
}
#endif
#endif
