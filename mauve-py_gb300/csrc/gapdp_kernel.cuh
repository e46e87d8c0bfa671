// The NWSmall wavefront kernel, full or banded (included by gapdp.cu).
//
// The DP matrix is cut into strips of 32*R rows; lane t of a warp owns rows
// [t*R, t*R+R) of a strip and sweeps the strip's columns on an anti-diagonal
// wavefront (lane t runs t columns behind lane 0).  Each step a lane computes
// an R x 1 column segment: the cells above it arrive from lane t-1 by
// __shfl_up_sync, the row above the strip comes from a row buffer written by
// lane 31 of the warp that ran the previous strip.  B codes and row-buffer
// entries are staged in per-warp shared rings one 32-step chunk ahead.
// Traceback nibbles (MU/types.h:30-43: 2 bits M source, 1 bit D<-M, 1 bit
// I<-M) are packed 8 per word, lane-minor, so each flush is one coalesced
// 128-byte warp store.
//
// Work split: persistent CTAs first take the large problems (the front of
// the wave's list, at least kCoopMinStrips strips) one per CTA: warp w runs
// strips w, w+8, w+16, ... as a pipeline, each warp consuming the bottom row
// its predecessor publishes in a per-CTA buffer; progress is exchanged
// through shared-memory counters every 32 steps, and every wait is bounded
// (a watchdog error instead of a hang).  Then each warp takes small problems
// on its own.
//
// Per cell the recurrences use Hopper/Blackwell DPX max-with-predicate
// (__vibmax_s32), which yields each maximum and its tie-broken traceback bit
// in one instruction.  The steady part of a strip (every lane inside the
// strip's columns) runs without per-step bounds checks; only the 31-step
// ramp-up and ramp-down of the wavefront take the checked path.
//
// Banded mode: strip k only spans columns [jlo_k, jhi_k] of a diagonal band
// (band.h), everything outside is -infinity, and the kernel also computes an
// upper bound on every path that leaves the band: the best exit-cell score
// plus the largest score the rest of the path could still collect.  From
// cell (i, j) the rest consumes A[i..LA) and B[j..LB); gap steps score <= 0
// and each match step pairs one base of each, scoring at most that base's
// best NUC_SP + 60 entry, so the rest scores at most
// min(sum of row maxima over A[i..LA), sum of column maxima over B[j..LB)).
// Those suffix sums come from per-problem totals and running prefix sums.  A
// banded result is accepted only when its score is strictly above the
// bound; then the reference's optimal path provably stays in the band and
// every traceback decision along it is the same as in the full DP.
#pragma once
#include "band.h"
#include "mvg_common.cuh"

namespace mvg {

constexpr int32_t kNeg = -(1 << 29);
constexpr int32_t kGap = -200;           // half of gap open -400
constexpr int32_t kMaxPair = 160;        // max NUC_SP + 60 (C/C, G/G)
constexpr int kDpThreads = 256;
constexpr int kDpWarps = kDpThreads / 32;
constexpr int kCoopMinStrips = 16;       // banded problems with at least this many strips use a whole CTA

enum : uint32_t { TB_MM = 0, TB_DM = 1, TB_IM = 2, TB_MD = 4, TB_MI = 8 };

// NUC_SP + 60 (range -65..160), packed: entry (a,b) = byte b of
// c_score_rows[a], stored with a +80 bias so every byte is in 15..240.
constexpr int kScoreBias = 80;
__constant__ uint32_t c_score_rows[4];  // this header has one includer (gapdp.cu)

struct DpJob {
  const uint8_t* sa;
  const uint64_t* oa;
  const uint8_t* sb;
  const uint64_t* ob;
  const uint32_t* order;   // problem ids of this wave: large problems first, each part largest first
  const uint64_t* tb_off;  // byte offset of each wave slot's traceback bits
  int nwork;
  int nbig;                // the first nbig slots are solved by whole CTAs
  uint32_t* tb;
  int4* rowbuf;
  int64_t rowbuf_stride;  // int4 entries per row buffer (one per warp)
  int32_t* scores;
  uint8_t* end_edge;  // 'M','D','I' per problem
  const int32_t* band_delta;  // banded mode: per problem
  const int32_t* band_half;
  uint8_t* accept;            // banded mode: 1 if the band result is exact
  uint32_t base_max;          // banded mode: best score of each base code, byte c = max + kScoreBias
  unsigned* counter;          // [0] large-problem claims (per CTA), [1] small-problem claims (per warp)
  uint32_t* err;
  long long spin_limit;       // polls before a cooperative-mode wait gives up (watchdog)
};

__host__ __device__ __forceinline__ int tb_words_per_lane(int W, int R) { return band_words_per_lane(W, R); }

template <int R>
struct DpLane {
  uint32_t arow[R];             // packed score row of A[i-1] per owned row
  int32_t lM[R], lD[R], lI[R];  // left neighbour (previous column) per row
};

// One wavefront step of one lane: rows r = 0..R-1 of column j.  Returns the
// R traceback nibbles.  M is carried with the gap open already added
// (Mg = M + kGap: the value both the D and the I recurrence read), so
// neither needs an add; the M recurrence adds twice the close to max(D, I)
// instead of once, which leaves every comparison, and so every tie-broken
// traceback bit, as it was.  (up*) = cells (i0-1, j), (dg*) = cells
// (i0-1, j-1); ADJ steps add goBadj to the left Mg (-kGap in column 1,
// where the reference opens for free).
template <int R, bool ADJ>
__device__ __forceinline__ uint32_t dp_column(DpLane<R>& L, int32_t upMg, int32_t upD, int32_t dgMg, int32_t dgD,
                                              int32_t dgI, uint32_t bsel, int32_t goBadj) {
  int32_t cuM = upMg, cuD = upD;            // (i-1, j)
  int32_t cdM = dgMg, cdD = dgD, cdI = dgI;  // (i-1, j-1)
  uint32_t nibs = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    // D(i,j) = max(M(i-1,j) + open, D(i-1,j)), ties to the M branch
    bool dm;
    const int32_t D = __vibmax_s32(cuM, cuD, &dm);
    // I(i,j) = max(M(i,j-1) + open, I(i,j-1)), ties to the M branch
    bool mi;
    const int32_t I = __vibmax_s32(ADJ ? L.lM[r] + goBadj : L.lM[r], L.lI[r], &mi);
    // M(i,j) = s + max(M, D + close, I + close) at (i-1,j-1), tie M > D > I;
    // both closes are -200, so max(D, I) is taken before adding the close.
    bool dge, mge;
    const int32_t DI = __vibmax_s32(cdD, cdI, &dge) + 2 * kGap;
    const int32_t best = __vibmax_s32(cdM, DI, &mge);
    const int32_t M = best + (int32_t)__byte_perm(L.arow[r], 0u, bsel) - kScoreBias;  // Mg
    const uint32_t tm = mge ? TB_MM : (dge ? TB_DM : TB_IM);
    nibs |= (tm | (dm ? TB_MD : 0u) | (mi ? TB_MI : 0u)) << (4 * r);
    cdM = L.lM[r];
    cdD = L.lD[r];
    cdI = L.lI[r];
    cuM = M;
    cuD = D;
    L.lM[r] = M;
    L.lD[r] = D;
    L.lI[r] = I;
  }
  return nibs;
}

// The same step without traceback bits (checkpointed passes): plain maxima
// instead of max-with-predicate, same values.
template <int R, bool ADJ>
__device__ __forceinline__ void dp_column_score(DpLane<R>& L, int32_t upMg, int32_t upD, int32_t dgMg, int32_t dgD,
                                                int32_t dgI, uint32_t bsel, int32_t goBadj) {
  int32_t cuM = upMg, cuD = upD;
  int32_t cdM = dgMg, cdD = dgD, cdI = dgI;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int32_t D = max(cuM, cuD);
    const int32_t I = max(ADJ ? L.lM[r] + goBadj : L.lM[r], L.lI[r]);
    const int32_t best = max(cdM, max(cdD, cdI) + 2 * kGap);
    const int32_t M = best + (int32_t)__byte_perm(L.arow[r], 0u, bsel) - kScoreBias;
    cdM = L.lM[r];
    cdD = L.lD[r];
    cdI = L.lI[r];
    cuM = M;
    cuD = D;
    L.lM[r] = M;
    L.lD[r] = D;
    L.lI[r] = I;
  }
}

// Checkpointed full DP.  Instead of traceback bits the forward pass keeps
// the cell states (Mg, D, I) the traceback needs to recompute any block of
// the matrix: the bottom row of every strip but the last (which the next
// strip reads as its top row, so it also replaces the row buffer), and,
// every kCkCols columns, the column of every strip.  The traceback then
// recomputes, with traceback bits, only the blocks of 32*R rows x kCkCols
// columns its path crosses (k_tb_ck).  Per problem slot (int4 entries):
//   row (k, j), k < nstrips - 1, 1 <= j <= LB   at k * LB + j - 1
//   column (k, b, q), 1 <= b < ncb, q < 32 R    at rows + (k * (ncb - 1) + b - 1) * 32 R + q
// (the state left of block b's first column b * kCkCols + 1).
constexpr int kCkCols = 128;

__host__ __device__ __forceinline__ int ck_nblocks(int LB) { return (LB + kCkCols - 1) / kCkCols; }
__host__ __device__ __forceinline__ int64_t ck_row_entries(int LA, int LB, int R) {
  const int nstrips = (LA + 32 * R - 1) / (32 * R);
  return (int64_t)(nstrips - 1) * LB;
}
__host__ __device__ __forceinline__ int64_t ck_col_entry(int LA, int LB, int R, int k, int b) {
  return ck_row_entries(LA, LB, R) + ((int64_t)k * (ck_nblocks(LB) - 1) + (b - 1)) * (32 * R);
}
__host__ __device__ __forceinline__ int64_t ck_entries(int LA, int LB, int R) {
  const int nstrips = (LA + 32 * R - 1) / (32 * R);
  return ck_row_entries(LA, LB, R) + (int64_t)nstrips * (ck_nblocks(LB) - 1) * (32 * R);
}

// Sum over s[from, to) of each base's best score (warp-wide, every lane
// gets the total).  base_max packs the biased maxima of codes 0..3.
__device__ __forceinline__ int32_t warp_best_sum(const uint8_t* s, int from, int to, uint32_t base_max) {
  const int lane = threadIdx.x & 31;
  int32_t acc = 0;
  for (int t = from + lane; t < to; t += 32) acc += (int32_t)__byte_perm(base_max, 0u, (s[t] & 3u) | 0x4440u) - kScoreBias;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  return acc;
}

// selector nibbles 1..3 = 4 pick zero bytes of the second operand
__device__ __forceinline__ int32_t best_of(uint32_t base_max, uint32_t code) {
  return (int32_t)__byte_perm(base_max, 0u, (code & 3u) | 0x4440u) - kScoreBias;
}

// Shared state of one CTA.
struct DpShared {
  uint8_t ringB[kDpWarps][128];
  int4 ringR[kDpWarps][64];
  volatile unsigned long long prog[kDpWarps];  // cooperative mode: (strip << 21) | last column published
  int bound;                                   // cooperative mode: CTA-wide band-exit bound
  int abort;                                   // cooperative mode: a wait gave up
  int claim;
};

// Solves problem slot w.  Strips kstart, kstart + kstep, ... are run by this
// warp; coop = true when the CTA's warps share the problem.
template <bool BANDED, int R, bool CK>
__device__ void dp_solve(const DpJob& J, DpShared& sh, int w, int kstart, int kstep, bool coop, int4* rowbuf_base,
                         int4* own_rowbuf) {
  static_assert(!(BANDED && CK), "checkpoints are kept for the full DP only");
  constexpr int SR = 32 * R;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint8_t* ringB = sh.ringB[wib];
  int4* ringR = sh.ringR[wib];
  // a cell outside the matrix, M carried as Mg (see dp_column)
  const int4 kNegCell = make_int4(kNeg + kGap, kNeg, kNeg, 0);
  const uint32_t p = J.order[w];
  const uint64_t a0 = J.oa[p], b0 = J.ob[p];
  const int LA = (int)(J.oa[p + 1] - a0), LB = (int)(J.ob[p + 1] - b0);
  const uint8_t* A = J.sa + a0;
  const uint8_t* B = J.sb + b0;
  const int nstrips = (LA + SR - 1) / SR;
  const int end_strip = (LA - 1) / SR;
  const int end_lane = ((LA - 1) % SR) / R;
  const int end_r = (LA - 1) % R;
  const Band band = BANDED ? make_band(LA, LB, J.band_delta[p], J.band_half[p], SR) : make_full(LA, LB, SR);
  // a band at least as wide as the matrix has no exits: nothing to bound
  const bool track = BANDED && J.band_half[p] <= (LA > LB ? LA : LB);
  int32_t bound = kNeg;  // best score of any path leaving the band (this warp's part)
  // banded mode: totals and running prefixes of the per-base best scores
  int32_t totA = 0, totB = 0, pa = 0, pb_lo = 0, pb_hi = 0;
  int pa_rows = 0, pb_lo_cols = 0;
  if (track) {
    totA = warp_best_sum(A, 0, LA, J.base_max);
    totB = warp_best_sum(B, 0, LB, J.base_max);
  }
  uint32_t* tbs = J.tb + J.tb_off[w] / 4;
  int4* ck = reinterpret_cast<int4*>(tbs);  // checkpointed pass: the slot's checkpoints
  if (!CK)
    for (int k = 0; k < kstart; ++k) tbs += (int64_t)tb_words_per_lane(band_hi(band, k) - band_lo(band, k) + 1, R) * 32;

  for (int k = kstart; k < nstrips; k += kstep) {
    const int row0 = k * SR;
    const int jlo = band_lo(band, k), jhi = band_hi(band, k);
    const int next_lo = k + 1 < nstrips ? band_lo(band, k + 1) : 1;
    const int prev_lo = k > 0 ? band_lo(band, k - 1) : 1, prev_hi = k > 0 ? band_hi(band, k - 1) : LB;
    const int W = jhi - jlo + 1;
    const int S = W + 31;
    const int wpl = tb_words_per_lane(W, R);
    // row buffers: the one this strip reads (previous strip's bottom row) and the one it writes
    // (checkpointed: the slot's row checkpoints k - 1 and k, indexed by column from 1)
    int4* rb_in = CK ? ck + (int64_t)(k - 1) * LB - 1
                     : coop ? rowbuf_base + (int64_t)((k - 1) & (kDpWarps - 1)) * J.rowbuf_stride : own_rowbuf;
    int4* rb_out = CK ? ck + (int64_t)k * LB - 1
                      : coop ? rowbuf_base + (int64_t)(k & (kDpWarps - 1)) * J.rowbuf_stride : own_rowbuf;
    const int producer = (k - 1) & (kDpWarps - 1);
    // cooperative mode: wait until the previous strip published column `col`
    auto wait_for = [&](int col) -> bool {
      if (!coop || k == 0) return true;
      if (col > prev_hi) col = prev_hi;
      if (col < prev_lo) return true;
      const unsigned long long need = ((unsigned long long)(k - 1) << 21) | (unsigned long long)col;
      bool ok = true;
      if (lane == 0) {
        long long spins = 0;
        while (sh.prog[producer] < need) {
          if (*(volatile int*)&sh.abort || ++spins > J.spin_limit) {
            ok = false;
            break;
          }
        }
        if (!ok) {
          *(volatile int*)&sh.abort = 1;
          set_error(J.err, kDevWatchdog);
        }
        __threadfence_block();
      }
      return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    };
    auto publish = [&](int col) {
      if (!coop) return;
      __syncwarp();
      if (lane == 31) {
        __threadfence_block();
        sh.prog[wib] = ((unsigned long long)k << 21) | (unsigned long long)col;
      }
    };
    DpLane<R> L;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = row0 + lane * R + r + 1;
      L.arow[r] = c_score_rows[(i <= LA ? A[i - 1] : 0u) & 3u];
    }
    // banded mode: prefix of the row maxima up to each owned row, the
    // strip's bottom row, and the column prefix at jlo-1 for lane 31
    int32_t rowpre[R];
    int32_t strip_pre = 0, run31 = 0, pb_next = 0;
    if (track) {
      // prefixes carried from the previous strip of this warp cover the
      // rows and columns up to it; only a gap (cooperative mode) is summed
      pa += warp_best_sum(A, pa_rows, row0, J.base_max);
      pa_rows = row0;
      int32_t lsum = 0;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = row0 + lane * R + r + 1;
        lsum += i <= LA ? best_of(J.base_max, A[i - 1]) : 0;
        rowpre[r] = lsum;
      }
      int32_t incl = lsum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) rowpre[r] += pa + incl - lsum;  // PA after row r
      strip_pre = pa + __shfl_sync(0xffffffffu, incl, 31);
      pb_lo += warp_best_sum(B, pb_lo_cols, jlo - 1, J.base_max);
      pb_lo_cols = jlo - 1;
      run31 = pb_lo;
      pb_next = pb_lo;  // prefix over B[0..next_lo-1), caught during the sweep
    }
    // Row above this strip at absolute column x: row 0 for the first strip,
    // else the previous strip's computed columns, its left boundary or -inf.
    // M is Mg throughout, except row 0's M at x > 0, which is read only
    // by matrix row 1, where the reference opens for free (M + 0), and as
    // a diagonal that can never win (-inf against at most -400).
    auto above = [&](int x) -> int4 {
      if (k == 0) return x == 0 ? make_int4(kGap, kNeg, kNeg, 0) : make_int4(kNeg, kNeg, 0, 0);
      if (x >= prev_lo && x <= prev_hi) return rb_in[x];
      if (x == prev_lo - 1) return prev_lo == 1 ? make_int4(kNeg + kGap, 0, kNeg, 0) : kNegCell;
      return kNegCell;
    };
    if (!wait_for(jlo + 63)) return;
    // prime the rings: B[jlo-1 .. jlo+62], row above at columns jlo .. jlo+63
    __syncwarp();
    ringB[lane] = jlo - 1 + lane < LB ? B[jlo - 1 + lane] : 0;
    ringB[32 + lane] = jlo + 31 + lane < LB ? B[jlo + 31 + lane] : 0;
    ringR[lane] = above(jlo + lane);
    ringR[32 + lane] = above(jlo + 32 + lane);
    const int4 dg0 = above(jlo - 1);
    __syncwarp();
    // left state (column jlo-1) per row: column 0 = (NEG, 0, NEG), else -inf
    const int32_t leftD = jlo == 1 ? 0 : kNeg;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      L.lM[r] = kNeg + kGap;
      L.lD[r] = leftD;
      L.lI[r] = kNeg;
    }
    int32_t pubM = kNeg + kGap, pubD = leftD, pubI = kNeg;  // bottom row, last computed column (M as Mg)
    int32_t upM = kNeg, upD = kNeg, upI = kNeg;      // row above, current column
    uint32_t acc = 0;
    const bool bottom_exit = track && lane == 31 && row0 + SR < LA;
    const bool writes_row = k + 1 < nstrips;
    bool alive = true;

    // one step; `checked` handles the wavefront's ramp-up and ramp-down
    auto step = [&](int s, bool checked) {
      if ((s & 31) == 0 && s > 0) {
        if ((s & 31) == 0 && writes_row && s >= 32) publish(jlo + s - 32);  // columns <= jlo+s-32 are written
        if (!wait_for(jlo + s + 63)) {
          alive = false;
          return;
        }
        // refill one chunk ahead: B at offsets s+32 .. s+63, row above at s+32 .. s+63
        __syncwarp();
        const int xb = jlo - 1 + s + 32 + lane;
        ringB[(s + 32 + lane) & 127] = xb < LB ? B[xb] : 0;
        ringR[(s + 32 + lane) & 63] = above(jlo + s + 32 + lane);
        __syncwarp();
      }
      const int jj = s - lane;  // column offset inside the strip
      const int j = jlo + jj;   // absolute column
      const int32_t rM = __shfl_up_sync(0xffffffffu, pubM, 1);
      const int32_t rD = __shfl_up_sync(0xffffffffu, pubD, 1);
      const int32_t rI = __shfl_up_sync(0xffffffffu, pubI, 1);
      const int4 v = ringR[s & 63];
      int32_t dgM = upM, dgD = upD, dgI = upI;
      if (s == 0 && lane == 0) {
        dgM = dg0.x;
        dgD = dg0.y;
        dgI = dg0.z;
      }
      upM = lane == 0 ? v.x : rM;
      upD = lane == 0 ? v.y : rD;
      upI = lane == 0 ? v.z : rI;
      const uint32_t bsel = (uint32_t)ringB[jj & 127] | 0x4440u;
      uint32_t nibs = 0;
      if (!checked || (jj >= 0 && jj < W)) {
        // column 1 (only in checked steps) opens for free
        if (CK) {
          if (checked)
            dp_column_score<R, true>(L, upM, upD, dgM, dgD, dgI, bsel, j == 1 ? -kGap : 0);
          else
            dp_column_score<R, false>(L, upM, upD, dgM, dgD, dgI, bsel, 0);
        } else {
          nibs = checked ? dp_column<R, true>(L, upM, upD, dgM, dgD, dgI, bsel, j == 1 ? -kGap : 0)
                         : dp_column<R, false>(L, upM, upD, dgM, dgD, dgI, bsel, 0);
        }
        if (checked && s == 0 && lane == 0 && k == 0 && LA == 1) {
          // NWSmall's last-row special case (MU/nwsmall.cpp:616-624) with
          // LA == 1: M(1,1) adds the open and close of position 0, and the
          // close of a one-position profile is not zeroed (stored as Mg).
          L.lM[0] = (int32_t)__byte_perm(L.arow[0], 0u, bsel) - kScoreBias + 2 * kGap;
          nibs = (nibs & ~3u) | TB_DM;
        }
        pubM = L.lM[R - 1];
        pubD = L.lD[R - 1];
        pubI = L.lI[R - 1];
        if (lane == 31 && writes_row) rb_out[j] = make_int4(pubM, pubD, pubI, 0);
        if (CK && ((jj + 1) & (kCkCols - 1)) == 0 && jj + 1 < W) {
          // column checkpoint: the state left of block (jj + 1) / kCkCols
          int4* col = ck + ck_col_entry(LA, LB, R, k, (jj + 1) / kCkCols) + lane * R;
#pragma unroll
          for (int r = 0; r < R; ++r) col[r] = make_int4(L.lM[r], L.lD[r], L.lI[r], 0);
        }
        if (track && lane == 31) {
          run31 += best_of(J.base_max, bsel);  // prefix over B[0..j)
          if (j == next_lo - 1) pb_next = run31;
          if (bottom_exit && j < next_lo) {
            const int32_t best = max(pubM - kGap, max(pubD, pubI));
            bound = max(bound, best + min(totA - strip_pre, totB - run31));
          }
        }
      } else if (jj == -1) {
        pubM = kNeg + kGap;
        pubD = leftD;
        pubI = kNeg;
      }
      if (CK) {
        // no traceback bits
      } else if (R == 8) {
        tbs[s * 32 + lane] = nibs;
      } else {  // 8/R steps per 32-bit word
        constexpr int kPer = 8 / R;
        acc |= nibs << (4 * R * (s % kPer));
        if ((s % kPer) == kPer - 1 || s == S - 1) {
          tbs[(s / kPer) * 32 + lane] = acc;
          acc = 0;
        }
      }
    };

    if (W >= 32) {
      // unchecked steps: every lane inside the strip and past column 1
      int s = 0;
      for (; s < 32 && alive; ++s) step(s, true);
      for (; s < W && alive; ++s) step(s, false);
      for (; s < S && alive; ++s) step(s, true);
    } else {
      for (int s = 0; s < S && alive; ++s) step(s, true);
    }
    if (!alive) return;
    if (writes_row) publish(jhi);  // whole bottom row written
    __syncwarp();
    // after the sweep each lane holds its rows' cells at column jhi
    if (k == end_strip && lane == end_lane) {
      int32_t eM = kNeg, eD = kNeg, eI = kNeg;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (r == end_r) {
          eM = L.lM[r] - kGap;
          eD = L.lD[r];
          eI = L.lI[r];
        }
      int32_t sc = eM;
      char e = 'M';
      if (eD > sc) {
        sc = eD;
        e = 'D';
      }
      if (eI > sc) {
        sc = eI;
        e = 'I';
      }
      J.scores[p] = sc;
      J.end_edge[p] = (uint8_t)e;
    }
    if (track) {
      // lane 31 swept every column of the strip: its running sum is the
      // prefix over B[0..jhi); carry the prefixes to this warp's next strip
      pb_hi = __shfl_sync(0xffffffffu, run31, 31);
      if (kstep == 1) {
        pa = strip_pre;
        pa_rows = row0 + SR;
        if (k + 1 < nstrips) {
          if (next_lo - 1 <= jhi) {  // lane 31 passed column next_lo-1 (or it is jlo-1)
            pb_lo = __shfl_sync(0xffffffffu, pb_next, 31);
            pb_lo_cols = next_lo - 1;
          } else {  // the next strip starts right of this one: sum the rest there
            pb_lo = pb_hi;
            pb_lo_cols = jhi;
          }
        }
      }
    }
    if (track && jhi < LB) {  // right-edge exits: an I step leaves the band
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = row0 + lane * R + r + 1;
        if (i <= LA) {
          const int32_t best = max(L.lM[r] - kGap, max(L.lD[r], L.lI[r]));
          bound = max(bound, best + min(totA - rowpre[r], totB - pb_hi));
        }
      }
    }
    // advance the traceback pointer past this warp's strip and the skipped ones
    if (!CK)
      for (int q = k; q < k + kstep && q < nstrips; ++q)
        tbs += (int64_t)tb_words_per_lane(band_hi(band, q) - band_lo(band, q) + 1, R) * 32;
  }
  if (BANDED) {
    // paths along row 0 past the band, or down column 0 past it (added once)
    if (track && kstart == 0) {
      const int hi0 = band_hi(band, 0);
      const int last_col0 = band_last_row_at_col1(band, LA);
      const int32_t pb0 = hi0 < LB ? warp_best_sum(B, 0, hi0, J.base_max) : 0;
      const int32_t pa0 = last_col0 < LA ? warp_best_sum(A, 0, last_col0, J.base_max) : 0;
      if (lane == 0) {
        if (hi0 < LB) bound = max(bound, min(totA, totB - pb0));
        if (last_col0 < LA) bound = max(bound, min(totA - pa0, totB));
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) bound = max(bound, __shfl_xor_sync(0xffffffffu, bound, d));
    if (coop) {
      if (lane == 0) atomicMax(&sh.bound, bound);
    } else {
      __syncwarp();
      if (lane == 0) J.accept[p] = J.scores[p] > bound ? 1 : 0;
    }
  }
}

template <bool BANDED, int R, bool CK = false>
__global__ void __launch_bounds__(kDpThreads, 2) k_gapdp_t(DpJob J) {
  __shared__ DpShared sh;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  int4* rowbuf_cta = J.rowbuf + (int64_t)blockIdx.x * kDpWarps * J.rowbuf_stride;
  int4* own_rowbuf = rowbuf_cta + (int64_t)wib * J.rowbuf_stride;
  // phase 1: large problems, one per CTA, strips pipelined across the warps
  for (;;) {
    if (threadIdx.x == 0) sh.claim = (int)atomicAdd(&J.counter[0], 1u);
    if (lane == 0) sh.prog[wib] = 0ull;
    if (threadIdx.x == 0) {
      sh.bound = kNeg;
      sh.abort = 0;
    }
    __syncthreads();
    const int w = sh.claim;
    if (w >= J.nbig) break;
    dp_solve<BANDED, R, CK>(J, sh, w, wib, kDpWarps, true, rowbuf_cta, own_rowbuf);
    __syncthreads();
    if (BANDED && threadIdx.x == 0) {
      const uint32_t p = J.order[w];
      J.accept[p] = (!sh.abort && J.scores[p] > sh.bound) ? 1 : 0;
    }
    __syncthreads();
  }
  // phase 2: small problems, one per warp
  for (;;) {
    int w = 0;
    if (lane == 0) w = J.nbig + (int)atomicAdd(&J.counter[1], 1u);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= J.nwork) break;
    dp_solve<BANDED, R, CK>(J, sh, w, 0, 1, false, rowbuf_cta, own_rowbuf);
  }
}

// Flags any byte above 3 in a concatenated code buffer.
__global__ void k_check_codes(const uint8_t* __restrict__ s, uint64_t n, uint32_t* err) {
  uint32_t bad = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t n16 = (((uintptr_t)s & 15) == 0) ? n / 16 : 0;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n16; q += stride) {
    const uint4 v = reinterpret_cast<const uint4*>(s)[q];
    bad |= (v.x | v.y | v.z | v.w) & 0xfcfcfcfcu;
  }
  for (uint64_t i = n16 * 16 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) bad |= s[i] & 0xfcu;
  if (bad) set_error(err, kDevBadBase);
}

}  // namespace mvg
