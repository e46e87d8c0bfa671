// The banded NWSmall kernel on a ring schedule (included by gapdp.cu after
// gapdp_kernel.cuh, whose recurrences and bound it shares).
//
// One warp solves one problem.  Rows are cut into groups of R (RingBand,
// band.h); lane g mod 32 runs group g, and the 32 lanes form a ring: lane t
// receives the bottom row of the group above it from lane t-1, lane 0 from
// lane 31, through one rotating shuffle per step.  Every group is as wide as
// the band (W columns) and starts one step after its predecessor reached the
// group's first column, so a lane never sweeps the staircase that a 32*R-row
// strip spans on a diagonal band, and there is no ramp-up or ramp-down per
// strip: the ring runs from the first group's start to the last group's end.
// A lane idles between its groups when the band is narrow for R; the host
// picks the smallest R whose schedule is valid (ring_eligible), which keeps
// lanes busy most of the time.
//
// Exactness: the kept region is a union of group rectangles.  A banded score
// is accepted only when it is strictly above an upper bound on every path
// that leaves the region, as in the strip kernel: each cell a path can leave
// from (the bottom row of a group left of the next group's first column, the
// right-most column of a group short of LB, row 0 right of group 0, column 0
// below the last group that reaches it) contributes its score plus
// min(sum of A's best-base scores below it, sum of B's right of it).  The
// prefix sums travel along the ring with each group start.
//
// Traceback words: each lane writes its R nibbles per step as one stream;
// nibble s*R + r of lane t is in word ((s*R + r) / 8) * 32 + t, so every
// store is one coalesced 128-byte row.
#pragma once
#include <limits.h>

#include "band.h"

namespace mvg {

struct RingJob {
  const uint8_t* sa;
  const uint64_t* oa;
  const uint8_t* sb;
  const uint64_t* ob;
  const uint32_t* order;   // problem ids of this launch, largest first
  const uint64_t* tb_off;  // byte offset of each slot's traceback words
  int nwork;
  uint32_t* tb;
  int32_t* scores;
  uint8_t* end_edge;
  const int32_t* band_delta;
  const int32_t* band_half;
  uint8_t* accept;
  uint32_t base_max;
  unsigned* counter;
  unsigned long long* cells;  // kept cells inside the matrix, summed over problems
};

constexpr int kRingThreads = 128;
constexpr int kRingA = 256;  // rows of A staged per warp (codes of the next groups to start)

// One column segment of R rows, as dp_column, with the R traceback nibbles
// returned in (R + 7) / 8 words (nibble r in word r / 8).
template <int R>
__device__ __forceinline__ void ring_column(DpLane<R>& L, int32_t upM, int32_t upD, int32_t dgM, int32_t dgD,
                                            int32_t dgI, uint32_t bsel, int32_t goB, int32_t goA0,
                                            uint32_t (&nw)[(R + 7) / 8]) {
  int32_t cuM = upM, cuD = upD;
  int32_t cdM = dgM, cdD = dgD, cdI = dgI;
#pragma unroll
  for (int q = 0; q < (R + 7) / 8; ++q) nw[q] = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int32_t goA = r == 0 ? goA0 : kGap;
    bool dm;
    const int32_t D = __vibmax_s32(cuM + goA, cuD, &dm);
    bool mi;
    const int32_t I = __vibmax_s32(L.lM[r] + goB, L.lI[r], &mi);
    bool dge, mge;
    const int32_t DI = __vibmax_s32(cdD, cdI, &dge) + kGap;
    const int32_t best = __vibmax_s32(cdM, DI, &mge);
    const int32_t M = best + (int32_t)__byte_perm(L.arow[r], 0u, bsel) - kScoreBias;
    const uint32_t tm = mge ? TB_MM : (dge ? TB_DM : TB_IM);
    nw[r >> 3] |= (tm | (dm ? TB_MD : 0u) | (mi ? TB_MI : 0u)) << (4 * (r & 7));
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

template <int R>
__device__ void ring_solve(const RingJob& J, uint8_t* ringB, uint8_t* ringA, int w) {
  constexpr int NW = (R + 7) / 8;
  const int lane = threadIdx.x & 31;
  const int src = (lane + 31) & 31;  // the ring's previous lane
  const uint32_t p = J.order[w];
  const uint64_t a0 = J.oa[p], b0 = J.ob[p];
  const int LA = (int)(J.oa[p + 1] - a0), LB = (int)(J.ob[p + 1] - b0);
  const uint8_t* A = J.sa + a0;
  const uint8_t* B = J.sb + b0;
  const RingBand b = make_ring_band(LA, LB, J.band_delta[p], J.band_half[p], R);
  const int G = b.G, W = b.W, lo0 = b.lo0;
  const int S = (int)b.steps;
  const int32_t totA = warp_best_sum(A, 0, LA, J.base_max);
  const int32_t totB = warp_best_sum(B, 0, LB, J.base_max);

  // warp-uniform: the next group to start, its first column, and the band
  // centre floor((gR+1)*LB/LA) of that group kept as quotient f, remainder m
  int gnext = 0;
  int f = LB / LA, m = LB % LA;
  const int qR = (int)((int64_t)R * LB / LA), rR = (int)((int64_t)R * LB % LA);
  const int shift = b.delta - b.half;
  int lo_next = f + shift;  // == lo0
  int lo_started = lo0;     // first column of the last group started
  int filled = lo0 - 1;     // ringB holds the B codes of columns (filled-128, filled]
  int filledA = 0;          // ringA holds rows [filledA - kRingA, filledA) of A

  // this lane's group
  int my_g = -1, my_end = INT_MIN, prev_hi = INT_MIN, next_lo = INT_MIN, end_col = INT_MIN, rexit_col = INT_MIN;
  int32_t goA0 = kGap, topI = kNeg, pa_end = 0, pb = 0;
  DpLane<R> L;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    L.arow[r] = 0;
    L.lM[r] = kNeg;
    L.lD[r] = kNeg;
    L.lI[r] = kNeg;
  }
  int32_t pubM = kNeg, pubD = kNeg, pubI = kNeg;     // this lane's bottom row, last column
  int32_t dgM = kNeg, dgD = kNeg, dgI = kNeg;        // cell above-left of the next column
  int32_t rawM = kNeg, rawD = kNeg, rawI = kNeg;     // what the previous lane published one step ago
  int32_t bound = kNeg, endsc = kNeg;
  int end_lane_edge = 0;
  uint32_t kept = 0;
  uint32_t acc = 0;
  uint32_t* tbp = J.tb + J.tb_off[w] / 4 + lane;

  for (int s = 0; s < S; ++s) {
    const int32_t rM = __shfl_sync(0xffffffffu, pubM, src);
    const int32_t rD = __shfl_sync(0xffffffffu, pubD, src);
    const int32_t rI = __shfl_sync(0xffffffffu, pubI, src);
    if (gnext < G && s - gnext == lo_next - lo0) {
      // A codes of the rows about to start, staged 128 rows at a time
      if (filledA < (gnext + 1) * R) {
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int i = filledA + k * 32 + lane;
          ringA[i & (kRingA - 1)] = i < LA ? A[i] : 0;
        }
        __syncwarp();
        filledA += 128;
      }
      // group gnext starts on lane gnext % 32; its predecessor (previous
      // lane) passes the prefix sums it carries
      const int32_t chain_pb = __shfl_sync(0xffffffffu, pb, src);
      const int32_t chain_pa = __shfl_sync(0xffffffffu, pa_end, src);
      const int g = gnext;
      const int lo_prev = lo_started;
      f += qR;
      m += rR;
      if (m >= LA) {
        m -= LA;
        ++f;
      }
      const int lo_after = f + shift;
      if (lane == (g & 31)) {
        const int my_lo = lo_next;
        my_g = g;
        my_end = my_lo + W - 1;
        prev_hi = g == 0 ? INT_MIN : lo_prev + W - 1;
        next_lo = g + 1 < G ? lo_after : INT_MIN;
        end_col = g == G - 1 ? LB : INT_MIN;
        rexit_col = my_end < LB ? my_end : INT_MIN;
        const int rows_here = LA - g * R < R ? LA - g * R : R;
        // cells of this group inside the matrix
        const int c0 = my_lo < 1 ? 1 : my_lo, c1 = my_end < LB ? my_end : LB;
        if (c1 >= c0) kept += (uint32_t)rows_here * (uint32_t)(c1 - c0 + 1);
        goA0 = g == 0 ? 0 : kGap;
        topI = g == 0 ? 0 : kNeg;
        int32_t pa = g == 0 ? 0 : chain_pa;
        if constexpr (R % 4 == 0) {  // the group's codes as whole words
          const uint32_t* ra = reinterpret_cast<const uint32_t*>(ringA);
#pragma unroll
          for (int q = 0; q < R / 4; ++q) {
            const uint32_t c4 = ra[((g * R) >> 2) + q & (kRingA / 4 - 1)];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int r = 4 * q + k;
              const uint32_t code = (c4 >> (8 * k)) & 3u;
              L.arow[r] = c_score_rows[code];
              if (r < rows_here) pa += best_of(J.base_max, code);
            }
          }
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const uint32_t code = ringA[(g * R + r) & (kRingA - 1)] & 3u;
            L.arow[r] = c_score_rows[code];
            if (r < rows_here) pa += best_of(J.base_max, code);
          }
        }
        pa_end = pa;
        // prefix of B's best scores before column my_lo: the predecessor
        // has just added column my_lo
        pb = (g == 0 || my_lo <= 0) ? 0 : chain_pb - best_of(J.base_max, ringB[my_lo & 127]);
        const int32_t leftD = my_lo - 1 == 0 ? 0 : kNeg;  // column 0 is (-inf, 0, -inf) below row 0
#pragma unroll
        for (int r = 0; r < R; ++r) {
          L.lM[r] = kNeg;
          L.lD[r] = leftD;
          L.lI[r] = kNeg;
        }
        // cell above-left of the first column: (gR, my_lo - 1)
        const int x = my_lo - 1;
        if (g == 0) {  // row 0: M(0,0) = 0, I(0,j) = 0 for j >= 1
          dgM = x == 0 ? 0 : kNeg;
          dgD = kNeg;
          dgI = x >= 1 ? 0 : kNeg;
        } else if (x <= 0) {
          dgM = kNeg;
          dgD = x == 0 ? 0 : kNeg;
          dgI = kNeg;
        } else if (x >= lo_prev) {  // the predecessor computed it two steps ago
          dgM = rawM;
          dgD = rawD;
          dgI = rawI;
        } else {
          dgM = kNeg;
          dgD = kNeg;
          dgI = kNeg;
        }
      }
      lo_started = lo_next;
      lo_next = lo_after;
      ++gnext;
    }
    // B codes of the running groups' columns: up to s - (gnext - 32) + lo0
    if (filled < s + 32 - gnext + lo0) {
      const int x = filled + 1 + lane;
      __syncwarp();
      ringB[x & 127] = (x >= 1 && x <= LB) ? B[x - 1] : 0;
      __syncwarp();
      filled += 32;
    }
    const int j = s - my_g + lo0;
    // the cell above: the predecessor's bottom row while inside its range;
    // for group 0 row 0 (I = 0 right of column 0; M(0,0) is set below)
    const bool from_ring = j <= prev_hi;
    int32_t aM = from_ring ? rM : kNeg;
    const int32_t aD = from_ring ? rD : kNeg;
    int32_t aI = from_ring ? rI : topI;
    uint32_t nw[NW];
#pragma unroll
    for (int q = 0; q < NW; ++q) nw[q] = 0;
    if (j <= my_end && j >= 1 && j <= LB && my_g >= 0) {
      const uint32_t bsel = (uint32_t)ringB[j & 127] | 0x4440u;
      ring_column<R>(L, aM, aD, dgM, dgD, dgI, bsel, j == 1 ? 0 : kGap, goA0, nw);
      if (LA == 1 && j == 1) {
        // NWSmall's last-row special case (MU/nwsmall.cpp:616-624) with
        // LA == 1: M(1,1) adds the open and close of position 0
        L.lM[0] = (int32_t)__byte_perm(L.arow[0], 0u, bsel) - kScoreBias + kGap;
        nw[0] = (nw[0] & ~3u) | TB_DM;
      }
      pubM = L.lM[R - 1];
      pubD = L.lD[R - 1];
      pubI = L.lI[R - 1];
      pb += (int32_t)__byte_perm(J.base_max, 0u, bsel) - kScoreBias;  // prefix over B[0..j)
      if (j < next_lo) {  // bottom-row exit
        const int32_t best = max(pubM, max(pubD, pubI));
        bound = max(bound, best + min(totA - pa_end, totB - pb));
      }
      if (j == end_col) {  // the end cell (LA, LB)
        const int er = LA - 1 - my_g * R;
        int32_t eM = kNeg, eD = kNeg, eI = kNeg;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r == er) {
            eM = L.lM[r];
            eD = L.lD[r];
            eI = L.lI[r];
          }
        int32_t sc = eM;
        int e = 'M';
        if (eD > sc) {
          sc = eD;
          e = 'D';
        }
        if (eI > sc) {
          sc = eI;
          e = 'I';
        }
        endsc = sc;
        end_lane_edge = e;
      }
      if (j == rexit_col) {  // right-edge exits of every row
        // the rows' best scores are the largest bytes of their score rows;
        // A's prefix before the group is pa_end minus their sum
        const int rows_here = LA - my_g * R < R ? LA - my_g * R : R;
        int32_t run = pa_end;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const uint32_t h = __vmaxu4(L.arow[r], L.arow[r] >> 16);
          if (r < rows_here) run -= (int32_t)max(h & 0xffu, (h >> 8) & 0xffu) - kScoreBias;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r < rows_here) {
            const uint32_t h = __vmaxu4(L.arow[r], L.arow[r] >> 16);
            run += (int32_t)max(h & 0xffu, (h >> 8) & 0xffu) - kScoreBias;
            const int32_t best = max(L.lM[r], max(L.lD[r], L.lI[r]));
            bound = max(bound, best + min(totA - run, totB - pb));
          }
        }
      }
    } else if (j <= my_end && j <= 0 && my_g >= 0) {
      // the left boundary column (D = 0 below row 0) or outside the matrix
      const int32_t d0 = j == 0 ? 0 : kNeg;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        L.lM[r] = kNeg;
        L.lD[r] = d0;
        L.lI[r] = kNeg;
      }
      pubM = kNeg;
      pubD = d0;
      pubI = kNeg;
      if (my_g == 0 && j == 0) {  // cell (0, 0)
        aM = 0;
        aI = kNeg;
      }
    } else {
      pubM = kNeg;
      pubD = kNeg;
      pubI = kNeg;
    }
    if constexpr (R < 8 && 8 % R == 0) {
      constexpr int kPer = 8 / R;
      acc |= nw[0] << (4 * R * (s % kPer));
      if ((s % kPer) == kPer - 1 || s == S - 1) {
        *tbp = acc;
        tbp += 32;
        acc = 0;
      }
    } else {
#pragma unroll
      for (int q = 0; q < NW; ++q) tbp[q * 32] = nw[q];
      tbp += NW * 32;
    }
    dgM = aM;
    dgD = aD;
    dgI = aI;
    rawM = rM;
    rawD = rD;
    rawI = rI;
  }
  // paths along row 0 past group 0, and down column 0 past the last group
  // that reaches it (both score 0 up to the exit)
  const int hi0 = lo0 + W - 1;
  const int32_t pb0 = hi0 < LB ? warp_best_sum(B, 0, hi0, J.base_max) : 0;
  int gcol = 0;
  while (gcol + 1 < G && ring_lo(b, gcol + 1) <= 1) ++gcol;
  const int last_col0 = (gcol + 1) * R;
  const int32_t pa0 = last_col0 < LA ? warp_best_sum(A, 0, last_col0, J.base_max) : 0;
  if (lane == 0) {
    if (hi0 < LB) bound = max(bound, min(totA, totB - pb0));
    if (last_col0 < LA) bound = max(bound, min(totA - pa0, totB));
  }
  unsigned long long kept64 = kept;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    bound = max(bound, __shfl_xor_sync(0xffffffffu, bound, d));
    kept64 += __shfl_xor_sync(0xffffffffu, kept64, d);
  }
  const int end_lane = (G - 1) & 31;
  const int32_t sc = __shfl_sync(0xffffffffu, endsc, end_lane);
  if (lane == end_lane) {
    J.scores[p] = sc;
    J.end_edge[p] = (uint8_t)end_lane_edge;
  }
  if (lane == 0) {
    J.accept[p] = sc > bound ? 1 : 0;
    if (J.cells) atomicAdd(J.cells, kept64);
  }
}

template <int R>
__global__ void __launch_bounds__(kRingThreads) k_gapdp_ring(RingJob J) {
  __shared__ uint8_t ringB[kRingThreads / 32][128];
  __shared__ __align__(16) uint8_t ringA[kRingThreads / 32][kRingA];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  for (;;) {
    int w = 0;
    if (lane == 0) w = (int)atomicAdd(J.counter, 1u);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= J.nwork) break;
    ring_solve<R>(J, ringB[wib], ringA[wib], w);
  }
}

// BitTraceBack (MU/bittraceback.cpp:138-210) over the ring layout, one
// thread per accepted problem; the path is written reversed at the end of
// the problem's slot, as k_traceback does.
__global__ void k_traceback_ring(const uint64_t* __restrict__ oa, const uint64_t* __restrict__ ob,
                                 const uint32_t* __restrict__ order, const uint8_t* __restrict__ rows_of,
                                 const uint64_t* __restrict__ tb_off, int nwork, const uint32_t* __restrict__ tb,
                                 const uint8_t* __restrict__ end_edge, const int32_t* __restrict__ band_delta,
                                 const int32_t* __restrict__ band_half, const uint8_t* __restrict__ accept,
                                 const uint64_t* __restrict__ path_off, char* __restrict__ paths,
                                 int64_t* __restrict__ path_len, uint32_t* err, int long_path) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += gridDim.x * blockDim.x) {
    const uint32_t p = order[w];
    if (!accept[p]) continue;
    const int LA = (int)(oa[p + 1] - oa[p]), LB = (int)(ob[p + 1] - ob[p]);
    if (LA + LB >= long_path) continue;  // k_traceback_win walks it
    const int R = rows_of[w];
    const RingBand b = make_ring_band(LA, LB, band_delta[p], band_half[p], R);
    const uint32_t* T = tb + tb_off[w] / 4;
    char* out = paths + path_off[p] + (LA + LB);
    int pa = LA, pb = LB;
    char cur = (char)end_edge[p];
    int64_t n = 0;
    const int64_t limit = (int64_t)LA + LB;
    int gc = -1, loc = 0, gc8 = -1, loc8 = 0;  // first column of the last group looked up (and 8 cells back)
    for (;;) {
      if (n >= limit) {
        set_error(err, kDevCapacity);
        break;
      }
      *(--out) = cur;
      ++n;
      uint32_t bits = 0;
      if (pa >= 1 && pb >= 1) {
        const int g = (pa - 1) / R, r = (pa - 1) - g * R;
        if (g != gc) {
          gc = g;
          loc = ring_lo(b, g);
        }
        if (pb < loc || pb > loc + b.W - 1) {  // outside an accepted band cannot happen
          set_error(err, kDevCapacity);
          break;
        }
        int64_t word;
        int sh;
        ring_tb_at(R, (int64_t)(pb + g - b.lo0), r, word, sh);
        bits = (T[word * 32 + (g & 31)] >> sh) & 15u;
        // start fetching the word of the cell 8 steps further along the
        // diagonal (most steps are matches), which may lie in another group
        // and column: each step's word is otherwise a dependent miss
        if (pa > 8 && pb > 8) {
          const int pa8 = pa - 8, pb8 = pb - 8;
          const int g8 = (pa8 - 1) / R, r8 = (pa8 - 1) - g8 * R;
          if (g8 != gc8) {
            gc8 = g8;
            loc8 = ring_lo(b, g8);
          }
          if (pb8 >= loc8 && pb8 <= loc8 + b.W - 1) {
            int64_t w8;
            int sh8;
            ring_tb_at(R, (int64_t)(pb8 + g8 - b.lo0), r8, w8, sh8);
            asm volatile("prefetch.global.L2 [%0];" ::"l"(T + w8 * 32 + (g8 & 31)));
          }
        }
      }
      char next;
      if (cur == 'M') {
        const uint32_t x = bits & 3u;
        next = x == TB_MM ? 'M' : (x == TB_DM ? 'D' : 'I');
        --pa;
        --pb;
      } else if (cur == 'D') {
        next = (bits & TB_MD) ? 'M' : 'D';
        --pa;
      } else {
        next = (bits & TB_MI) ? 'M' : 'I';
        --pb;
      }
      if (pa == 0 && pb == 0) break;
      if (pa < 0 || pb < 0) {
        set_error(err, kDevCapacity);
        break;
      }
      cur = next;
    }
    path_len[p] = n;
  }
}

}  // namespace mvg
