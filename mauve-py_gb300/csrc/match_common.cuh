// Device-side pieces of the seed matcher shared by the genome-pair matcher
// (match.cu) and the batched gap anchor search (gapsearch.cu): the hash
// entry, the unique-seed run test and its tile counts, MheCompare /
// Contains, the reference's lower_bound probe sequence and the warp
// ExtendMatch.  Included once per translation unit; nothing here has a
// host-side symbol except the k_pair_count template.
#pragma once
#include "mvg_internal.h"
#include "prim.cuh"

namespace mvg {

constexpr int kTableSize = 40000;  // LM/MemHash.h:30 DEFAULT_MEM_TABLE_SIZE

struct Mhe {
  int64_t s0, s1, len, off;
};

struct MatchCtx {
  const uint32_t* g[2];
  int64_t n[2];
  SeedDesc s;
};

// ------------------------------------------------------------------ join

// Both genomes' seeds sorted in one array by (seed bits, strand, genome).  A
// seed unique in each genome (counted once in each, strand ignored:
// LM/PairwiseMatchFinder.cpp:37-71 over LM/MatchFinder.cpp:172-340) is a run
// of equal seed bits with exactly two members, one per genome; runs come in
// ascending seed order, the reference's enumeration order.  Key i opens such
// a run when pair_flag(i).
template <typename K>
__device__ __forceinline__ bool pair_flag(const K* __restrict__ keys, int64_t n, int64_t i) {
  const uint64_t k0 = (uint64_t)keys[i], cur = k0 >> 2;
  if (i + 1 >= n || (i > 0 && ((uint64_t)keys[i - 1] >> 2) == cur)) return false;
  const uint64_t k1 = (uint64_t)keys[i + 1];
  return (k1 >> 2) == cur && ((k0 ^ k1) & 1ull) && (i + 2 == n || ((uint64_t)keys[i + 2] >> 2) != cur);
}

constexpr int kPairItems = 8;  // consecutive keys per thread
constexpr int kPairTile = 256 * kPairItems;

// Pass 1: the number of pairs opened in each tile of kPairTile keys.
template <typename K>
__global__ void __launch_bounds__(256) k_pair_count(const K* __restrict__ keys, int64_t n, uint32_t* __restrict__ bsum) {
  const int64_t i0 = (int64_t)blockIdx.x * kPairTile + (int64_t)threadIdx.x * kPairItems;
  uint32_t c = 0;
#pragma unroll 4
  for (int k = 0; k < kPairItems; ++k)
    if (i0 + k < n) c += pair_flag(keys, n, i0 + k);
  for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
  __shared__ uint32_t ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; ++w) t += ws[w];
    bsum[blockIdx.x] = t;
  }
}

// ------------------------------------------------------- bucket replay

// LM/MatchHashEntry.cpp:164-200 (Contains), two genomes, both present.
__device__ __forceinline__ bool mhe_contains(const Mhe& c, const Mhe& m) {
  if (c.off != m.off) return false;
  const int64_t diff = m.s0 - c.s0;
  if (c.s0 == 0) return false;
  if (diff < 0 || (uint64_t)c.len < (uint64_t)(m.len + diff)) return false;
  const int64_t diff_rc = m.len - c.len + diff;
  const int64_t diff_i = m.s1 - c.s1;
  if (m.s1 == 0 && c.s1 == 0) return true;
  if (m.s1 < 0 && diff_rc == diff_i) return true;
  return diff == diff_i;
}

// LM/MatchHashEntry.cpp:48-67 (strict_start_lessthan_ptr).
__device__ __forceinline__ bool mhe_strict_lt(const Mhe& a, const Mhe& b, int L) {
  int64_t x = a.s0 < 0 ? -a.s0 + a.len - L : a.s0;
  int64_t y = b.s0 < 0 ? -b.s0 + b.len - L : b.s0;
  if (x != y) return x < y;
  x = a.s1 < 0 ? -a.s1 + a.len - L : a.s1;
  y = b.s1 < 0 ? -b.s1 + b.len - L : b.s1;
  if (x != y) return x < y;
  return false;
}

// LM/MatchHashEntry.h:121-143 (MheCompare) for pairwise entries.
__device__ __forceinline__ bool mhe_less(const Mhe& a, const Mhe& b, int L) {
  if (mhe_contains(a, b) || mhe_contains(b, a)) return false;
  return mhe_strict_lt(a, b, L);
}

// std::lower_bound's bisection: the comparator is not a strict weak order,
// so the probe sequence decides which entry is tested and is kept exactly.
__device__ __forceinline__ int64_t lower_bound_mhe(const Mhe* __restrict__ v, int64_t n, const Mhe& x, int L) {
  int64_t first = 0, len = n;
  while (len > 0) {
    int64_t half = len >> 1, mid = first + half;
    if (mhe_less(v[mid], x, L)) {
      first = mid + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  return first;
}

// ExtendMatch (LM/MatchFinder.h:218-374) for two genomes, executed by a full
// warp.  The reference cycles through four phases (jump left and right by
// the seed length until the first mismatching window, then try the L
// single-base offsets left and right and move to the furthest matching one)
// and restarts while a single-base phase moves.
//
// Every window pair a phase tests lies on the match's diagonal: in the entry
// orientation S0, the pair tested at step size k from the current left edge
// is the pair at displacement ML + k from the entry left edge (ML = total
// moved in even phases), and in the inverted orientation the pair at MR + k
// from the entry right edge (MR = total moved in odd phases); positive
// starts move by exactly those amounts and negative starts stay.  The room
// a phase has (the genome-end clamp) is likewise C - ML or C' - MR.  So the
// two sides never interact: each side's total is the fixpoint of (jump,
// single) on its own match bits, and the four-phase cycle only interleaves
// the two fixpoint iterations.  Here the warp computes the two fixpoints one
// after the other on match bits cached in per-warp shared rings (1024
// displacements per fill); the walk itself is warp-uniform scalar work.
// For a same-strand pair a window pair matches iff the pattern-selected
// bases are equal (equal canonical mers with equal strand bits); other
// pairs use the canonical-mer test itself.
constexpr int kExtRing = 128;    // words per side: the last 4096 displacements
constexpr int kExtChunk = 1024;  // displacements per fill (32 per lane)

struct ExtRing {
  uint32_t w[2][kExtRing];
};

// 2-bit mask of the pattern's bases in a 64-bit window (base 0 in bits 63:62).
__device__ __forceinline__ uint64_t pattern_mask64(const SeedDesc& s) {
  uint64_t m = 0;
  for (int r = 0; r < s.nruns; ++r)
    for (int b = 0; b < s.run_len[r]; ++b) m |= 3ull << (62 - 2 * (s.run_start[r] + b));
  return m;
}

// Window start (0-based) in genome q of the pair at displacement u from the
// entry state's edge (st, len), or -1 outside the genome.
__device__ __forceinline__ int64_t ext_start(int64_t st, int64_t len, int64_t u, int L, int64_t n) {
  if (st > 0 && u >= st) return -1;  // a left step past the genome start (the phases never take it)
  const int64_t sq = st > 0 ? st - u : st;
  const int64_t get = sq < 0 ? -sq + len + u - L : sq;
  const int64_t x = get - 1;
  return (x >= 0 && x + L <= n) ? x : -1;
}

// 64 bases (128 bits, big-endian, base p in bits 127:126) from 2-bit words;
// reads words p/16 .. p/16 + 4.
__device__ __forceinline__ void window128(const uint32_t* __restrict__ g, uint64_t p, uint64_t& hi, uint64_t& lo) {
  const uint64_t q = p >> 4;
  const uint32_t sh = (uint32_t)(p & 15) * 2;
  const uint64_t H = ((uint64_t)__ldg(g + q) << 32) | __ldg(g + q + 1);
  const uint64_t M = ((uint64_t)__ldg(g + q + 2) << 32) | __ldg(g + q + 3);
  const uint32_t T = __ldg(g + q + 4);
  if (sh == 0) {
    hi = H;
    lo = M;
  } else {
    hi = (H << sh) | (M >> (64 - sh));
    lo = (M << sh) | (uint64_t)(T >> (32 - sh));
  }
}

static __device__ void ext_fill(const MatchCtx& c, int64_t st0, int64_t st1, int64_t len, int64_t u0, uint64_t pmask,
                         uint32_t* ring) {
  const int lane = threadIdx.x & 31;
  const int L = c.s.L;
  const bool same = (st0 > 0) == (st1 > 0);
  uint32_t word = 0;
  bool done = false;
  // Same-strand pairs: the lane's 32 windows lie in one 64-base stretch of
  // each genome (both move the same way with u), so one XOR of the two
  // stretches gives all 32 window tests.
  if (same) {
    const int64_t U = u0 + lane * 32;
    const int64_t a0 = ext_start(st0, len, U, L, c.n[0]), a31 = ext_start(st0, len, U + 31, L, c.n[0]);
    const int64_t b0 = ext_start(st1, len, U, L, c.n[1]), b31 = ext_start(st1, len, U + 31, L, c.n[1]);
    const bool down = st0 > 0;  // window starts decrease with u
    const int64_t amin = down ? a31 : a0, bmin = down ? b31 : b0;
    if (a0 >= 0 && a31 >= 0 && b0 >= 0 && b31 >= 0 && amin + 80 <= c.n[0] && bmin + 80 <= c.n[1]) {
      uint64_t ah, al, bh, bl;
      window128(c.g[0], (uint64_t)amin, ah, al);
      window128(c.g[1], (uint64_t)bmin, bh, bl);
      const uint64_t dh = ah ^ bh, dl = al ^ bl;
#pragma unroll 4
      for (int t = 0; t < 32; ++t) {
        const int j = down ? 31 - t : t;  // window start amin + j
        const uint64_t w = j == 0 ? dh : ((dh << (2 * j)) | (dl >> (64 - 2 * j)));
        word |= (uint32_t)((w & pmask) == 0) << t;
      }
      if (U == 0) word &= ~1u;  // displacement 0 is not a step
      done = true;
    }
  }
  for (int t = 0; t < 32 && !done; ++t) {
    const int64_t u = u0 + lane * 32 + t;
    const int64_t xa = ext_start(st0, len, u, L, c.n[0]);
    const int64_t xb = ext_start(st1, len, u, L, c.n[1]);
    bool b = false;
    if (u >= 1 && xa >= 0 && xb >= 0) {
      if (same) {
        b = ((window64(c.g[0], (uint64_t)xa) ^ window64(c.g[1], (uint64_t)xb)) & pmask) == 0;
      } else {
        const uint64_t ca = canonical_mer(c.g[0], (uint64_t)xa, c.s);
        const uint64_t cb = canonical_mer(c.g[1], (uint64_t)xb, c.s);
        const bool pa = st0 > 0 ? !(ca & 1ull) : (bool)(ca & 1ull);
        const bool pb = st1 > 0 ? !(cb & 1ull) : (bool)(cb & 1ull);
        b = (ca & c.s.seed_mask) == (cb & c.s.seed_mask) && pa == pb;
      }
    }
    word |= (uint32_t)b << t;
  }
  ring[((u0 >> 5) + lane) & (kExtRing - 1)] = word;
  __syncwarp();
}

static __device__ void warp_extend(const MatchCtx& c, Mhe& m, ExtRing& R) {
  const int lane = threadIdx.x & 31;
  const int L = c.s.L;
  const uint64_t pmask = pattern_mask64(c.s);
  const int64_t e0 = m.s0, e1 = m.s1, elen = m.len;  // entry state S0
  int64_t moved[2] = {0, 0};                          // ML, MR
#pragma unroll 1
  for (int sd = 0; sd < 2; ++sd) {
    const int64_t sg = sd == 0 ? 1 : -1;
    const int64_t s0 = sg * e0, s1 = sg * e1;
    // room of this side: min over both genomes of the distance to the end
    const int64_t r0 = s0 > 0 ? s0 - 1 : (s0 < 0 ? c.n[0] - elen + s0 + 1 : -1);
    const int64_t r1 = s1 > 0 ? s1 - 1 : (s1 < 0 ? c.n[1] - elen + s1 + 1 : -1);
    const int64_t room0 = r0 < r1 ? r0 : r1;
    uint32_t* ring = R.w[sd];
    int64_t filled = 0;
    auto ensure = [&](int64_t umax) {
      while (filled <= umax) {
        ext_fill(c, s0, s1, elen, filled, pmask, ring);
        filled += kExtChunk;
      }
    };
    auto bit = [&](int64_t u) -> bool { return (ring[(u >> 5) & (kExtRing - 1)] >> (u & 31)) & 1u; };
    int64_t u = 0;
    for (;;) {
      // jump phase: k-1 good jumps before the first mismatching window
      int64_t room = room0 - u;
      const int64_t nj = room >= L ? room / L : 0;
      // 32 jumps per ballot: lane t tests jump kb + t
      int64_t good = nj;
      for (int64_t kb = 1; kb <= nj; kb += 32) {
        const int64_t klast = kb + 31 < nj ? kb + 31 : nj;
        ensure(u + klast * L);
        const int64_t kk = kb + lane;
        const bool miss = kk <= nj && !bit(u + kk * L);
        const unsigned mm = __ballot_sync(0xffffffffu, miss);
        if (mm) {
          good = kb - 1 + (__ffs(mm) - 1);
          break;
        }
      }
      u += good * L;
      // single-base phase: the furthest matching offset in 1..min(room, L)
      room = room0 - u;
      const int64_t ms = room > 0 ? (room < L ? room : L) : 0;
      if (ms <= 0) break;
      ensure(u + ms);
      // bits of displacements u+1 .. u+ms (ms <= 32): the highest set one
      const int64_t b0 = u + 1;
      const uint64_t two = ((uint64_t)ring[((b0 >> 5) + 1) & (kExtRing - 1)] << 32) |
                           ring[(b0 >> 5) & (kExtRing - 1)];
      uint64_t win = two >> (b0 & 31);
      win &= ms >= 64 ? ~0ull : ((1ull << ms) - 1);
      if (!win) break;
      u += 64 - __clzll(win);
    }
    moved[sd] = u;
  }
  m.len = elen + moved[0] + moved[1];
  m.s0 = e0 > 0 ? e0 - moved[0] : e0 + moved[1];
  m.s1 = e1 > 0 ? e1 - moved[0] : e1 + moved[1];
}

// lower_bound_mhe over the sorted order given by a map (logical position ->
// slot in E): the same probes on the same logical array.
__device__ __forceinline__ int64_t lower_bound_mapped(const Mhe* __restrict__ E, const uint32_t* __restrict__ M,
                                                      int64_t n, const Mhe& x, int L) {
  int64_t first = 0, len = n;
  while (len > 0) {
    int64_t half = len >> 1, mid = first + half;
    if (mhe_less(E[M[mid]], x, L)) {
      first = mid + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  return first;
}

}  // namespace mvg
