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
// two sides never interact: each side's total is where its own walk stops.
// The match bits are filled 1024 displacements at a time into a per-warp
// ring, and each fill's 32 words are searched for the stop (stop_in_word),
// one word per lane.  For a same-strand pair a window pair matches iff the
// pattern-selected bases are equal (equal canonical mers with equal strand
// bits); other pairs use the canonical-mer test itself.
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

// Reverse complement of 32 bases in 64 bits (complement = the 2-bit code
// inverted; base order reversed).
__device__ __forceinline__ uint64_t revcomp64(uint64_t x) {
  const uint64_t r = __brevll(~x);  // groups reversed, bits inside groups swapped
  return ((r >> 1) & 0x5555555555555555ull) | ((r & 0x5555555555555555ull) << 1);
}

// The top 64 bits of the 128-bit value hi:lo shifted left by s (0 <= s < 128).
__device__ __forceinline__ uint64_t top64(uint64_t hi, uint64_t lo, int s) {
  if (s == 0) return hi;
  if (s < 64) return (hi << s) | (lo >> (64 - s));
  return lo << (s - 64);
}

// One warp's fill: match bits of displacements u0 .. u0 + 32 * nlanes - 1
// into ring words (u0 / 32 + lane) mod RING, lanes below nlanes (no
// synchronisation).
template <int RING>
__device__ __forceinline__ void ext_fill_ring(const MatchCtx& c, int64_t st0, int64_t st1, int64_t len, int64_t u0,
                                              uint64_t pmask, uint32_t* ring, int nlanes = 32) {
  if ((int)(threadIdx.x & 31) >= nlanes) return;
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
  } else if (c.s.sym) {
    // Opposite strands with a symmetric pattern.  Per window the reference's
    // test is "canonical mers equal and strands opposite", which for a mer
    // set {f, rc(f)} means: B's forward mer is the reverse complement of A's,
    // and A's mer is not its own reverse complement (then both canonical
    // forms are the forward one).  With a symmetric pattern rc(mer(x)) =
    // mer(rc(x)), so both are masked window comparisons: A's window against
    // the reverse complement of B's (which moves the same way as A's, at a
    // fixed offset), and, where that holds, A's window against its own
    // reverse complement.
    const int64_t U = u0 + lane * 32;
    const int64_t a0 = ext_start(st0, len, U, L, c.n[0]), a31 = ext_start(st0, len, U + 31, L, c.n[0]);
    const int64_t b0 = ext_start(st1, len, U, L, c.n[1]), b31 = ext_start(st1, len, U + 31, L, c.n[1]);
    const bool adown = st0 > 0;  // A's window starts decrease with u, B's increase (and vice versa)
    const int64_t amin = adown ? a31 : a0, bmin = adown ? b0 : b31;
    if (a0 >= 0 && a31 >= 0 && b0 >= 0 && b31 >= 0 && amin + 80 <= c.n[0] && bmin + 80 <= c.n[1]) {
      uint64_t ah, al, bh, bl;
      window128(c.g[0], (uint64_t)amin, ah, al);
      window128(c.g[1], (uint64_t)bmin, bh, bl);
      // reverse complements of the two 64-base stretches: base k is the
      // complement of base 63 - k
      const uint64_t rah = revcomp64(al), ral = revcomp64(ah);
      const uint64_t rbh = revcomp64(bl), rbl = revcomp64(bh);
#pragma unroll 4
      for (int t = 0; t < 32; ++t) {
        const int ja = adown ? 31 - t : t;  // A's window start amin + ja
        const int jb = adown ? t : 31 - t;  // B's window start bmin + jb
        // rc of the window at stretch offset j is the reverse stretch's window at 64 - L - j
        const uint64_t aw = top64(ah, al, 2 * ja);
        bool b = ((aw ^ top64(rbh, rbl, 2 * (64 - L - jb))) & pmask) == 0;
        if (b) b = ((aw ^ top64(rah, ral, 2 * (64 - L - ja))) & pmask) != 0;
        word |= (uint32_t)b << t;
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
  ring[((u0 >> 5) + lane) & (RING - 1)] = word;
}

static __device__ void ext_fill(const MatchCtx& c, int64_t st0, int64_t st1, int64_t len, int64_t u0, uint64_t pmask,
                                uint32_t* ring) {
  ext_fill_ring<kExtRing>(c, st0, st1, len, u0, pmask, ring);
  __syncwarp();
}

// Where a side's walk stops.  On one side of the entry the walk starts at
// displacement 0 and, with bit(u) = "the window pair at displacement u
// matches" (0 beyond the genome ends), jumps by L while the window L further
// matches, then moves to the furthest matching window within L, and repeats.
// Every position it reaches is 0 or a matching window, every move is at most
// L, and it moves on from q exactly when one of bits q+1 .. q+L is set.  So
// it can never pass a run of L clear bits, and it stops at the first
// position q in {0} or the set bits whose next L bits are all clear.  Here
// that q is found word by word: for the 64 bits of words i, i+1, the clear
// runs of length L are the bits of y = AND of L shifts of ~x, and the
// candidates of word i whose next L bits are clear are its set bits (and
// the start) at positions r with bit r+1 of y set.
__device__ __forceinline__ uint32_t stop_in_word(uint32_t w, uint32_t w_next, bool first, int L) {
  uint64_t y = ~(((uint64_t)w_next << 32) | w);
  for (int have = 1; have < L;) {  // y bit j: clear bits j .. j+have-1
    const int sh = have < L - have ? have : L - have;
    y &= y >> sh;
    have += sh;
  }
  return (w | (first ? 1u : 0u)) & (uint32_t)(y >> 1);
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
    const int64_t room = r0 < r1 ? r0 : r1;
    uint32_t* ring = R.w[sd];
    int64_t filled = 0, checked = 0;  // displacements filled, words checked
    for (int k = 0;; ++k) {
      // most matches stop within a few windows: the first fill is 256 displacements
      const int nlanes = k == 0 ? 8 : 32;
      ext_fill_ring<kExtRing>(c, s0, s1, elen, filled, pmask, ring, nlanes);
      __syncwarp();
      filled += 32 * nlanes;
      const int64_t last = filled / 32 - 1;  // words below it have their successor filled
      const int64_t i = checked + lane;
      uint32_t hit = 0;
      if (i < last) hit = stop_in_word(ring[i & (kExtRing - 1)], ring[(i + 1) & (kExtRing - 1)], i == 0, L);
      const unsigned any = __ballot_sync(0xffffffffu, hit != 0);
      if (any) {
        const int f = __ffs(any) - 1;  // the lowest word with a stop holds the first one
        const uint32_t h = __shfl_sync(0xffffffffu, hit, f);
        moved[sd] = 32 * (checked + f) + (__ffs(h) - 1);
        break;
      }
      checked = last;
      if (filled > room + 2 * kExtChunk + 64) {  // never reached: the bits beyond the room are clear
        moved[sd] = room > 0 ? room : 0;
        break;
      }
    }
  }
  m.len = elen + moved[0] + moved[1];
  m.s0 = e0 > 0 ? e0 - moved[0] : e0 + moved[1];
  m.s1 = e1 > 0 ? e1 - moved[0] : e1 + moved[1];
}

// ExtendMatch by a whole CTA (every thread calls it with the same entry and
// gets the same result): per side the match bits are filled in chunks of
// 1024, 2048, 4096, then 8192 displacements (one warp per 1024), and after
// each chunk every thread checks one word of it for the walk's stopping
// point (stop_in_word); the first one wins.  The ring keeps the last 16,384
// displacements, so the previous chunk's last word is still there.
constexpr int kCtaRing = 512;  // words per side
struct CtaExtRing {
  uint32_t w[2][kCtaRing];
  uint32_t red[32];
};

static __device__ void cta_extend(const MatchCtx& c, Mhe& m, CtaExtRing& R) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;  // at most 8: a chunk fits half the ring
  const int L = c.s.L;
  const uint64_t pmask = pattern_mask64(c.s);
  const int64_t e0 = m.s0, e1 = m.s1, elen = m.len;
  int64_t moved[2] = {0, 0};
#pragma unroll 1
  for (int sd = 0; sd < 2; ++sd) {
    const int64_t sg = sd == 0 ? 1 : -1;
    const int64_t s0 = sg * e0, s1 = sg * e1;
    uint32_t* ring = R.w[sd];
    // room: the nearer genome end; every bit beyond it is clear, so the stop
    // is found once the fills pass it by L (the bound below is never reached)
    const int64_t r0 = s0 > 0 ? s0 - 1 : (s0 < 0 ? c.n[0] - elen + s0 + 1 : -1);
    const int64_t r1 = s1 > 0 ? s1 - 1 : (s1 < 0 ? c.n[1] - elen + s1 + 1 : -1);
    const int64_t room = r0 < r1 ? r0 : r1;
    int64_t filled = 0, checked = 0;  // displacements filled, words checked
    for (int k = 0;; ++k) {
      // 256 displacements first (most matches stop there), then 1, 2, 4 and 8 warps' worth
      const int nw = k == 0 ? 1 : (k < 4 ? min(nwarps, 1 << (k - 1)) : nwarps);
      const int nlanes = k == 0 ? 8 : 32;
      __syncthreads();  // every thread is past its reads of the words refilled now
      if (wid < nw)
        ext_fill_ring<kCtaRing>(c, s0, s1, elen, filled + (int64_t)wid * kExtChunk, pmask, ring, nlanes);
      __syncthreads();
      filled += (int64_t)nw * 32 * nlanes;
      const int64_t last = filled / 32 - 1;  // words below it have their successor filled
      uint32_t q = 0xffffffffu;
      const int64_t i = checked + threadIdx.x;
      if (i < last) {
        const uint32_t hit = stop_in_word(ring[i & (kCtaRing - 1)], ring[(i + 1) & (kCtaRing - 1)], i == 0, L);
        if (hit) q = (uint32_t)(32 * i) + (uint32_t)(__ffs(hit) - 1);
      }
      q = __reduce_min_sync(0xffffffffu, q);
      if (lane == 0) R.red[wid] = q;
      __syncthreads();
      q = 0xffffffffu;
      for (int w = 0; w < nwarps; ++w) q = min(q, R.red[w]);
      checked = last;
      if (q != 0xffffffffu || filled > room + 2 * kExtChunk * 8 + 64) {
        moved[sd] = q != 0xffffffffu ? q : (room > 0 ? room : 0);
        break;
      }
    }
    __syncthreads();  // the ring and the reduction words are reused
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
