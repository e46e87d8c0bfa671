// Device primitives shared by the seed and match kernels: an exclusive scan
// over uint32 and a stable LSD radix sort of (key, uint32 value) pairs.
//
// Radix sort, one 8-bit digit per pass:
//   k_digit_hist   per-tile digit counts           (reads keys once)
//   scan           exclusive scan of the digit-major count table
//   k_digit_scatter stages the tile in shared memory in stable digit order,
//                   then writes each digit's run contiguously (coalesced).
// Stability inside a tile comes from ranking 256-element chunks in order with
// __match_any_sync peer masks and per-warp counts, so equal digits keep their
// input order and the whole sort is stable.
#pragma once
#include "mvg_common.cuh"

namespace mvg {

constexpr int kScanTile = 4096;  // elements per scan block (256 threads x 16)
constexpr int kSortThreads = 256;
constexpr int kSortTile = 2048;  // elements per sort block (8 chunks of 256)

// ------------------------------------------------------------------ scan

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread (blockDim.x == 256).
// Returns the exclusive prefix; *total gets the block sum.
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t* total) {
  __shared__ uint32_t wsum[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t x = lane < 8 ? wsum[lane] : 0;
    uint32_t y = warp_incl_scan(x);
    if (lane < 8) wsum[lane] = y - x;
    if (lane == 7 && total) *total = y;
  }
  __syncthreads();
  uint32_t r = wsum[wid] + inc - v;
  __syncthreads();
  return r;
}

// Pass 1: per-block sums of tiles of kScanTile elements.
__global__ void k_scan_reduce(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ bsum);
// Pass 2: exclusive scan of the block sums (one block, loops over chunks).
__global__ void k_scan_bsums(uint32_t* __restrict__ bsum, int64_t nb, uint32_t* __restrict__ total);
// Pass 3: exclusive scan of each tile plus its block prefix.
__global__ void k_scan_down(const uint32_t* in, int64_t n, const uint32_t* __restrict__ bsum, uint32_t* out);

// Host side: exclusive scan of n uint32 into out (may alias in); *d_total
// (device) gets the sum.  scratch needs scan_scratch_words(n) words.
inline int64_t scan_scratch_words(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }
void exclusive_scan(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* scratch, uint32_t* d_total,
                    cudaStream_t st, uint64_t* launches);

// ------------------------------------------------------------ radix sort

template <typename K>
__global__ void k_digit_hist(const K* __restrict__ keys, int64_t n, int shift, uint32_t* __restrict__ counts,
                             int nblocks) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  const int64_t end = min(base + kSortTile, n);
  for (int64_t i = base + threadIdx.x; i < end; i += kSortThreads) {
    uint32_t d = (uint32_t)(keys[i] >> shift) & 255u;
    atomicAdd(&h[d], 1u);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads) k_digit_scatter(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                                K* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
                                                                int shift, const uint32_t* __restrict__ counts,
                                                                const uint32_t* __restrict__ offsets, int nblocks) {
  __shared__ K skey[kSortTile];
  __shared__ uint32_t sval[kSortTile];
  __shared__ uint32_t wcnt[8][256];
  __shared__ uint32_t run[256];
  __shared__ uint32_t lstart[256];
  __shared__ uint32_t gbase[256];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  const int tile_n = (int)min((int64_t)kSortTile, n - base);

  uint32_t mycount = counts[(int64_t)tid * nblocks + blockIdx.x];
  gbase[tid] = offsets[(int64_t)tid * nblocks + blockIdx.x];
  uint32_t ls = block_excl_scan256(mycount, nullptr);
  lstart[tid] = ls;
  run[tid] = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) wcnt[w][tid] = 0;
  __syncthreads();

  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int c = 0; c < kSortTile; c += kSortThreads) {
    const int li = c + tid;
    const bool valid = li < tile_n;
    K key = 0;
    uint32_t val = 0, d = 256u + (uint32_t)lane;  // invalid lanes get private digits
    if (valid) {
      key = kin[base + li];
      val = vin[base + li];
      d = (uint32_t)(key >> shift) & 255u;
    }
    uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t lrank = __popc(peers & lt_mask);
    if (valid && lrank == 0) wcnt[wid][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t r = run[d] + lrank;
      for (int w = 0; w < wid; ++w) r += wcnt[w][d];
      const uint32_t lp = lstart[d] + r;
      skey[lp] = key;
      sval[lp] = val;
    }
    __syncthreads();
    {
      uint32_t s = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) {
        s += wcnt[w][tid];
        wcnt[w][tid] = 0;
      }
      run[tid] += s;
    }
    __syncthreads();
    if (c + kSortThreads >= tile_n) break;
  }
  for (int i = tid; i < tile_n; i += kSortThreads) {
    K key = skey[i];
    uint32_t d = (uint32_t)(key >> shift) & 255u;
    int64_t o = (int64_t)gbase[d] + (i - (int)lstart[d]);
    kout[o] = key;
    vout[o] = sval[i];
  }
}

// Stable LSD radix sort of (keys, vals) on bits [0, nbits).  Ping-pongs
// between the input arrays and the alternates; returns which buffer holds
// the result (0 = keys/vals, 1 = alt).  scratch: radix_scratch_words(n).
inline int64_t radix_scratch_words(int64_t n) {
  int64_t nb = (n + kSortTile - 1) / kSortTile;
  return 2 * 256 * nb + scan_scratch_words(256 * nb) + 2;
}

template <typename K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n, int nbits,
                     uint32_t* scratch, cudaStream_t st, uint64_t* launches) {
  if (n <= 0) return 0;
  const int nb = (int)((n + kSortTile - 1) / kSortTile);
  uint32_t* counts = scratch;
  uint32_t* offsets = scratch + (int64_t)256 * nb;
  uint32_t* sscr = offsets + (int64_t)256 * nb;
  uint32_t* total = sscr + scan_scratch_words((int64_t)256 * nb);
  K* ka = keys;
  K* kb = keys_alt;
  uint32_t* va = vals;
  uint32_t* vb = vals_alt;
  int which = 0;
  for (int shift = 0; shift < nbits; shift += 8) {
    k_digit_hist<K><<<nb, kSortThreads, 0, st>>>(ka, n, shift, counts, nb);
    exclusive_scan(counts, offsets, (int64_t)256 * nb, sscr, total, st, launches);
    k_digit_scatter<K><<<nb, kSortThreads, 0, st>>>(ka, va, kb, vb, n, shift, counts, offsets, nb);
    if (launches) *launches += 2;
    K* tk = ka;
    ka = kb;
    kb = tk;
    uint32_t* tv = va;
    va = vb;
    vb = tv;
    which ^= 1;
  }
  return which;
}

// ------------------------------------- reduce-then-scan radix sort
//
// Stable LSD sort by 8-bit digits, three kernels per pass and no waits
// between tiles:
//   k_rts_count    per tile of kTile keys: its 256 digit counts, stored
//                  tile-major (one coalesced 1 KB row per tile), and added
//                  into the counts of the tile's chunk (ctiles tiles)
//   k_rts_offsets  one block per chunk: every digit's global start (from
//                  all chunks' sums) plus the chunks before this one, then
//                  the chunk's tiles' rows turned into output offsets in
//                  place
//   k_rts_scatter  per tile: keys ranked stably in shared memory and
//                  written out digit run by digit run
// Rows are read and written whole, so every count access is coalesced; the
// chunk sums make the offsets kernel a two-level scan with no serial walk
// over thousands of tiles.
namespace os {
constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
}  // namespace os

struct RtsGeom {
  int64_t ntiles, ctiles, nchunks;
  int npass;
};

// Chunks of at least 64 tiles and at most about 128 chunks.
inline RtsGeom rts_geom(int64_t n, int nbits) {
  RtsGeom g;
  g.npass = (nbits + 7) / 8;
  g.ntiles = (n + os::kTile - 1) / os::kTile;
  int64_t ct = (g.ntiles + 127) / 128;
  ct = (ct + 3) & ~3ll;
  g.ctiles = ct < 64 ? 64 : ct;
  g.nchunks = (g.ntiles + g.ctiles - 1) / g.ctiles;
  return g;
}

// Scratch layout: the tile count rows (ntiles x 256 words, reused by every
// pass), then each pass's chunk sums (nchunks x 256 words per pass, zeroed
// before the sort).  nchunks <= min(ntiles, 128), so sizing by that bound
// makes a scratch sized for n and nbits fit every smaller sort.
inline int64_t rts_scratch_words(int64_t n, int nbits) {
  const RtsGeom g = rts_geom(n, nbits);
  const int64_t cap = g.ntiles < 128 ? g.ntiles : 128;
  return g.ntiles * 256 + (int64_t)g.npass * cap * 256 + 16;
}
inline uint32_t* rts_counts(uint32_t* scratch) { return scratch; }
inline uint32_t* rts_csum(uint32_t* scratch, const RtsGeom& g) { return scratch + g.ntiles * 256; }

template <typename K>
__global__ void __launch_bounds__(os::kThreads) k_rts_count(const K* __restrict__ keys, int64_t n, int shift,
                                                            uint32_t* __restrict__ counts, uint32_t* __restrict__ csum,
                                                            int64_t ctiles) {
  __shared__ uint32_t h[8][256];
  const int tid = threadIdx.x, wid = tid >> 5;
#pragma unroll
  for (int w = 0; w < 8; ++w) h[w][tid] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * os::kTile;
  uint32_t d[os::kItems];
#pragma unroll
  for (int k = 0; k < os::kItems; ++k) {
    const int64_t i = base + k * os::kThreads + tid;
    d[k] = i < n ? ((uint32_t)(keys[i] >> shift) & 255u) : 256u;
  }
#pragma unroll
  for (int k = 0; k < os::kItems; ++k)
    if (d[k] < 256u) atomicAdd(&h[wid][d[k]], 1u);
  __syncthreads();
  uint32_t s = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) s += h[w][tid];
  counts[(int64_t)blockIdx.x * 256 + tid] = s;
  if (s) atomicAdd(&csum[((int64_t)blockIdx.x / ctiles) * 256 + tid], s);
}

// Block c, 1024 threads: thread (q, d) handles digit d for a quarter q of
// the chunk sums and a quarter of chunk c's tiles.
__global__ void k_rts_offsets(uint32_t* __restrict__ counts, int64_t ntiles, const uint32_t* __restrict__ csum,
                              int64_t ctiles, int64_t nchunks);

template <typename K>
__global__ void __launch_bounds__(os::kThreads, sizeof(K) == 4 ? 4 : 3)
    k_rts_scatter(const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
                  uint32_t* __restrict__ vout, int64_t n, int shift, const uint32_t* __restrict__ offsets) {
  using namespace os;
  constexpr bool kPacked = sizeof(K) == 4;  // (key, value) as one 8-byte word in shared memory
  __shared__ __align__(16) uint32_t sbuf[kPacked ? 2 * kTile : kTile * (sizeof(K) / 4 + 1)];
  __shared__ uint32_t wofs[8][256];  // per-warp digit counts, then each warp's first slot per digit
  __shared__ uint32_t gofs[256];     // output index of the tile's slot 0 for each digit
  uint2* skv = reinterpret_cast<uint2*>(sbuf);
  K* skey = reinterpret_cast<K*>(sbuf);
  uint32_t* sval = sbuf + kTile * (sizeof(K) / 4);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int w = 0; w < 8; ++w) wofs[w][tid] = 0;
  const uint32_t gbase = offsets[(int64_t)blockIdx.x * 256 + tid];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTile;
  const int tile_n = (int)min((int64_t)kTile, n - base);
  // warp w owns tile items [256 w, 256 w + 256): item 256 w + 32 k + lane
  K key[kItems];
  uint32_t val[kItems], dig[kItems], rank[kItems];
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const int li = wid * 256 + 32 * k + lane;
    if (li < tile_n) {
      key[k] = kin[base + li];
      val[k] = vin[base + li];
      dig[k] = (uint32_t)(key[k] >> shift) & 255u;
    } else {
      key[k] = 0;
      val[k] = 0;
      dig[k] = 256u + (uint32_t)lane;  // private digit: never shares a rank
    }
  }
  // stable rank inside the warp: earlier rounds, then lower lanes
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const uint32_t d = dig[k];
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t before = d < 256u ? wofs[wid][d] : 0u;
    rank[k] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (d < 256u && (peers & lt_mask) == 0) wofs[wid][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  uint32_t wpre[8], mine = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    wpre[w] = mine;
    mine += wofs[w][tid];
  }
  const uint32_t lstart = block_excl_scan256(mine, nullptr);
#pragma unroll
  for (int w = 0; w < 8; ++w) wofs[w][tid] = lstart + wpre[w];
  gofs[tid] = gbase - lstart;  // gbase >= lstart: earlier digits of this tile precede it
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const uint32_t d = dig[k];
    if (d < 256u) {
      const uint32_t lp = wofs[wid][d] + rank[k];
      if constexpr (kPacked) {
        skv[lp] = make_uint2((uint32_t)key[k], val[k]);
      } else {
        skey[lp] = key[k];
        sval[lp] = val[k];
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < tile_n; i += kThreads) {
    K k;
    uint32_t v;
    if constexpr (kPacked) {
      const uint2 kv = skv[i];
      k = (K)kv.x;
      v = kv.y;
    } else {
      k = skey[i];
      v = sval[i];
    }
    const uint32_t d = (uint32_t)(k >> shift) & 255u;
    const int64_t o = (int64_t)gofs[d] + i;
    kout[o] = k;
    vout[o] = v;
  }
}

// counted: the producer of the keys already wrote the first pass's tile
// count rows and chunk sums (rts_counts, rts_csum) for tiles of os::kTile,
// and zeroed the other passes' chunk sums.
template <typename K>
int rts_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n, int nbits,
                   uint32_t* scratch, cudaStream_t st, uint64_t* launches, bool counted = false) {
  if (n <= 0) return 0;
  const RtsGeom g = rts_geom(n, nbits);
  uint32_t* counts = rts_counts(scratch);
  uint32_t* csum = rts_csum(scratch, g);
  if (!counted) cudaMemsetAsync(csum, 0, (size_t)g.npass * g.nchunks * 256 * 4, st);
  K* ka = keys;
  K* kb = keys_alt;
  uint32_t* va = vals;
  uint32_t* vb = vals_alt;
  int which = 0;
  for (int p = 0; p < g.npass; ++p) {
    uint32_t* cs = csum + (int64_t)p * g.nchunks * 256;
    if (p > 0 || !counted) {
      k_rts_count<K><<<(unsigned)g.ntiles, os::kThreads, 0, st>>>(ka, n, 8 * p, counts, cs, g.ctiles);
      if (launches) *launches += 1;
    }
    k_rts_offsets<<<(unsigned)g.nchunks, 1024, 0, st>>>(counts, g.ntiles, cs, g.ctiles, g.nchunks);
    k_rts_scatter<K><<<(unsigned)g.ntiles, os::kThreads, 0, st>>>(ka, va, kb, vb, n, 8 * p, counts);
    K* tk = ka;
    ka = kb;
    kb = tk;
    uint32_t* tv = va;
    va = vb;
    vb = tv;
    which ^= 1;
  }
  if (launches) *launches += 2 * g.npass;
  return which;
}

// The sort the workspace paths use: reduce-then-scan passes below 2^31
// elements, the older three-kernel passes above.  scratch:
// sort_scratch_words(n, nbits) words.
inline int64_t sort_scratch_words(int64_t n, int nbits) {
  const int64_t a = radix_scratch_words(n), b = rts_scratch_words(n, nbits);
  return a > b ? a : b;
}

template <typename K>
int sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n, int nbits, uint32_t* scratch,
               cudaStream_t st, uint64_t* launches, uint32_t* err) {
  (void)err;
  if (n < (1ll << 31)) return rts_sort_pairs<K>(keys, vals, keys_alt, vals_alt, n, nbits, scratch, st, launches);
  return radix_sort_pairs<K>(keys, vals, keys_alt, vals_alt, n, nbits, scratch, st, launches);
}

}  // namespace mvg
