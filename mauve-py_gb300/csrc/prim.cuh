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

// ------------------------------------------------- one-sweep radix sort
//
// Same stable LSD result as radix_sort_pairs, one kernel per 8-bit digit:
//   k_os_hist   all passes' digit histograms in one read of the keys
//   k_os_scan   exclusive scan of each pass's 256 counts
//   k_os_pass   per tile (claimed in order through an atomic counter): keys
//               and values held in registers, the tile's digit counts
//               published at once, the counts of all earlier tiles gathered
//               by decoupled look-back (each state word carries a flag and
//               a 30-bit count in one 32-bit store), the tile ranked stably
//               in shared memory and written out digit run by digit run.
// A tile only waits for tiles claimed before it, which are already running,
// so the look-back always finishes; each wait is still bounded and a give-up
// raises kDevWatchdog.  n must stay below 2^30.
namespace os {
constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
constexpr uint32_t kAgg = 1u << 30, kPre = 2u << 30, kVal = (1u << 30) - 1;
constexpr long long kSpin = 1ll << 22;
}  // namespace os

inline int64_t onesweep_scratch_words(int64_t n, int nbits) {
  const int64_t npass = (nbits + 7) / 8;
  const int64_t ntiles = (n + os::kTile - 1) / os::kTile;
  return npass * ntiles * 256 + npass * 256 + npass + 16;
}

template <typename K>
__global__ void __launch_bounds__(256) k_os_hist(const K* __restrict__ keys, int64_t n, int npass,
                                                 uint32_t* __restrict__ ghist) {
  __shared__ uint32_t h[8][256];
  for (int p = 0; p < 8; ++p) h[p][threadIdx.x] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const K k = keys[i];
    for (int p = 0; p < npass; ++p) atomicAdd(&h[p][(uint32_t)(k >> (8 * p)) & 255u], 1u);
  }
  __syncthreads();
  for (int p = 0; p < npass; ++p)
    if (h[p][threadIdx.x]) atomicAdd(&ghist[p * 256 + threadIdx.x], h[p][threadIdx.x]);
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void k_os_scan(uint32_t* __restrict__ ghist);

template <typename K>
__global__ void __launch_bounds__(os::kThreads, sizeof(K) == 4 ? 4 : 3) k_os_pass(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                         K* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
                                                         int shift, const uint32_t* __restrict__ gstart,
                                                         uint32_t* state, uint32_t* tile_ctr, uint32_t* err) {
  using namespace os;
  __shared__ K skey[kTile];
  __shared__ uint32_t sval[kTile];
  __shared__ uint32_t whist[8][256];  // per-warp digit counts, then per-warp offsets
  __shared__ uint32_t lstart[256];
  __shared__ uint32_t gbase[256];
  __shared__ uint32_t s_tile;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
#pragma unroll
  for (int w = 0; w < 8; ++w) whist[w][tid] = 0;
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t base = tile * kTile;
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
    const uint32_t before = d < 256u ? whist[wid][d] : 0u;
    rank[k] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (d < 256u && (peers & lt_mask) == 0) whist[wid][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: the tile count and each warp's offset inside the digit's run
  uint32_t mine = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    const uint32_t c = whist[w][tid];
    whist[w][tid] = mine;
    mine += c;
  }
  // publish this tile's counts, then look back over earlier tiles, kWin
  // tiles per step (independent loads issued together; a tile not yet
  // published is re-read, bounded)
  uint32_t* st = state + tile * 256 + tid;
  *(volatile uint32_t*)st = (tile == 0 ? kPre : kAgg) | mine;
  constexpr int kWin = 8;
  uint32_t excl = 0;
  int64_t t0 = tile - 1;
  if (t0 >= 0) {
    // usually the previous tile has its inclusive prefix out already
    const uint32_t x = *(const volatile uint32_t*)(state + t0 * 256 + tid);
    if (x & kPre) {
      excl = x & kVal;
      t0 = -1;
    }
  }
  for (int64_t t = t0; t >= 0; t -= kWin) {
    uint32_t v[kWin];
#pragma unroll
    for (int q = 0; q < kWin; ++q) v[q] = t - q >= 0 ? *(const volatile uint32_t*)(state + (t - q) * 256 + tid) : kPre;
    bool done = false;
#pragma unroll
    for (int q = 0; q < kWin; ++q) {
      if (done) break;
      if (t - q < 0) {
        done = true;
        break;
      }
      uint32_t x = v[q];
      const volatile uint32_t* p = state + (t - q) * 256 + tid;
      long long spins = 0;
      while ((x & ~kVal) == 0 && ++spins < kSpin) x = *p;
      if ((x & ~kVal) == 0) {
        set_error(err, kDevWatchdog);
        done = true;
        break;
      }
      excl += x & kVal;
      if (x & kPre) done = true;
    }
    if (done) break;
  }
  if (tile > 0) *(volatile uint32_t*)st = kPre | (excl + mine);
  gbase[tid] = gstart[tid] + excl;
  lstart[tid] = block_excl_scan256(mine, nullptr);
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const uint32_t d = dig[k];
    if (d < 256u) {
      const uint32_t lp = lstart[d] + whist[wid][d] + rank[k];
      skey[lp] = key[k];
      sval[lp] = val[k];
    }
  }
  __syncthreads();
  for (int i = tid; i < tile_n; i += kThreads) {
    const K k = skey[i];
    const uint32_t d = (uint32_t)(k >> shift) & 255u;
    const int64_t o = (int64_t)gbase[d] + (i - (int)lstart[d]);
    kout[o] = k;
    vout[o] = sval[i];
  }
}

// Stable LSD sort of (keys, vals) on bits [0, nbits); returns which buffer
// holds the result (0 = keys/vals, 1 = alt).  scratch:
// onesweep_scratch_words(n, nbits) words.  n < 2^30.
template <typename K>
int onesweep_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n, int nbits,
                        uint32_t* scratch, cudaStream_t st, uint64_t* launches, uint32_t* err) {
  if (n <= 0) return 0;
  const int npass = (nbits + 7) / 8;
  const int64_t ntiles = (n + os::kTile - 1) / os::kTile;
  uint32_t* state = scratch;
  uint32_t* ghist = state + (int64_t)npass * ntiles * 256;
  uint32_t* ctr = ghist + npass * 256;
  cudaMemsetAsync(scratch, 0, (size_t)onesweep_scratch_words(n, nbits) * 4, st);
  int hb = (int)((n + 255) / 256);
  if (hb > 152 * 8) hb = 152 * 8;
  k_os_hist<K><<<hb, 256, 0, st>>>(keys, n, npass, ghist);
  k_os_scan<<<npass, 256, 0, st>>>(ghist);
  K* ka = keys;
  K* kb = keys_alt;
  uint32_t* va = vals;
  uint32_t* vb = vals_alt;
  int which = 0;
  for (int p = 0; p < npass; ++p) {
    k_os_pass<K><<<(unsigned)ntiles, os::kThreads, 0, st>>>(ka, va, kb, vb, n, 8 * p, ghist + p * 256,
                                                            state + (int64_t)p * ntiles * 256, ctr + p, err);
    K* tk = ka;
    ka = kb;
    kb = tk;
    uint32_t* tv = va;
    va = vb;
    vb = tv;
    which ^= 1;
  }
  if (launches) *launches += 2 + npass;
  return which;
}

// ------------------------------------- reduce-then-scan radix sort
//
// The same stable LSD result again, three kernels per 8-bit digit and no
// waits between tiles: every tile's digit counts first (k_rts_count, one
// read of the keys), then one block per digit turns its row of tile counts
// into output offsets (k_rts_rowscan, starting at the digit's global start
// from k_os_hist), then each tile ranks its keys stably in shared memory
// and writes them out digit run by digit run (k_rts_scatter).  Compared with
// one sweep it reads the keys once more per pass but never serialises
// tiles on their predecessors' prefixes, which with thousands of tiles in
// flight is the one-sweep pass's critical path.
template <typename K>
__global__ void __launch_bounds__(os::kThreads) k_rts_count(const K* __restrict__ keys, int64_t n, int shift,
                                                            uint32_t* __restrict__ counts, int64_t ntiles) {
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
  counts[(int64_t)tid * ntiles + blockIdx.x] = s;
}

// Row d of the digit-major count table -> offsets, in place.
__global__ void k_rts_rowscan(uint32_t* __restrict__ counts, int64_t ntiles, const uint32_t* __restrict__ gstart);

template <typename K>
__global__ void __launch_bounds__(os::kThreads, sizeof(K) == 4 ? 4 : 3)
    k_rts_scatter(const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
                  uint32_t* __restrict__ vout, int64_t n, int shift, const uint32_t* __restrict__ offsets,
                  int64_t ntiles) {
  using namespace os;
  __shared__ K skey[kTile];
  __shared__ uint32_t sval[kTile];
  __shared__ uint32_t whist[8][256];  // per-warp digit counts, then per-warp offsets
  __shared__ uint32_t lstart[256];
  __shared__ uint32_t gbase[256];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int w = 0; w < 8; ++w) whist[w][tid] = 0;
  gbase[tid] = offsets[(int64_t)tid * ntiles + blockIdx.x];
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
    const uint32_t before = d < 256u ? whist[wid][d] : 0u;
    rank[k] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (d < 256u && (peers & lt_mask) == 0) whist[wid][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  uint32_t mine = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    const uint32_t c = whist[w][tid];
    whist[w][tid] = mine;
    mine += c;
  }
  lstart[tid] = block_excl_scan256(mine, nullptr);
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const uint32_t d = dig[k];
    if (d < 256u) {
      const uint32_t lp = lstart[d] + whist[wid][d] + rank[k];
      skey[lp] = key[k];
      sval[lp] = val[k];
    }
  }
  __syncthreads();
  for (int i = tid; i < tile_n; i += kThreads) {
    const K k = skey[i];
    const uint32_t d = (uint32_t)(k >> shift) & 255u;
    const int64_t o = (int64_t)gbase[d] + (i - (int)lstart[d]);
    kout[o] = k;
    vout[o] = sval[i];
  }
}

inline int64_t rts_scratch_words(int64_t n, int nbits) {
  const int64_t npass = (nbits + 7) / 8;
  const int64_t ntiles = (n + os::kTile - 1) / os::kTile;
  return ntiles * 256 + npass * 256 + 16;
}

// Scratch layout: the digit-major tile count table (ntiles * 256 words),
// then each pass's 256 global digit counts.
inline uint32_t* rts_counts(uint32_t* scratch) { return scratch; }
inline uint32_t* rts_ghist(uint32_t* scratch, int64_t n) {
  return scratch + ((n + os::kTile - 1) / os::kTile) * 256;
}

// counted: the producer of the keys already wrote every pass's global digit
// counts (rts_ghist, zeroed before) and the first pass's tile counts
// (rts_counts) while writing the keys in tiles of os::kTile.
template <typename K>
int rts_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n, int nbits,
                   uint32_t* scratch, cudaStream_t st, uint64_t* launches, bool counted = false) {
  if (n <= 0) return 0;
  const int npass = (nbits + 7) / 8;
  const int64_t ntiles = (n + os::kTile - 1) / os::kTile;
  uint32_t* counts = rts_counts(scratch);
  uint32_t* ghist = rts_ghist(scratch, n);
  if (!counted) {
    cudaMemsetAsync(ghist, 0, (size_t)npass * 256 * 4, st);
    int hb = (int)((n + 255) / 256);
    if (hb > 152 * 8) hb = 152 * 8;
    k_os_hist<K><<<hb, 256, 0, st>>>(keys, n, npass, ghist);
    if (launches) *launches += 1;
  }
  k_os_scan<<<npass, 256, 0, st>>>(ghist);
  K* ka = keys;
  K* kb = keys_alt;
  uint32_t* va = vals;
  uint32_t* vb = vals_alt;
  int which = 0;
  for (int p = 0; p < npass; ++p) {
    if (p > 0 || !counted) {
      k_rts_count<K><<<(unsigned)ntiles, os::kThreads, 0, st>>>(ka, n, 8 * p, counts, ntiles);
      if (launches) *launches += 1;
    }
    k_rts_rowscan<<<256, 256, 0, st>>>(counts, ntiles, ghist + p * 256);
    k_rts_scatter<K><<<(unsigned)ntiles, os::kThreads, 0, st>>>(ka, va, kb, vb, n, 8 * p, counts, ntiles);
    K* tk = ka;
    ka = kb;
    kb = tk;
    uint32_t* tv = va;
    va = vb;
    vb = tv;
    which ^= 1;
  }
  if (launches) *launches += 1 + 2 * npass;
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
