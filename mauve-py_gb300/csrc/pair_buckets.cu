// The pairwise matcher's seed join by buckets: the seeds unique in each of
// the two genomes, in mer order, without sorting the whole key array.
//
// The SearchRange merge of the two sorted mer lists (LM/MatchFinder.cpp:
// 172-340, driven by LM/PairwiseMatchFinder.cpp:37-71) hashes every mer that
// occurs exactly once in each genome, in increasing mer order.  Only that
// order and the run structure (how often a mer occurs in each genome) matter,
// so the keys need not be sorted as one array:
//
//   k_pb_keys     keys of both genomes (mer << 2 | strand << 1 | genome,
//                 2w + 2 <= 32 bits) and positions, plus every tile's bucket
//                 counts (bucket = the mer's top BB bits), one row per tile
//   k_pb_csum     per-chunk sums of the count rows
//   k_pb_scan     every bucket's start and size; chunk starts
//   k_pb_offsets  count rows -> each tile's first slot in each bucket
//   k_pb_scatter  (key, position) pairs into their buckets; the order
//                 inside a bucket is arbitrary (shared-memory atomics)
//   k_pb_local    one block per bucket: a stable LSD sort by the rest of the
//                 mer and the genome bit (in shared memory, or through global
//                 memory in chunks when the bucket is larger), then the runs:
//                 a mer with one position in each genome is a pair, staged
//                 as (position in A, position in B | reverse << 31) at the
//                 bucket's start, and counted
//
// Buckets are in mer order and each is sorted by mer, so the staged pairs
// taken bucket by bucket are in the order the merge hashes them.  Positions
// are below 2^25 on this path (the host takes the full sort beyond that), so
// bit 31 of the B position is free for the strand relation.
#include <algorithm>

#include "mvg_internal.h"
#include "prim.cuh"

namespace mvg {

namespace pb {
constexpr int kKeyThreads = 1024;
constexpr int kLocThreads = 256;
constexpr int kLocWarps = kLocThreads / 32;
constexpr int kCap = 3072;      // bucket elements sorted in shared memory
constexpr int kLocItems = kCap / kLocThreads;
constexpr int kMaxDigit = 64;   // chunked in-bucket passes: digits of at most 6 bits
constexpr int kSmemDigit = 512; // shared-memory in-bucket passes: digits of at most 9 bits
constexpr int kGroups = 512;    // groups of a bucket split by its top 9 in-bucket bits
constexpr int kGroupMax = 256;  // larger groups: radix passes for the bucket instead
constexpr int kChunkTiles = 32;
}  // namespace pb

PairBucketGeom pair_bucket_geom(uint64_t n, int w) {
  PairBucketGeom g;
  int bb = 4;
  while (bb < 14 && ((uint64_t)2048 << bb) < n) ++bb;  // about 2048 keys per bucket at most
  if (bb > 2 * w) bb = 2 * w;
  g.bbits = bb;
  g.nbuckets = 1 << bb;
  g.tile = std::max<int64_t>(16384, 4ll * g.nbuckets);
  g.ntiles = (int64_t)((n + g.tile - 1) / g.tile);
  g.nchunks = (g.ntiles + pb::kChunkTiles - 1) / pb::kChunkTiles;
  // in-bucket key: the mer bits below the bucket, then the genome bit; an
  // odd number of passes leaves a chunked sort's result in the scratch copy
  const int lbits = 2 * w - bb + 1;
  int np = (lbits + 5) / 6;
  if ((np & 1) == 0) ++np;
  g.npass = np;
  g.dbits = (lbits + np - 1) / np;
  g.lbits = lbits;
  g.spass = (lbits + 8) / 9;
  g.sbits = (lbits + g.spass - 1) / g.spass;
  return g;
}

// ------------------------------------------------------------------ keys

__global__ void __launch_bounds__(pb::kKeyThreads) k_pb_keys(const uint32_t* __restrict__ ga, uint64_t ca,
                                                             const uint32_t* __restrict__ gb, uint64_t cb, SeedDesc s,
                                                             uint32_t* __restrict__ keys, uint32_t* __restrict__ pos,
                                                             uint32_t* __restrict__ counts, int bbits, int64_t tile) {
  extern __shared__ uint32_t h[];  // nbuckets counts
  __shared__ uint32_t lut[8][256];
  const int tid = threadIdx.x;
  const int nbk = 1 << bbits;
  seed_lut_build32(s, lut);
  for (int d = tid; d < nbk; d += pb::kKeyThreads) h[d] = 0;
  __syncthreads();
  const int nb = seed_bytes(s);
  const bool quad = nb <= 7;  // four positions from one 32-base window
  const int sh = 32 - 2 * s.w, bsh = 2 * s.w + 2 - bbits;  // keys have 2w + 2 bits
  const uint64_t n = ca + cb;
  const uint64_t base = (uint64_t)blockIdx.x * (uint64_t)tile;
  for (int64_t o = 4 * tid; o < tile; o += 4 * pb::kKeyThreads) {
    const uint64_t p0 = base + (uint64_t)o;
    if (p0 >= n) break;
    if (quad && p0 + 4 <= n && (p0 + 4 <= ca || p0 >= ca)) {
      const bool in_b = p0 >= ca;
      const uint64_t q0 = in_b ? p0 - ca : p0;
      const uint64_t win = window64(in_b ? gb : ga, q0);
      uint32_t kk[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t f = gather_mer32(win, u, lut, nb);
        const uint32_t r = revcomp_mer32(f, s.w);
        const uint32_t m = f < r ? f : r;
        kk[u] = ((((m >> sh) << 1) | (m & 1u)) << 1) | (in_b ? 1u : 0u);
        atomicAdd(&h[kk[u] >> bsh], 1u);
      }
      *reinterpret_cast<uint4*>(keys + p0) = make_uint4(kk[0], kk[1], kk[2], kk[3]);
      *reinterpret_cast<uint4*>(pos + p0) =
          make_uint4((uint32_t)q0, (uint32_t)q0 + 1, (uint32_t)q0 + 2, (uint32_t)q0 + 3);
    } else {
      for (int u = 0; u < 4; ++u) {
        const uint64_t p = p0 + u;
        if (p >= n) break;
        const bool in_b = p >= ca;
        const uint64_t q = in_b ? p - ca : p;
        const uint32_t f = gather_mer32(window64(in_b ? gb : ga, q), 0, lut, nb);
        const uint32_t r = revcomp_mer32(f, s.w);
        const uint32_t m = f < r ? f : r;
        const uint32_t key = ((((m >> sh) << 1) | (m & 1u)) << 1) | (in_b ? 1u : 0u);
        keys[p] = key;
        pos[p] = (uint32_t)q;
        atomicAdd(&h[key >> bsh], 1u);
      }
    }
  }
  __syncthreads();
  uint32_t* row = counts + (int64_t)blockIdx.x * nbk;
  for (int d = tid; d < nbk; d += pb::kKeyThreads) row[d] = h[d];
}

// ------------------------------------------------------- bucket offsets

// Block (x, c): buckets 256x .. 256x+255 summed over chunk c's tiles.
__global__ void __launch_bounds__(256) k_pb_csum(const uint32_t* __restrict__ counts, int64_t ntiles, int nbk,
                                                 uint32_t* __restrict__ csum) {
  const int d = blockIdx.x * 256 + threadIdx.x;
  if (d >= nbk) return;
  const int64_t c = blockIdx.y;
  const int64_t t0 = c * pb::kChunkTiles, t1 = min(ntiles, t0 + pb::kChunkTiles);
  uint32_t s = 0;
#pragma unroll 8
  for (int64_t t = t0; t < t1; ++t) s += counts[t * nbk + d];
  csum[c * nbk + d] = s;
}

// One block of 1024 threads, 16 consecutive buckets per thread (nbk <=
// 16384): every bucket's total over the chunks and its start (exclusive
// scan over buckets).
__global__ void __launch_bounds__(1024) k_pb_scan(const uint32_t* __restrict__ csum, int64_t nchunks, int nbk,
                                                  uint32_t* __restrict__ bstart, uint32_t* __restrict__ bsize) {
  constexpr int kPer = 16;
  __shared__ uint32_t wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int d0 = tid * kPer;
  uint32_t tot[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) tot[k] = 0;
  if (d0 < nbk) {
#pragma unroll 4
    for (int64_t c = 0; c < nchunks; ++c) {
      const uint4* q = reinterpret_cast<const uint4*>(csum + c * nbk + d0);
#pragma unroll
      for (int k = 0; k < kPer / 4; ++k) {
        const uint4 v = q[k];
        tot[4 * k] += v.x;
        tot[4 * k + 1] += v.y;
        tot[4 * k + 2] += v.z;
        tot[4 * k + 3] += v.w;
      }
    }
  }
  uint32_t mine = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) mine += tot[k];
  const uint32_t inc = warp_incl_scan(mine);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const uint32_t x = wsum[lane];
    const uint32_t y = warp_incl_scan(x);
    wsum[lane] = y - x;
  }
  __syncthreads();
  if (d0 >= nbk) return;
  uint32_t start = wsum[wid] + inc - mine;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    bstart[d0 + k] = start;
    bsize[d0 + k] = tot[k];
    start += tot[k];
  }
}

// Block (x, c): chunk c's tiles' first slots per bucket (offs): the
// bucket's start plus the earlier chunks' sums, then the chunk's count rows
// (all loads issued before any store).
__global__ void __launch_bounds__(256) k_pb_offsets(const uint32_t* __restrict__ counts, int64_t ntiles, int nbk,
                                                    const uint32_t* __restrict__ csum,
                                                    const uint32_t* __restrict__ bstart, uint32_t* __restrict__ offs) {
  const int d = blockIdx.x * 256 + threadIdx.x;
  if (d >= nbk) return;
  const int64_t c = blockIdx.y;
  const int64_t t0 = c * pb::kChunkTiles;
  const int nt = (int)min((int64_t)pb::kChunkTiles, ntiles - t0);
  uint32_t v[pb::kChunkTiles];
#pragma unroll
  for (int k = 0; k < pb::kChunkTiles; ++k) v[k] = k < nt ? counts[(t0 + k) * nbk + d] : 0u;
  uint32_t run = bstart[d];
  for (int64_t cc = 0; cc < c; ++cc) run += csum[cc * nbk + d];
#pragma unroll
  for (int k = 0; k < pb::kChunkTiles; ++k) {
    if (k < nt) offs[(t0 + k) * nbk + d] = run;
    run += v[k];
  }
}

// Exclusive scan of n <= 16384 counts by one block of 1024 threads (16
// consecutive counts each); *total gets the sum.
__global__ void __launch_bounds__(1024) k_pb_scan_small(const uint32_t* __restrict__ in, int n,
                                                        uint32_t* __restrict__ out, uint32_t* __restrict__ total) {
  constexpr int kPer = 16;
  __shared__ uint32_t wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int i0 = tid * kPer;
  uint32_t v[kPer], mine = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    v[k] = i0 + k < n ? in[i0 + k] : 0u;
    mine += v[k];
  }
  const uint32_t inc = warp_incl_scan(mine);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const uint32_t x = wsum[lane];
    const uint32_t y = warp_incl_scan(x);
    wsum[lane] = y - x;
    if (lane == 31 && total) *total = y;
  }
  __syncthreads();
  uint32_t r = wsum[wid] + inc - mine;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    if (i0 + k < n) out[i0 + k] = r;
    r += v[k];
  }
}

void pair_scan_small(const uint32_t* in, int n, uint32_t* out, uint32_t* total, cudaStream_t st) {
  k_pb_scan_small<<<1, 1024, 0, st>>>(in, n, out, total);
}

// ------------------------------------------------------------- scatter

__global__ void __launch_bounds__(pb::kKeyThreads) k_pb_scatter(const uint32_t* __restrict__ keys,
                                                                const uint32_t* __restrict__ pos, uint64_t n,
                                                                const uint32_t* __restrict__ offsets, int bbits,
                                                                int bsh, int64_t tile, uint2* __restrict__ out) {
  extern __shared__ uint32_t cur[];  // next free slot per bucket
  const int nbk = 1 << bbits;
  const uint32_t* row = offsets + (int64_t)blockIdx.x * nbk;
  for (int d = threadIdx.x; d < nbk; d += pb::kKeyThreads) cur[d] = row[d];
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * (uint64_t)tile;
  const uint64_t end = min(n, base + (uint64_t)tile);
  for (uint64_t i = base + threadIdx.x; i < end; i += pb::kKeyThreads) {
    const uint32_t k = keys[i];
    const uint32_t slot = atomicAdd(&cur[k >> bsh], 1u);
    out[slot] = make_uint2(k, pos[i]);
  }
}

// ---------------------------------------------------- in-bucket sort

struct LocalSmem {
  uint32_t whist[pb::kLocWarps][pb::kSmemDigit];  // per-warp digit counts, then each warp's first slot
  uint32_t run[pb::kMaxDigit];                    // chunked sort: slots used so far by each digit
  uint32_t dstart[pb::kMaxDigit];                 // chunked sort: each digit's first slot in the bucket
  uint32_t wpairs[pb::kLocWarps];
  uint32_t total;
};

// In-bucket key: the mer bits below the bucket bits, then the genome bit.
__device__ __forceinline__ uint32_t pb_lkey(uint32_t key, int lbits) {
  return (((key >> 2) << 1) | (key & 1u)) & ((1u << lbits) - 1u);
}

// Stable rank of up to kLocItems * 32 items per warp: warp w takes items
// [w * rounds * 32, (w + 1) * rounds * 32) of src[0, n) in order, counting
// its digits in S.whist[w].  Items past n get private digits.
__device__ __forceinline__ void pb_rank(const uint2* src, int n, int rounds, int shift, uint32_t mask, int lbits,
                                        LocalSmem& S, uint2 (&item)[pb::kLocItems],
                                        uint32_t (&rank)[pb::kLocItems]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int wbase = wid * rounds * 32;
#pragma unroll
  for (int k = 0; k < pb::kLocItems; ++k) {
    if (k < rounds) {
      const int li = wbase + k * 32 + lane;
      uint32_t d;
      if (li < n) {
        item[k] = src[li];
        d = (pb_lkey(item[k].x, lbits) >> shift) & mask;
      } else {
        item[k] = make_uint2(0u, 0u);
        d = 0x10000u + (uint32_t)lane;  // private digit: shares no rank
      }
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t before = d < 0x10000u ? S.whist[wid][d] : 0u;
      rank[k] = before + __popc(peers & lt_mask);
      __syncwarp();
      if (d < 0x10000u && (peers & lt_mask) == 0) S.whist[wid][d] = before + __popc(peers);
      __syncwarp();
    }
  }
}

// One stable LSD pass of a bucket held in shared memory (n <= kCap): rank,
// one scan over (digit, warp) counts, scatter.  Digits of up to 9 bits.
__device__ void pb_pass_smem(const uint2* src, uint2* dst, int n, int shift, uint32_t mask, int lbits,
                             LocalSmem& S) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ndig = (int)mask + 1;
  const int rounds = (n + pb::kLocThreads - 1) / pb::kLocThreads;
  for (int d = lane; d < ndig; d += 32) S.whist[wid][d] = 0;
  __syncwarp();
  uint2 item[pb::kLocItems];
  uint32_t rank[pb::kLocItems];
  pb_rank(src, n, rounds, shift, mask, lbits, S, item, rank);
  __syncthreads();
  // thread t: digits 2t and 2t + 1 (ndig is a power of two up to 512)
  const int d0 = 2 * tid;
  uint32_t c0 = 0, c1 = 0;
  if (d0 < ndig) {
#pragma unroll
    for (int w = 0; w < pb::kLocWarps; ++w) {
      c0 += S.whist[w][d0];
      c1 += S.whist[w][d0 + 1];
    }
  }
  uint32_t r = block_excl_scan256(c0 + c1, nullptr);
  if (d0 < ndig) {
#pragma unroll
    for (int w = 0; w < pb::kLocWarps; ++w) {
      const uint32_t x = S.whist[w][d0];
      S.whist[w][d0] = r;
      r += x;
    }
#pragma unroll
    for (int w = 0; w < pb::kLocWarps; ++w) {
      const uint32_t x = S.whist[w][d0 + 1];
      S.whist[w][d0 + 1] = r;
      r += x;
    }
  }
  __syncthreads();
  const int wbase = wid * rounds * 32;
#pragma unroll
  for (int k = 0; k < pb::kLocItems; ++k)
    if (k < rounds && wbase + k * 32 + lane < n)
      dst[S.whist[wid][(pb_lkey(item[k].x, lbits) >> shift) & mask] + rank[k]] = item[k];
  __syncthreads();
}

// One stable LSD pass over a bucket too large for shared memory: src and
// dst in global memory, chunks of kCap elements in order, digits of up to 6
// bits.
__device__ void pb_pass_chunked(const uint2* src, uint2* dst, int n, int shift, uint32_t mask, int lbits,
                                LocalSmem& S) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ndig = (int)mask + 1;
  if (tid < pb::kMaxDigit) {
    S.run[tid] = 0;
    S.dstart[tid] = 0;
  }
  __syncthreads();
  for (int i = tid; i < n; i += pb::kLocThreads) atomicAdd(&S.dstart[(pb_lkey(src[i].x, lbits) >> shift) & mask], 1u);
  __syncthreads();
  if (wid == 0) {  // exclusive scan of at most 64 counts by one warp
    const uint32_t a = lane < ndig ? S.dstart[lane] : 0u, b = lane + 32 < ndig ? S.dstart[lane + 32] : 0u;
    const uint32_t ia = warp_incl_scan(a), ib = warp_incl_scan(b);
    const uint32_t ta = __shfl_sync(0xffffffffu, ia, 31);
    if (lane < ndig) S.dstart[lane] = ia - a;
    if (lane + 32 < ndig) S.dstart[lane + 32] = ta + ib - b;
  }
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += pb::kCap) {
    const int cn = min(pb::kCap, n - c0);
    const int rounds = (cn + pb::kLocThreads - 1) / pb::kLocThreads;
    for (int d = lane; d < ndig; d += 32) S.whist[wid][d] = 0;
    __syncwarp();
    uint2 item[pb::kLocItems];
    uint32_t rank[pb::kLocItems];
    pb_rank(src + c0, cn, rounds, shift, mask, lbits, S, item, rank);
    __syncthreads();
    if (tid < ndig) {  // per digit: the warps' first slots in this chunk
      uint32_t r = S.dstart[tid] + S.run[tid];
#pragma unroll
      for (int w = 0; w < pb::kLocWarps; ++w) {
        const uint32_t x = S.whist[w][tid];
        S.whist[w][tid] = r;
        r += x;
      }
      S.run[tid] = r - S.dstart[tid];
    }
    __syncthreads();
    const int wbase = wid * rounds * 32;
#pragma unroll
    for (int k = 0; k < pb::kLocItems; ++k)
      if (k < rounds && wbase + k * 32 + lane < cn)
        dst[S.whist[wid][(pb_lkey(item[k].x, lbits) >> shift) & mask] + rank[k]] = item[k];
    __syncthreads();
  }
}

// Runs of the sorted bucket v[0, n): element i opens a pair when it and
// i + 1 hold the same mer from different genomes and neither i - 1 nor
// i + 2 holds that mer.  Pairs are written in order to stage[0, count),
// which must not overlap v; returns the count.
__device__ uint32_t pb_pairs(const uint2* v, int n, uint2* stage, LocalSmem& S) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = min(16, max(1, (n + pb::kLocThreads - 1) / pb::kLocThreads));
  uint32_t total = 0;
  for (int c0 = 0; c0 < n; c0 += pb::kLocThreads * per) {
    const int i0 = c0 + tid * per;  // thread t: elements i0 .. i0 + per - 1
    uint32_t flags = 0;
    for (int k = 0; k < per; ++k) {
      const int i = i0 + k;
      if (i + 1 >= n) break;
      const uint32_t k0 = v[i].x, k1 = v[i + 1].x, m = k0 >> 2;  // key >> 2: the mer
      if ((k1 >> 2) != m || ((k0 ^ k1) & 1u) == 0) continue;
      if (i > 0 && (v[i - 1].x >> 2) == m) continue;
      if (i + 2 < n && (v[i + 2].x >> 2) == m) continue;
      flags |= 1u << k;
    }
    const uint32_t cnt = __popc(flags);
    const uint32_t inc = warp_incl_scan(cnt);
    if (lane == 31) S.wpairs[wid] = inc;
    __syncthreads();
    if (tid == 0) {
      uint32_t r = 0;
      for (int w = 0; w < pb::kLocWarps; ++w) {
        const uint32_t x = S.wpairs[w];
        S.wpairs[w] = r;
        r += x;
      }
      S.total = r;
    }
    __syncthreads();
    uint32_t j = total + S.wpairs[wid] + inc - cnt;
    const uint32_t chunk_pairs = S.total;
    while (flags) {
      const int k = __ffs(flags) - 1;
      flags &= flags - 1;
      const uint2 x = v[i0 + k], y = v[i0 + k + 1];
      const bool a_first = (x.x & 1u) == 0;
      const uint2 ea = a_first ? x : y, eb = a_first ? y : x;
      // SetDirection (LM/MemHash.cpp:189-207): B is reversed relative to A
      // when the two occurrences have different strand bits
      const uint32_t rev = ((ea.x >> 1) ^ (eb.x >> 1)) & 1u;
      stage[j++] = make_uint2(ea.y, eb.y | (rev << 31));
    }
    total += chunk_pairs;
    __syncthreads();
  }
  return total;
}

// Block b finds the unique pairs of bucket b.  A bucket of at most cap
// (<= kCap) keys is loaded into shared memory as (in-bucket key | strand <<
// 31, position) and split by its top in-bucket bits (up to 9) into at most
// 512 groups of a few keys each (shared-memory atomics place a group's keys
// in any order).  Then one thread per key: a key whose mer occurs exactly
// twice in its group, once per genome, and which is the A occurrence, is a
// pair (marked, and counted for its group); after one scan over the groups
// each pair's slot is its group's first slot plus the number of the group's
// pairs with a smaller mer.  If a group holds more than kGroupMax keys the
// bucket is instead sorted by stable radix passes of up to 9 bits.  Larger
// buckets are sorted in chunks between their region of `buf` and the same
// region of `alt` in an odd number of passes of up to 6 bits, which leaves
// them in `alt`.  The staged pairs go to the bucket's region of `buf`, which
// the keys no longer occupy.
__global__ void __launch_bounds__(pb::kLocThreads) k_pb_local(uint2* __restrict__ buf, uint2* __restrict__ alt,
                                                              const uint32_t* __restrict__ bstart,
                                                              const uint32_t* __restrict__ bsize, int lbits, int npass,
                                                              int dbits, int spass, int sbits, int cap,
                                                              uint32_t* __restrict__ pcount) {
  extern __shared__ __align__(16) uint2 sbuf[];  // 2 * kCap elements
  __shared__ LocalSmem S;
  __shared__ uint32_t gcnt[pb::kGroups], gbeg[pb::kGroups], gcur[pb::kGroups], gpair[pb::kGroups];
  constexpr uint32_t kMark = 1u << 30, kKey = kMark - 1u;
  const int tid = threadIdx.x;
  const int b = blockIdx.x;
  const int n = (int)bsize[b];
  uint2* g = buf + bstart[b];
  uint2* h = alt + bstart[b];
  uint32_t np;
  if (n <= cap) {
    // group bits: mer bits only (never the genome bit), at most 9
    const int hbits = lbits - 1 < 9 ? lbits - 1 : 9, lo = lbits - hbits, ng = 1 << hbits;
    uint2* s0 = sbuf;
    uint2* s1 = sbuf + pb::kCap;
    for (int d = tid; d < pb::kGroups; d += pb::kLocThreads) {
      gcnt[d] = 0;
      gpair[d] = 0;
    }
    __syncthreads();
    for (int i = tid; i < n; i += pb::kLocThreads) {
      const uint2 it = g[i];
      const uint32_t lk = pb_lkey(it.x, lbits);
      s0[i] = make_uint2(lk | (((it.x >> 1) & 1u) << 31), it.y);
      atomicAdd(&gcnt[lk >> lo], 1u);
    }
    __syncthreads();
    // thread t: groups 2t and 2t + 1
    const int d0 = 2 * tid;
    const uint32_t c0 = d0 < ng ? gcnt[d0] : 0u, c1 = d0 + 1 < ng ? gcnt[d0 + 1] : 0u;
    const uint32_t st = block_excl_scan256(c0 + c1, nullptr);
    if (d0 < ng) gbeg[d0] = gcur[d0] = st;
    if (d0 + 1 < ng) gbeg[d0 + 1] = gcur[d0 + 1] = st + c0;
    __syncthreads();
    for (int i = tid; i < n; i += pb::kLocThreads) {
      const uint2 e = s0[i];
      s1[atomicAdd(&gcur[(e.x & kKey) >> lo], 1u)] = e;
    }
    const bool big = __syncthreads_or(c0 > (uint32_t)pb::kGroupMax || c1 > (uint32_t)pb::kGroupMax);
    if (!big) {
      // the A occurrence of each pair: its pair record into s0 (free now)
      for (int i = tid; i < n; i += pb::kLocThreads) {
        const uint32_t x = s1[i].x, lk = x & kKey, m = lk >> 1;
        const int d = (int)(lk >> lo), e0 = (int)gbeg[d], e1 = e0 + (int)gcnt[d];
        int cnt = 0, other = 0;
        for (int j = e0; j < e1; ++j)
          if (((s1[j].x & kKey) >> 1) == m) {
            ++cnt;
            if (j != i) other = j;
          }
        if (cnt == 2 && (lk & 1u) == 0) {
          const uint2 y = s1[other];
          if (y.x & 1u) {
            // SetDirection (LM/MemHash.cpp:189-207): B is reversed relative
            // to A when the two occurrences have different strand bits
            const uint32_t rev = (x ^ y.x) >> 31;
            s0[i] = make_uint2(s1[i].y, y.y | (rev << 31));
            atomicOr(&s1[i].x, kMark);
            atomicAdd(&gpair[d], 1u);
          }
        }
      }
      __syncthreads();
      const uint32_t q0 = d0 < ng ? gpair[d0] : 0u, q1 = d0 + 1 < ng ? gpair[d0 + 1] : 0u;
      const uint32_t pst = block_excl_scan256(q0 + q1, &S.total);
      if (d0 < ng) gcur[d0] = pst;
      if (d0 + 1 < ng) gcur[d0 + 1] = pst + q0;
      __syncthreads();
      for (int i = tid; i < n; i += pb::kLocThreads) {
        const uint32_t x = s1[i].x;
        if (!(x & kMark)) continue;
        const uint32_t m = (x & kKey) >> 1;
        const int d = (int)((x & kKey) >> lo), e0 = (int)gbeg[d], e1 = e0 + (int)gcnt[d];
        uint32_t r = 0;
        for (int j = e0; j < e1; ++j) {
          const uint32_t y = s1[j].x;
          r += (y & kMark) && ((y & kKey) >> 1) < m;
        }
        g[gcur[d] + r] = s0[i];
      }
      np = S.total;
    } else {
      for (int i = tid; i < n; i += pb::kLocThreads) s0[i] = g[i];
      __syncthreads();
      const uint32_t mask = (1u << sbits) - 1u;
      for (int p = 0; p < spass; ++p) {
        pb_pass_smem(s0, s1, n, p * sbits, mask, lbits, S);
        uint2* t = s0;
        s0 = s1;
        s1 = t;
      }
      np = pb_pairs(s0, n, g, S);
    }
  } else {
    const uint32_t mask = (1u << dbits) - 1u;
    const uint2* src = g;
    uint2* dst = h;
    for (int p = 0; p < npass; ++p) {
      pb_pass_chunked(src, dst, n, p * dbits, mask, lbits, S);
      uint2* t = (uint2*)src;
      src = dst;
      dst = t;
    }
    np = pb_pairs(src, n, g, S);  // npass is odd: the sorted bucket is in alt
  }
  if (tid == 0) pcount[b] = np;
}

// ------------------------------------------------------------------ host

int pair_buckets(Ctx* c, const uint32_t* ga, uint64_t ca, const uint32_t* gb, uint64_t cb, const SeedDesc& s,
                 PairStage* out) {
  const uint64_t n = ca + cb;
  const PairBucketGeom g = pair_bucket_geom(n, s.w);
  const int nbk = g.nbuckets;
  Workspace& ws = c->ws;
  const uint64_t n4 = (n + 3) & ~3ull;  // positions start on a 16-byte boundary (vector stores)
  uint32_t* kp = (uint32_t*)ws.get(c, 30, (size_t)n4 * 8 + 64);
  uint2* bufp = (uint2*)ws.get(c, 31, (size_t)n * 8 + 64);
  // count rows, then the tiles' first slots (ntiles x nbk each)
  uint32_t* counts = (uint32_t*)ws.get(c, 32, (size_t)g.ntiles * nbk * 8 + 64);
  uint32_t* tabs = (uint32_t*)ws.get(c, 33, ((size_t)g.nchunks * nbk + 4 * (size_t)nbk) * 4 + 256);
  if (!kp || !bufp || !counts || !tabs) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  uint32_t* keys = kp;
  uint32_t* pos = kp + n4;
  uint32_t* offs = counts + (size_t)g.ntiles * nbk;
  uint32_t* csum = tabs;
  uint32_t* bstart = csum + (size_t)g.nchunks * nbk;
  uint32_t* bsize = bstart + nbk;
  uint32_t* pcount = bsize + nbk;
  uint32_t* pbase = pcount + nbk;
  static bool attr = false;  // once per process: more than 48 KB of dynamic shared memory
  if (!attr) {
    MVG_CUDA_TRY(cudaFuncSetAttribute(k_pb_keys, cudaFuncAttributeMaxDynamicSharedMemorySize, (16384 + 64) * 4));
    MVG_CUDA_TRY(cudaFuncSetAttribute(k_pb_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (16384 + 64) * 4));
    MVG_CUDA_TRY(cudaFuncSetAttribute(k_pb_local, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(2 * pb::kCap * sizeof(uint2))));
    attr = true;
  }
  const size_t hsm = (size_t)nbk * 4;
  k_pb_keys<<<(unsigned)g.ntiles, pb::kKeyThreads, hsm, c->stream>>>(ga, ca, gb, cb, s, keys, pos, counts, g.bbits,
                                                                     g.tile);
  const dim3 grid2((unsigned)((nbk + 255) / 256), (unsigned)g.nchunks);
  k_pb_csum<<<grid2, 256, 0, c->stream>>>(counts, g.ntiles, nbk, csum);
  k_pb_scan<<<1, 1024, 0, c->stream>>>(csum, g.nchunks, nbk, bstart, bsize);
  k_pb_offsets<<<grid2, 256, 0, c->stream>>>(counts, g.ntiles, nbk, csum, bstart, offs);
  stage_mark(c, "seed_scatter");
  k_pb_scatter<<<(unsigned)g.ntiles, pb::kKeyThreads, hsm, c->stream>>>(keys, pos, n, offs, g.bbits,
                                                                        2 * s.w + 2 - g.bbits, g.tile, bufp);
  stage_mark(c, "seed_local");
  const int cap = std::min(c->pair_bucket_cap, pb::kCap);
  k_pb_local<<<(unsigned)nbk, pb::kLocThreads, 2 * pb::kCap * sizeof(uint2), c->stream>>>(
      bufp, (uint2*)kp, bstart, bsize, g.lbits, g.npass, g.dbits, g.spass, g.sbits, cap, pcount);
  c->launches += 6;
  MVG_CUDA_TRY(cudaGetLastError());
  out->stage = bufp;
  out->bstart = bstart;
  out->pcount = pcount;
  out->pbase = pbase;
  out->nbuckets = nbk;
  return 0;
}

}  // namespace mvg

extern "C" int mvg_set_pair_bucket_cap(mvg_handle h, int cap) {
  using namespace mvg;
  if (!h || cap < 32 || cap > pb::kCap) return report_error(MVG_ERR_ARG, "cap must be in 32..3072");
  reinterpret_cast<Ctx*>(h)->pair_bucket_cap = cap;
  return 0;
}
