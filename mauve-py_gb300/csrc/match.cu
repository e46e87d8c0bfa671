// Pairwise seed matching and maximal-match extension (two genomes).
//
// The reference (PairwiseMatchFinder over MemHash) walks the two sorted mer
// lists in key order, hashes every seed that is unique in both genomes into
// one of 40,000 buckets by its generalised offset, skips a seed whose bucket
// already holds a match containing it, and otherwise extends the seed to a
// maximal spaced-seed match and inserts it in sorted position.  Only seeds
// in the same bucket ever interact, so on the GPU:
//
//   pair_sort (seeds.cu)                 both genomes' seed keys in one
//                                       stable radix sort, a genome bit
//                                       below the SML key
//   k_pair_count / k_pair_emit           seeds unique in each genome (strand
//                                       ignored): runs of two, one per
//                                       genome, in ascending seed order =
//                                       the reference's hash order; counted
//                                       per tile, then each pair's
//                                       SetDirection + CalculateOffset +
//                                       bucket id written in that order
//   stable radix sort by bucket          keeps key order inside a bucket
//   k_bucket_replay                      per bucket (a CTA for big buckets,
//                                       a warp for the rest) replays the
//                                       reference's sequence of containment
//                                       tests and inserts exactly: many seeds
//                                       are tested at once against the
//                                       current bucket, the first one not
//                                       contained is extended by its warp
//                                       (match bits of the diagonal cached
//                                       in shared memory) and inserted, and
//                                       the seeds after it are re-tested
//   k_emit                               GetMatchList order: bucket 0..39999,
//                                       then bucket vector order
#include <cooperative_groups.h>

#include "match_common.cuh"

namespace mvg {

// Pass 2 (after the tile counts are scanned): each pair's slot and its hash
// entry: HashMatch (LM/MemHash.cpp:167-187) -> SetDirection (:189-207) ->
// CalculateOffset (LM/MatchHashEntry.cpp:141-162) -> bucket.  A tile's
// entries (at most one per two keys) are staged in shared memory and
// written out contiguously.
template <typename K>
__global__ void __launch_bounds__(256) k_pair_emit(const K* __restrict__ keys, const uint32_t* __restrict__ pos,
                                                   int64_t n, const uint32_t* __restrict__ bstart, int L,
                                                   Mhe* __restrict__ mhe, uint32_t* __restrict__ bucket,
                                                   uint32_t* __restrict__ order) {
  __shared__ Mhe sm[kPairTile / 2];
  __shared__ uint32_t sbk[kPairTile / 2];
  __shared__ uint32_t tile_pairs;
  const int64_t i0 = (int64_t)blockIdx.x * kPairTile + (int64_t)threadIdx.x * kPairItems;
  uint32_t flags = 0;
#pragma unroll
  for (int k = 0; k < kPairItems; ++k)
    if (i0 + k < n && pair_flag(keys, n, i0 + k)) flags |= 1u << k;
  uint32_t li = block_excl_scan256(__popc(flags), &tile_pairs);
  while (flags) {
    const int k = __ffs(flags) - 1;
    flags &= flags - 1;
    const int64_t i = i0 + k;
    const uint64_t k0 = (uint64_t)keys[i], k1 = (uint64_t)keys[i + 1];
    const bool a_first = (k0 & 1ull) == 0;
    const uint64_t ka = a_first ? k0 : k1, kb = a_first ? k1 : k0;
    Mhe m;
    m.s0 = (int64_t)(a_first ? pos[i] : pos[i + 1]) + 1;
    m.s1 = (int64_t)(a_first ? pos[i + 1] : pos[i]) + 1;
    m.len = L;
    const bool ref_forward = !((ka >> 1) & 1ull);
    if (ref_forward == (bool)((kb >> 1) & 1ull)) m.s1 = -m.s1;
    m.off = m.s1 - m.s0;
    if (m.s1 < 0) m.off -= m.len;
    const int64_t t = kTableSize;
    sbk[li] = (uint32_t)(((m.off % t) + t) % t);
    sm[li] = m;
    ++li;
  }
  __syncthreads();
  const uint32_t j0 = bstart[blockIdx.x], np = tile_pairs;
  for (uint32_t q = threadIdx.x; q < np; q += blockDim.x) {
    mhe[j0 + q] = sm[q];
    bucket[j0 + q] = sbk[q];
    order[j0 + q] = j0 + q;
  }
}

// The same hash entries from pairs staged per seed-join bucket
// (pair_buckets.cu): bucket b's pairs go to slots pbase[b] .. in order.
__global__ void __launch_bounds__(256) k_stage_emit(const uint2* __restrict__ stage, const uint32_t* __restrict__ bstart,
                                                    const uint32_t* __restrict__ pcount,
                                                    const uint32_t* __restrict__ pbase, int L, Mhe* __restrict__ mhe,
                                                    uint32_t* __restrict__ bucket, uint32_t* __restrict__ order) {
  const int b = blockIdx.x;
  const uint32_t np = pcount[b], s0 = bstart[b], j0 = pbase[b];
  for (uint32_t q = threadIdx.x; q < np; q += blockDim.x) {
    const uint2 e = stage[s0 + q];
    Mhe m;
    m.s0 = (int64_t)e.x + 1;
    m.s1 = (int64_t)(e.y & 0x7fffffffu) + 1;
    m.len = L;
    if (e.y >> 31) m.s1 = -m.s1;
    m.off = m.s1 - m.s0;
    if (m.s1 < 0) m.off -= m.len;
    const int64_t t = kTableSize;
    mhe[j0 + q] = m;
    bucket[j0 + q] = (uint32_t)(((m.off % t) + t) % t);
    order[j0 + q] = j0 + q;
  }
}

// Buckets with at least kBigBucket seeds get a whole CTA: seeds are staged
// kChunk at a time in shared memory and every open seed of the chunk is
// tested at once against the bucket's entries; the first one not contained
// is extended by warp 0 and inserted, and the test resumes right after it,
// exactly as in the sequential replay.  CTAs past the big buckets run the
// warp-per-bucket replay (32 seeds per test round), 8 buckets each.
constexpr uint32_t kBigBucket = 512;
constexpr int kChunk = 1024;  // seeds staged per chunk (dynamic shared memory)
// Buckets with at least kClusterBucket seeds are replayed by a cluster of
// kClusterCtas CTAs (k_bucket_replay_cluster); one whose entries outgrow the
// per-CTA copy is marked kRedo and replayed by k_bucket_replay instead.
constexpr uint32_t kClusterBucket = 16384;
static_assert(kBigBucket < 0x8000u && kClusterBucket < 0x8000u, "bucket thresholds must be exact in the bucket order");
constexpr int kClusterCtas = 8;
constexpr int kLocalCap = 1536;
constexpr uint32_t kRedo = 0xffffffffu;
extern __shared__ __align__(16) unsigned char replay_dyn_smem[];
static_assert(sizeof(CtaExtRing) <= 8 * sizeof(ExtRing), "the CTA ring reuses the eight warp rings");

__global__ void __launch_bounds__(256) k_bucket_replay(MatchCtx c, const Mhe* __restrict__ mhe,
                                                       const uint32_t* __restrict__ sorted_pair,
                                                       const uint32_t* __restrict__ bstart,
                                                       const uint32_t* __restrict__ bcount,
                                                       const uint32_t* __restrict__ border, Mhe* ent,
                                                       uint32_t* emap, uint32_t* __restrict__ nent_out,
                                                       unsigned long long* __restrict__ coll, int nclusters,
                                                       int redo_pass) {
  __shared__ ExtRing s_ring[8];
  __shared__ Mhe s_x;
  __shared__ long long s_at;
  __shared__ int s_nbig;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int L = c.s.L;
  if (tid == 0) {  // buckets are sorted by descending seed count: count the big ones
    int lo = 0, len = kTableSize;
    while (len > 0) {
      int half = len >> 1;
      if (bcount[border[lo + half]] >= kBigBucket) {
        lo += half + 1;
        len -= half + 1;
      } else {
        len = half;
      }
    }
    s_nbig = lo;
  }
  __syncthreads();
  const int nbig = s_nbig;
  // the cluster pass owns the nclusters largest buckets (if big enough);
  // the redo pass replays only those it handed back
  const bool cluster_owned = (int)blockIdx.x < nclusters && bcount[border[blockIdx.x]] >= kClusterBucket;
  if (redo_pass && !(cluster_owned && nent_out[border[blockIdx.x]] == kRedo)) return;
  if (!redo_pass && cluster_owned) return;
  if ((int)blockIdx.x >= nbig) {
    // ------------------------------------------------ warp per bucket
    const int idx = nbig + ((int)blockIdx.x - nbig) * 8 + wid;
    if (idx >= kTableSize) return;
    const uint32_t b = border[idx];
    const uint32_t cnt = bcount[b];
    if (cnt == 0) return;
    Mhe* E = ent + bstart[b];
    const uint32_t* sp = sorted_pair + bstart[b];
    int64_t n = 0;
    unsigned long long ncoll = 0;
    for (uint32_t base = 0; base < cnt; base += 32) {
      const uint32_t i = base + lane;
      Mhe m = {0, 0, 0, 0};
      if (i < cnt) m = mhe[sp[i]];
      unsigned pending = __ballot_sync(0xffffffffu, i < cnt);
      while (pending) {
        bool coll_here = true;
        if (pending & (1u << lane)) {
          int64_t at = lower_bound_mhe(E, n, m, L);
          coll_here = at != n && !mhe_less(E[at], m, L) && !mhe_less(m, E[at], L);
        }
        const unsigned fresh = __ballot_sync(0xffffffffu, (pending & (1u << lane)) && !coll_here);
        if (!fresh) break;
        const int f = __ffs(fresh) - 1;
        ncoll += __popc(pending & ((1u << f) - 1u));
        pending &= ~((2u << f) - 1u);
        Mhe x;
        x.s0 = __shfl_sync(0xffffffffu, m.s0, f);
        x.s1 = __shfl_sync(0xffffffffu, m.s1, f);
        x.len = __shfl_sync(0xffffffffu, m.len, f);
        x.off = __shfl_sync(0xffffffffu, m.off, f);
        warp_extend(c, x, s_ring[wid]);
        const int64_t at = lower_bound_mhe(E, n, x, L);
        for (int64_t hi = n - 1; hi >= at; hi -= 32) {
          const int64_t k = hi - lane;
          Mhe t;
          if (k >= at) t = E[k];
          __syncwarp();
          if (k >= at) E[k + 1] = t;
          __syncwarp();
        }
        if (lane == 0) E[at] = x;
        __syncwarp();
        ++n;
      }
      ncoll += __popc(pending);
    }
    uint32_t* Mp = emap + bstart[b];  // warp mode keeps the entries in sorted order
    for (int64_t k = lane; k < n; k += 32) Mp[k] = (uint32_t)k;
    if (lane == 0) {
      nent_out[b] = (uint32_t)n;
      atomicAdd(coll, ncoll);
    }
    return;
  }
  // ------------------------------------------------------- CTA per bucket
  // Seeds are staged kChunk at a time in shared memory.  A round tests the
  // chunk's open seeds (kChunk / 256 per thread) against the current
  // entries; the first one not contained is extended and inserted, the ones
  // before it are collisions, and the next round starts right after it -
  // the reference's sequence of tests and inserts, seed by seed.
  Mhe* s_chunk = reinterpret_cast<Mhe*>(replay_dyn_smem);
  __shared__ uint32_t s_wmin[8];
  const uint32_t b = border[blockIdx.x];
  const uint32_t cnt = bcount[b];
  // Entries are appended to the bucket's region G in insertion order; their
  // sorted order is the map Mp (logical position -> slot), so an insert
  // moves 4-byte map words in blocks of 2048 (two barriers per block)
  // instead of 32-byte entries 256 at a time.
  Mhe* G = ent + bstart[b];
  uint32_t* Mp = emap + bstart[b];
  const uint32_t* sp = sorted_pair + bstart[b];
  int64_t n = 0;
  unsigned long long ncoll = 0;
  // number of this thread's chunk slots (cbase + tid + 256 j) in [lo, hi)
  auto mine_in = [&](uint32_t cbase, uint32_t lo, uint32_t hi) -> uint32_t {
    const int64_t first = (int64_t)cbase + tid;
    const int64_t j0 = lo > first ? ((int64_t)lo - first + 255) / 256 : 0;
    const int64_t j1 = hi > first ? ((int64_t)hi - first + 255) / 256 : 0;
    return j1 > j0 ? (uint32_t)(j1 - j0) : 0u;
  };
  for (uint32_t cbase = 0; cbase < cnt; cbase += kChunk) {
    const uint32_t cend = min(cnt, cbase + (uint32_t)kChunk);
    __syncthreads();  // the previous chunk is fully consumed
    for (uint32_t i = cbase + tid; i < cend; i += 256) s_chunk[i - cbase] = mhe[sp[i]];
    __syncthreads();
    uint32_t pos = cbase;
    while (pos < cend) {
      uint32_t myf = 0xffffffffu;
      {
        const int64_t first = (int64_t)cbase + tid;
        int64_t i = pos > first ? first + ((int64_t)pos - first + 255) / 256 * 256 : first;
        for (; i < cend; i += 256) {
          const Mhe m = s_chunk[i - cbase];
          const int64_t at = lower_bound_mapped(G, Mp, n, m, L);
          const bool contained = at != n && !mhe_less(G[Mp[at]], m, L) && !mhe_less(m, G[Mp[at]], L);
          if (!contained) {
            myf = (uint32_t)i;
            break;
          }
        }
      }
      const uint32_t wmin = __reduce_min_sync(0xffffffffu, myf);
      if (lane == 0) s_wmin[wid] = wmin;
      __syncthreads();
      uint32_t f = 0xffffffffu;
#pragma unroll
      for (int q = 0; q < 8; ++q) f = min(f, s_wmin[q]);
      if (f == 0xffffffffu) {
        ncoll += mine_in(cbase, pos, cend);
        pos = cend;
        break;
      }
      ncoll += mine_in(cbase, pos, f);
      Mhe x = s_chunk[f - cbase];
      cta_extend(c, x, *reinterpret_cast<CtaExtRing*>(s_ring));  // the warp rings are idle in this mode
      if (wid == 0) {
        const int64_t at = lower_bound_mapped(G, Mp, n, x, L);
        if (lane == 0) {
          s_x = x;
          s_at = at;
        }
      }
      __syncthreads();
      const int64_t at = s_at;
      for (int64_t hi = n; hi > at; hi -= 2048) {  // Mp[at, n) -> Mp[at + 1, n + 1)
        const int64_t lo = hi - 2048 > at ? hi - 2048 : at;
        uint32_t v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int64_t k = lo + tid + 256 * q;
          if (k < hi) v[q] = Mp[k];
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int64_t k = lo + tid + 256 * q;
          if (k < hi) Mp[k + 1] = v[q];
        }
        __syncthreads();
      }
      if (tid == 0) {
        G[n] = s_x;
        Mp[at] = (uint32_t)n;
      }
      ++n;
      __syncthreads();
      pos = f + 1;
    }
  }
  if (tid == 0) nent_out[b] = (uint32_t)n;
  if (ncoll) atomicAdd(coll, ncoll);
}

// The largest buckets, one per cluster of kClusterCtas CTAs on as many SMs.
// Every CTA keeps its own copy of the bucket's entries (appended, with a
// uint16 sorted-order map) in shared memory and tests its seeds of each
// 16384-seed chunk (8 per thread, in rows of 2048) against it, one row per
// round at first and twice as many rows after every round that finds no
// fresh seed (halved after an insert); the CTAs' first fresh seeds meet in every
// CTA's shared memory (distributed shared memory stores + cluster barrier),
// the CTA owning the first one extends it and sends the new entry and its
// sorted position to every CTA, and all insert it.  The result is the same
// sequence of tests and inserts as the one-CTA replay.  A bucket that grows
// past kLocalCap entries is left untouched and marked kRedo.
constexpr int kClusterItems = 8;  // seeds per thread and chunk
constexpr int kClusterRow = kClusterCtas * 256;
constexpr int kClusterChunk = kClusterRow * kClusterItems;

__device__ __forceinline__ int64_t lower_bound_local(const Mhe* __restrict__ E, const uint16_t* __restrict__ M,
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

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(256, 1)
    k_bucket_replay_cluster(MatchCtx c, const Mhe* __restrict__ mhe, const uint32_t* __restrict__ sorted_pair,
                            const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bcount,
                            const uint32_t* __restrict__ border, Mhe* ent, uint32_t* emap,
                            uint32_t* __restrict__ nent_out, unsigned long long* __restrict__ coll) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const unsigned rank = cl.block_rank();
  Mhe* lent = reinterpret_cast<Mhe*>(replay_dyn_smem);                  // kLocalCap entries
  uint16_t* lmap = reinterpret_cast<uint16_t*>(lent + kLocalCap);      // kLocalCap map words
  __shared__ CtaExtRing s_ring;
  __shared__ uint32_t s_wmin[8];
  __shared__ uint32_t s_cmin[kClusterCtas];  // written by every CTA of the cluster
  __shared__ Mhe s_seed;                     // the fresh seed, inside the owning CTA
  __shared__ Mhe s_x;                        // the new entry, written by the owning CTA
  __shared__ long long s_at;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int L = c.s.L;
  const int cid = (int)(blockIdx.x / kClusterCtas);
  for (int idx = cid; idx == cid; ++idx) {  // the cid-th largest bucket
    const uint32_t b = border[idx];
    const uint32_t cnt = bcount[b];
    if (cnt < kClusterBucket) break;
    const uint32_t* sp = sorted_pair + bstart[b];
    int64_t n = 0;
    bool overflow = false;
    unsigned long long ncoll = 0;
    int rows = 1;  // item rows tested per round
    for (uint32_t cbase = 0; cbase < cnt && !overflow; cbase += kClusterChunk) {
      const uint32_t cend = min(cnt, cbase + (uint32_t)kClusterChunk);
      // slot of item j: cbase + j * kClusterRow + rank * 256 + tid (item order = slot order)
      const uint32_t slot0 = cbase + rank * 256 + tid;
      Mhe m[kClusterItems];
#pragma unroll
      for (int j = 0; j < kClusterItems; ++j) {
        const uint32_t slot = slot0 + j * kClusterRow;
        m[j] = slot < cend ? mhe[sp[slot]] : Mhe{0, 0, 0, 0};
      }
      uint32_t pos = cbase;
      while (pos < cend) {
        const int rlo = (int)((pos - cbase) / kClusterRow);
        const uint32_t limit = min(cend, cbase + (uint32_t)min(kClusterItems, rlo + rows) * kClusterRow);
        uint32_t myf = kRedo;
#pragma unroll
        for (int j = 0; j < kClusterItems; ++j) {
          const uint32_t slot = slot0 + j * kClusterRow;
          if (myf == kRedo && slot < limit && slot >= pos) {
            const int64_t at = lower_bound_local(lent, lmap, n, m[j], L);
            if (!(at != n && !mhe_less(lent[lmap[at]], m[j], L) && !mhe_less(m[j], lent[lmap[at]], L))) myf = slot;
          }
        }
        const uint32_t wmin = __reduce_min_sync(0xffffffffu, myf);
        if (lane == 0) s_wmin[wid] = wmin;
        __syncthreads();
        if (tid < kClusterCtas) {
          uint32_t v = kRedo;
#pragma unroll
          for (int q = 0; q < 8; ++q) v = min(v, s_wmin[q]);
          *cl.map_shared_rank(&s_cmin[rank], tid) = v;  // thread j tells CTA j
        }
        cl.sync();
        uint32_t f = kRedo;
#pragma unroll
        for (int q = 0; q < kClusterCtas; ++q) f = min(f, s_cmin[q]);
        // this thread's seeds in [pos, min(f, limit)) were tested and are collisions
#pragma unroll
        for (int j = 0; j < kClusterItems; ++j) {
          const uint32_t slot = slot0 + j * kClusterRow;
          if (slot < limit && slot >= pos && slot < f) ++ncoll;
        }
        if (f == kRedo) {
          pos = limit;
          rows = min(kClusterItems, 2 * rows);
          cl.sync();  // every CTA has read s_cmin before the next round writes it
          continue;
        }
        const unsigned owner = ((f - cbase) % kClusterRow) / 256;
        if (n == kLocalCap) {  // no room for the entry: hand the bucket to the one-CTA replay
          overflow = true;
          cl.sync();
          break;
        }
        if (rank == owner) {
#pragma unroll
          for (int j = 0; j < kClusterItems; ++j)
            if (slot0 + j * kClusterRow == f) s_seed = m[j];
          __syncthreads();
          Mhe x = s_seed;
          cta_extend(c, x, s_ring);  // the whole owning CTA
          if (wid == 0) {
            const int64_t at = lower_bound_local(lent, lmap, n, x, L);
            if (lane < kClusterCtas) {  // lane j sends the entry to CTA j
              *cl.map_shared_rank(&s_x, lane) = x;
              *cl.map_shared_rank(&s_at, lane) = at;
            }
          }
        }
        cl.sync();
        const int64_t at = s_at;
        for (int64_t hi = n; hi > at; hi -= 2048) {  // lmap[at, n) -> lmap[at + 1, n + 1)
          const int64_t lo = hi - 2048 > at ? hi - 2048 : at;
          uint16_t v[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int64_t k = lo + tid + 256 * q;
            if (k < hi) v[q] = lmap[k];
          }
          __syncthreads();
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int64_t k = lo + tid + 256 * q;
            if (k < hi) lmap[k + 1] = v[q];
          }
          __syncthreads();
        }
        if (tid == 0) {
          lent[n] = s_x;
          lmap[at] = (uint16_t)n;
        }
        ++n;
        __syncthreads();
        pos = f + 1;
        rows = rows > 1 ? rows / 2 : 1;
      }
    }
    // ncoll of the CTAs that finished: summed per CTA
    if (overflow) {
      if (rank == 0 && tid == 0) nent_out[b] = kRedo;
    } else {
      if (rank == 0) {
        Mhe* G = ent + bstart[b];
        uint32_t* Mp = emap + bstart[b];
        for (int64_t k = tid; k < n; k += 256) {
          G[k] = lent[lmap[k]];
          Mp[k] = (uint32_t)k;
        }
        if (tid == 0) nent_out[b] = (uint32_t)n;
      }
      for (int d = 16; d > 0; d >>= 1) ncoll += __shfl_xor_sync(0xffffffffu, ncoll, d);
      if (lane == 0 && ncoll) atomicAdd(coll, ncoll);
    }
    cl.sync();  // the shared copies are reset for the next bucket
  }
}

// Segment of each bucket in the bucket-sorted pair list: two lower_bounds.
__global__ void k_bucket_bounds(const uint32_t* __restrict__ sorted_bucket, int64_t np, uint32_t* __restrict__ start,
                                uint32_t* __restrict__ cnt) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < kTableSize; b += gridDim.x * blockDim.x) {
    int64_t lo[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const uint32_t key = (uint32_t)b + q;
      int64_t first = 0, len = np;
      while (len > 0) {
        const int64_t half = len >> 1;
        if (sorted_bucket[first + half] < key) {
          first += half + 1;
          len -= half + 1;
        } else {
          len = half;
        }
      }
      lo[q] = first;
    }
    start[b] = (uint32_t)lo[0];
    cnt[b] = (uint32_t)(lo[1] - lo[0]);
  }
}

// Largest-first order of the buckets on 16-bit keys (two radix passes
// instead of four): counts below 32,768 exactly, larger ones in steps of
// 128 up to about 4.2 M (clamped above).  The key never decreases with the
// count, and every threshold the replay tests on this order (kBigBucket,
// kClusterBucket) is exact, so those tests stay monotone along it; buckets
// of equal key keep index order.
__device__ __forceinline__ uint32_t lpt_key16(uint32_t c) {
  const uint32_t k = c < 0x8000u ? c : 0x8000u + min(0x7fffu, (c - 0x8000u) >> 7);
  return 0xffffu - k;
}

__global__ void k_lpt_keys(const uint32_t* __restrict__ cnt, uint32_t* __restrict__ key, uint32_t* __restrict__ id) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kTableSize; i += gridDim.x * blockDim.x) {
    key[i] = lpt_key16(cnt[i]);
    id[i] = i;
  }
}

// GetMatchList (LM/MemHash.h:182-203): bucket order, then vector order.
__global__ void k_emit(const Mhe* __restrict__ ent, const uint32_t* __restrict__ emap, const uint32_t* __restrict__ bstart,
                       const uint32_t* __restrict__ nent,
                       const uint32_t* __restrict__ ooff, int64_t* __restrict__ out, uint64_t cap) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int b = gw; b < kTableSize; b += nw) {
    const uint32_t n = nent[b];
    const Mhe* E = ent + bstart[b];
    const uint32_t* M = emap + bstart[b];  // sorted order
    for (uint32_t k = lane; k < n; k += 32) {
      const uint64_t o = (uint64_t)ooff[b] + k;
      if (o < cap) {
        const Mhe& e = E[M[k]];
        out[3 * o + 0] = e.s0;
        out[3 * o + 1] = e.s1;
        out[3 * o + 2] = e.len;
      }
    }
  }
}

int pairwise_matches_dev(Ctx* c, const uint8_t* d_a, uint64_t na, const uint8_t* d_b, uint64_t nb, uint64_t seed,
                         int64_t* d_out, uint64_t cap, uint64_t* count) {
  const SeedDesc s = make_seed_desc(seed);
  if (s.L == 0 || s.L > 31) return report_error(MVG_ERR_ARG, "invalid seed pattern");
  if (na >= 0x7fffffffull || nb >= 0x7fffffffull) return report_error(MVG_ERR_ARG, "genome longer than 2^31-1");
  c->stats = MatchStats();
  *count = 0;
  stage_begin_call(c);
  stage_mark(c, "pack");
  Workspace& ws = c->ws;
  uint32_t* ga = (uint32_t*)ws.get(c, 20, packed_words(na) * 4);
  uint32_t* gb = (uint32_t*)ws.get(c, 21, packed_words(nb) * 4);
  if (!ga || !gb) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
  int rc;
  if ((rc = pack_sequence(c, d_a, na, ga))) return rc;
  if ((rc = pack_sequence(c, d_b, nb, gb))) return rc;
  const uint64_t ca = na >= (uint64_t)s.L ? na - s.L + 1 : 0;
  const uint64_t cb = nb >= (uint64_t)s.L ? nb - s.L + 1 : 0;
  if (ca == 0 || cb == 0) return check_device_error(c);
  // 32-bit keys up to 2^25 of them: the bucketed join; otherwise one sort
  // of both genomes' keys and a join over its runs
  const bool bucketed = 2 * s.w + 2 <= 32 && ca + cb <= kPairBucketMaxKeys;
  SmlKeys sk;
  PairStage ps;
  int64_t nk = 0, ptiles = 0;
  uint32_t* pbs = nullptr;
  uint32_t* d_npairs = nullptr;
  stage_mark(c, "sml_sort");
  if (bucketed) {
    if ((rc = pair_buckets(c, ga, ca, gb, cb, s, &ps))) return rc;
    stage_mark(c, "unique_join");
    d_npairs = (uint32_t*)ws.get(c, 34, 64);
    if (!d_npairs) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    pair_scan_small(ps.pcount, ps.nbuckets, ps.pbase, d_npairs, c->stream);
    c->launches++;
  } else {
    if ((rc = pair_sort(c, ga, ca, gb, cb, s, &sk))) return rc;
    stage_mark(c, "unique_join");
    nk = (int64_t)sk.count;
    ptiles = (nk + kPairTile - 1) / kPairTile;
    pbs = (uint32_t*)ws.get(c, 37, (ptiles + 4) * 4 + 64);
    if (!pbs) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    d_npairs = pbs + ptiles + 2;
    if (sk.wide)
      k_pair_count<uint64_t><<<(unsigned)ptiles, 256, 0, c->stream>>>((const uint64_t*)sk.keys, nk, pbs);
    else
      k_pair_count<uint32_t><<<(unsigned)ptiles, 256, 0, c->stream>>>((const uint32_t*)sk.keys, nk, pbs);
    k_scan_bsums<<<1, 256, 0, c->stream>>>(pbs, ptiles, d_npairs);
    c->launches += 2;
  }
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, d_npairs, 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  const int64_t npairs = (int64_t)(uint32_t)c->h_scalars[0];
  if ((rc = check_device_error(c))) return rc;
  c->stats.pairs = npairs;
  if (npairs == 0) return 0;

  Mhe* mhe = (Mhe*)ws.get(c, 38, npairs * sizeof(Mhe));
  uint32_t* bk0 = (uint32_t*)ws.get(c, 39, npairs * 4);
  uint32_t* bk1 = (uint32_t*)ws.get(c, 40, npairs * 4);
  uint32_t* or0 = (uint32_t*)ws.get(c, 41, npairs * 4);
  uint32_t* or1 = (uint32_t*)ws.get(c, 42, npairs * 4);
  uint32_t* sscr = (uint32_t*)ws.get(c, 43, sort_scratch_words(npairs > kTableSize ? npairs : kTableSize, 32) * 4);
  // per-bucket tables: count, start, nent, lpt key/id x2, out offsets, scan scratch, totals
  uint32_t* btab = (uint32_t*)ws.get(c, 44, (size_t)kTableSize * 4 * 10 + scan_scratch_words(kTableSize) * 4 + 256);
  Mhe* ent = (Mhe*)ws.get(c, 45, npairs * sizeof(Mhe));
  uint32_t* emap = (uint32_t*)ws.get(c, 48, npairs * sizeof(uint32_t));
  if (!mhe || !bk0 || !bk1 || !or0 || !or1 || !sscr || !btab || !ent || !emap)
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  uint32_t* bcount = btab;
  uint32_t* bstart = btab + kTableSize;
  uint32_t* nent = btab + 2 * kTableSize;
  uint32_t* lk0 = btab + 3 * kTableSize;
  uint32_t* li0 = btab + 4 * kTableSize;
  uint32_t* lk1 = btab + 5 * kTableSize;
  uint32_t* li1 = btab + 6 * kTableSize;
  uint32_t* ooff = btab + 7 * kTableSize;
  uint32_t* bscr = btab + 10 * kTableSize;
  uint32_t* tot = bscr + scan_scratch_words(kTableSize);
  // 64-bit counter: round up to an 8-byte boundary (the table above is uint32)
  unsigned long long* d_coll = (unsigned long long*)(((uintptr_t)(tot + 4) + 7) & ~(uintptr_t)7);

  stage_mark(c, "hash_bucket_sort");
  if (bucketed)
    k_stage_emit<<<(unsigned)ps.nbuckets, 256, 0, c->stream>>>(ps.stage, ps.bstart, ps.pcount, ps.pbase, s.L, mhe,
                                                               bk0, or0);
  else if (sk.wide)
    k_pair_emit<uint64_t><<<(unsigned)ptiles, 256, 0, c->stream>>>((const uint64_t*)sk.keys, sk.pos, nk, pbs, s.L,
                                                                   mhe, bk0, or0);
  else
    k_pair_emit<uint32_t><<<(unsigned)ptiles, 256, 0, c->stream>>>((const uint32_t*)sk.keys, sk.pos, nk, pbs, s.L,
                                                                   mhe, bk0, or0);
  c->launches++;
  int which = sort_pairs<uint32_t>(bk0, or0, bk1, or1, npairs, 16, sscr, c->stream, &c->launches, c->d_err);
  uint32_t* sorted_pair = which ? or1 : or0;
  const uint32_t* sorted_bucket = which ? bk1 : bk0;
  MVG_CUDA_TRY(cudaMemsetAsync(nent, 0, (size_t)kTableSize * 4, c->stream));
  MVG_CUDA_TRY(cudaMemsetAsync(d_coll, 0, 8, c->stream));
  k_bucket_bounds<<<grid_for(kTableSize, 256), 256, 0, c->stream>>>(sorted_bucket, npairs, bstart, bcount);
  c->launches++;
  k_lpt_keys<<<grid_for(kTableSize, 256), 256, 0, c->stream>>>(bcount, lk0, li0);
  c->launches++;
  which = sort_pairs<uint32_t>(lk0, li0, lk1, li1, kTableSize, 16, sscr, c->stream, &c->launches, c->d_err);
  const uint32_t* border = which ? li1 : li0;
  MatchCtx mc;
  mc.g[0] = ga;
  mc.g[1] = gb;
  mc.n[0] = (int64_t)na;
  mc.n[1] = (int64_t)nb;
  mc.s = s;
  stage_mark(c, "bucket_replay");
  static bool replay_attr = false;  // once per process: more than 48 KB of shared memory
  const size_t cl_smem = (size_t)kLocalCap * (sizeof(Mhe) + sizeof(uint16_t));
  if (!replay_attr) {
    MVG_CUDA_TRY(cudaFuncSetAttribute(k_bucket_replay, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(kChunk * sizeof(Mhe))));
    MVG_CUDA_TRY(cudaFuncSetAttribute(k_bucket_replay_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)cl_smem));
    replay_attr = true;
  }
  int sms = 0;
  MVG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const int nclusters = sms / kClusterCtas > 0 ? sms / kClusterCtas : 1;
  // the largest buckets on clusters (aux stream) beside everything else
  MVG_CUDA_TRY(cudaEventRecord(c->fork, c->stream));
  MVG_CUDA_TRY(cudaStreamWaitEvent(c->aux, c->fork, 0));
  k_bucket_replay_cluster<<<nclusters * kClusterCtas, 256, cl_smem, c->aux>>>(mc, mhe, sorted_pair, bstart, bcount,
                                                                            border, ent, emap, nent, d_coll);
  MVG_CUDA_TRY(cudaEventRecord(c->join, c->aux));
  c->launches++;
  k_bucket_replay<<<kTableSize, 256, kChunk * sizeof(Mhe), c->stream>>>(mc, mhe, sorted_pair, bstart, bcount, border,
                                                                        ent, emap, nent, d_coll, nclusters, 0);
  MVG_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join, 0));
  // buckets the cluster pass handed back (more entries than a CTA's copy holds)
  k_bucket_replay<<<nclusters, 256, kChunk * sizeof(Mhe), c->stream>>>(mc, mhe, sorted_pair, bstart, bcount, border,
                                                                       ent, emap, nent, d_coll, nclusters, 1);
  c->launches++;
  c->launches++;
  stage_mark(c, "emit");
  exclusive_scan(nent, ooff, kTableSize, bscr, tot + 1, c->stream, &c->launches);
  k_emit<<<kTableSize / 8, 256, 0, c->stream>>>(ent, emap, bstart, nent, ooff, d_out, cap);
  c->launches++;
  stage_end(c);
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, tot + 1, 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars + 1, d_coll, 8, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if ((rc = check_device_error(c))) return rc;
  const uint64_t nm = (uint32_t)c->h_scalars[0];
  c->stats.matches = nm;
  c->stats.collisions = c->h_scalars[1];
  *count = nm;
  if (nm > cap) return report_error(MVG_ERR_CAPACITY, "match output buffer too small");
  return 0;
}

}  // namespace mvg
