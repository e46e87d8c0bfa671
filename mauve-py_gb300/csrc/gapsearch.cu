// Batched gap anchor search: ProgressiveAligner::pairwiseAnchorSearch
// (LM/ProgressiveAligner.cpp:590-679) for every inter-anchor gap of a
// recursion round in one pass over the GPU.
//
// Per gap the reference cuts the two gap sequences out of the genomes, picks
// the seed weight getDefaultSeedWeight of their mean length (no search below
// MIN_DNA_SEED_WEIGHT = 5, LM/SeedMasks.h:375), builds a DNAMemorySML of each
// with the rank-0 spaced seed, runs MemHash::FindMatches (seeds unique in both
// gap sequences, hashed by diagonal offset into 40,000 buckets, extended to
// maximal matches), then EliminateOverlaps_v2 (LM/ProgressiveAligner.h:302-392)
// and LengthFilter(MIN_ANCHOR_LENGTH + 3) (LM/MatchList.h:680-692), and shifts
// the anchors to genome coordinates.  Gaps never interact, so here all gaps
// are one segmented problem:
//
//   k_gs_pack        each gap's sequences 2-bit packed into their own word
//                    range (zero padded like translate32's buffer)
//   k_gs_keys        canonical rank-0 seed mer of every gap position with the
//                    gap's own seed: key = gap << 32 | mer bits | strand | genome
//   radix sort       one stable LSD sort of all gaps' keys
//   k_pair_count /   runs of one key per genome inside a gap (the unique-seed
//   k_gs_pair_emit   enumeration), hash entry and bucket key gap << 16 | bucket
//   radix sort       by bucket key: segments = (gap, bucket), seed order kept
//   k_gs_replay      one warp per segment replays the reference's containment
//                    tests, extensions and inserts (the genome matcher's warp
//                    replay, with the gap's sequences and seed)
//   k_gs_emit        GetMatchList order per gap: bucket, then MheCompare order
//   host             EliminateOverlaps_v2 with std::sort (the order of equal
//                    left ends is the library sort's, as in the reference),
//                    LengthFilter, shift to genome coordinates
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "match_common.cuh"

namespace mvg {

constexpr int kGsMinWeight = 5;      // MIN_DNA_SEED_WEIGHT, LM/SeedMasks.h:375
constexpr int64_t kGsMinAnchor = 12;  // MIN_ANCHOR_LENGTH + 3, LM/Aligner.h:266
constexpr int kGsSlot = 80;           // workspace slots 80..95

// translate32's table (LM/SortedMerList.cpp:29-47) for this module; bit 7
// flags '-'.  Rank-0 seeds by weight (LM/SeedMasks.h:298-321).
__constant__ uint8_t c_gs_base[256];
__constant__ SeedDesc c_gs_seed[32];

struct GapDev {
  uint64_t src[2];   // first base of the gap in genome A / B
  uint64_t word[2];  // first packed word of the gap's A / B sequence
  uint64_t key[2];   // first key slot of the gap's A / B positions
  uint32_t len[2];   // gap lengths
  int32_t w;         // seed weight
  int32_t pad;
};

// Index of the last gap whose field `off` is <= x (offsets ascending).
__device__ __forceinline__ int gap_of(const GapDev* __restrict__ g, int n, int side, int which, uint64_t x) {
  int lo = 0, len = n;
  while (len > 0) {
    const int half = len >> 1;
    const uint64_t v = which == 0 ? g[lo + half].word[side] : g[lo + half].key[side];
    if (v <= x) {
      lo += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return lo - 1;
}

// One thread per packed word of all gaps' sequences (A words, then B words).
__global__ void k_gs_pack(const uint8_t* __restrict__ ga, const uint8_t* __restrict__ gb,
                          const GapDev* __restrict__ gaps, int ngaps, uint64_t words_a, uint64_t words_b,
                          uint32_t* __restrict__ pa, uint32_t* __restrict__ pb, uint32_t* err) {
  const uint64_t total = words_a + words_b, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
    const int side = t < words_a ? 0 : 1;
    const uint64_t w = side ? t - words_a : t;
    const int g = gap_of(gaps, ngaps, side, 0, w);
    const GapDev& d = gaps[g];
    const uint8_t* s = (side ? gb : ga) + d.src[side];
    const uint64_t b0 = (w - d.word[side]) * 16;
    uint32_t word = 0, bad = 0;
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const uint64_t i = b0 + k;
      if (i < d.len[side]) {
        const uint32_t v = c_gs_base[s[i]];
        bad |= v;
        word |= (v & 3u) << (30 - 2 * k);
      }
    }
    if (bad & 0x80u) set_error(err, kDevGapChar);
    (side ? pb : pa)[w] = word;
  }
}

// One thread per seed position of all gaps (A positions, then B positions):
// key = gap << kshift | (seed bits, strand) << 1 | genome, value = position
// in the gap sequence, kshift = 2 * (largest seed weight) + 2 so that the
// sort covers no unused bits.  The (2w+1)-bit SML key orders as the
// reference's mers.
__global__ void k_gs_keys(const uint32_t* __restrict__ pa, const uint32_t* __restrict__ pb,
                          const GapDev* __restrict__ gaps, int ngaps, uint64_t keys_a, uint64_t keys_b, int kshift,
                          uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint64_t total = keys_a + keys_b, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
    const int side = t < keys_a ? 0 : 1;
    const uint64_t k = side ? t - keys_a : t;
    const int g = gap_of(gaps, ngaps, side, 1, k);
    const GapDev& d = gaps[g];
    const SeedDesc& s = c_gs_seed[d.w];
    const uint64_t p = k - d.key[side];
    const uint64_t m = canonical_mer((side ? pb : pa) + d.word[side], p, s);
    const uint64_t sml = ((m >> (64 - 2 * s.w)) << 1) | (m & 1ull);
    keys[t] = ((uint64_t)g << kshift) | (sml << 1) | (uint64_t)side;
    vals[t] = (uint32_t)p;
  }
}

// Hash entries of the unique-seed pairs (k_pair_emit's HashMatch /
// SetDirection / CalculateOffset, LM/MemHash.cpp:167-207,
// LM/MatchHashEntry.cpp:141-162) with each gap's seed length; the bucket key
// puts the gap above the bucket so one sort groups (gap, bucket) segments.
__global__ void __launch_bounds__(256) k_gs_pair_emit(const uint64_t* __restrict__ keys,
                                                      const uint32_t* __restrict__ pos, int64_t n,
                                                      const uint32_t* __restrict__ tstart, int kshift,
                                                      const GapDev* __restrict__ gaps, Mhe* __restrict__ mhe,
                                                      uint64_t* __restrict__ bkey, uint32_t* __restrict__ order) {
  const int64_t i0 = (int64_t)blockIdx.x * kPairTile + (int64_t)threadIdx.x * kPairItems;
  __shared__ uint32_t tile_pairs;
  uint32_t flags = 0;
#pragma unroll
  for (int k = 0; k < kPairItems; ++k)
    if (i0 + k < n && pair_flag(keys, n, i0 + k)) flags |= 1u << k;
  uint32_t li = block_excl_scan256(__popc(flags), &tile_pairs) + tstart[blockIdx.x];
  while (flags) {
    const int k = __ffs(flags) - 1;
    flags &= flags - 1;
    const int64_t i = i0 + k;
    const uint64_t k0 = keys[i], k1 = keys[i + 1];
    const bool a_first = (k0 & 1ull) == 0;
    const uint64_t ka = a_first ? k0 : k1, kb = a_first ? k1 : k0;
    const uint32_t g = (uint32_t)(k0 >> kshift);
    Mhe m;
    m.s0 = (int64_t)(a_first ? pos[i] : pos[i + 1]) + 1;
    m.s1 = (int64_t)(a_first ? pos[i + 1] : pos[i]) + 1;
    m.len = c_gs_seed[gaps[g].w].L;
    const bool ref_forward = !((ka >> 1) & 1ull);
    if (ref_forward == (bool)((kb >> 1) & 1ull)) m.s1 = -m.s1;
    m.off = m.s1 - m.s0;
    if (m.s1 < 0) m.off -= m.len;
    const int64_t ts = kTableSize;
    mhe[li] = m;
    bkey[li] = ((uint64_t)g << 16) | (uint64_t)(((m.off % ts) + ts) % ts);
    order[li] = li;
    ++li;
  }
}

// Segment starts of the bucket-sorted entries: flag 1 where the bucket key
// changes.
__global__ void k_gs_seg_flags(const uint64_t* __restrict__ bkey, int64_t n, uint32_t* __restrict__ flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flag[i] = (i == 0 || bkey[i] != bkey[i - 1]) ? 1u : 0u;
}

__global__ void k_gs_seg_fill(const uint64_t* __restrict__ bkey, int64_t n, const uint32_t* __restrict__ flag,
                              const uint32_t* __restrict__ sidx, uint32_t* __restrict__ seg_start,
                              uint32_t* __restrict__ seg_gap) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (flag[i]) {
      seg_start[sidx[i]] = (uint32_t)i;
      seg_gap[sidx[i]] = (uint32_t)(bkey[i] >> 16);
    }
}

// One warp per (gap, bucket) segment, taken in turn from a counter: the
// reference's AddHashEntry sequence (LM/MemHash.cpp:209-251) over the
// segment's seeds in key order.  32 seeds are tested at a time against the
// bucket's sorted entries; the first one not contained is extended
// (ExtendMatch, LM/MatchFinder.h:218-374, inside the gap's sequences) and
// inserted at its lower_bound, and testing resumes after it.
__global__ void __launch_bounds__(256, 3) k_gs_replay(const uint32_t* __restrict__ pa, const uint32_t* __restrict__ pb,
                                                   const GapDev* __restrict__ gaps, const Mhe* __restrict__ mhe,
                                                   const uint32_t* __restrict__ sorted,
                                                   const uint32_t* __restrict__ seg_start,
                                                   const uint32_t* __restrict__ seg_gap, uint32_t nseg,
                                                   uint32_t nentries, Mhe* __restrict__ ent,
                                                   uint32_t* __restrict__ nent, unsigned* __restrict__ counter) {
  __shared__ ExtRing s_ring[8];
  __shared__ MatchCtx s_ctx[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  MatchCtx& c = s_ctx[wid];
  for (;;) {
    uint32_t sg = 0;
    if (lane == 0) sg = atomicAdd(counter, 1u);
    sg = __shfl_sync(0xffffffffu, sg, 0);
    if (sg >= nseg) return;
    const uint32_t st = seg_start[sg];
    const uint32_t cnt = (sg + 1 < nseg ? seg_start[sg + 1] : nentries) - st;
    const GapDev& d = gaps[seg_gap[sg]];
    if (lane == 0) {
      c.g[0] = pa + d.word[0];
      c.g[1] = pb + d.word[1];
      c.n[0] = d.len[0];
      c.n[1] = d.len[1];
      c.s = c_gs_seed[d.w];
    }
    __syncwarp();
    const int L = c.s.L;
    Mhe* E = ent + st;
    const uint32_t* sp = sorted + st;
    int64_t n = 0;
    for (uint32_t base = 0; base < cnt; base += 32) {
      const uint32_t i = base + lane;
      Mhe m = {0, 0, 0, 0};
      if (i < cnt) m = mhe[sp[i]];
      unsigned pending = __ballot_sync(0xffffffffu, i < cnt);
      while (pending) {
        bool coll_here = true;
        if (pending & (1u << lane)) {
          const int64_t at = lower_bound_mhe(E, n, m, L);
          coll_here = at != n && !mhe_less(E[at], m, L) && !mhe_less(m, E[at], L);
        }
        const unsigned fresh = __ballot_sync(0xffffffffu, (pending & (1u << lane)) && !coll_here);
        if (!fresh) break;
        const int f = __ffs(fresh) - 1;
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
    }
    if (lane == 0) nent[sg] = (uint32_t)n;
    __syncwarp();
  }
}

// Entries of each segment in bucket order (segments are already in (gap,
// bucket) order), rows (start A, start B, length) in gap coordinates.
__global__ void k_gs_emit(const Mhe* __restrict__ ent, const uint32_t* __restrict__ seg_start,
                          const uint32_t* __restrict__ nent, const uint32_t* __restrict__ ooff, uint32_t nseg,
                          int64_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t s = gw; s < nseg; s += nw) {
    const Mhe* E = ent + seg_start[s];
    for (uint32_t k = lane; k < nent[s]; k += 32) {
      const uint64_t o = (uint64_t)ooff[s] + k;
      out[3 * o + 0] = E[k].s0;
      out[3 * o + 1] = E[k].s1;
      out[3 * o + 2] = E[k].len;
    }
  }
}

// ------------------------------------------------------------------ host

static std::mutex g_gs_mu;
static int g_gs_ready_dev = -1;

static int gs_upload_tables(int device) {
  std::lock_guard<std::mutex> lk(g_gs_mu);
  if (g_gs_ready_dev == device) return 0;
  uint8_t t[256] = {};
  for (const char* p = "cCbByY"; *p; ++p) t[(uint8_t)*p] = 1;
  for (const char* p = "gGsSkK"; *p; ++p) t[(uint8_t)*p] = 2;
  t[(uint8_t)'t'] = t[(uint8_t)'T'] = 3;
  t[(uint8_t)'-'] = 0x80;
  MVG_CUDA_TRY(cudaMemcpyToSymbol(c_gs_base, t, 256));
  SeedDesc sd[32];
  for (int w = 0; w < 32; ++w) sd[w] = make_seed_desc(w >= kGsMinWeight ? mvg_get_seed(w, 0) : 0);
  MVG_CUDA_TRY(cudaMemcpyToSymbol(c_gs_seed, sd, sizeof(sd)));
  g_gs_ready_dev = device;
  return 0;
}

namespace {
struct Anchor {
  int64_t s[2];
  int64_t len;
};
int64_t left_end(const Anchor& m, int q) { return m.s[q] < 0 ? -m.s[q] : m.s[q]; }
// CropStart / CropEnd (LM/UngappedLocalAlignment.h:137-152 over
// LM/HybridAbstractMatch.h:271-290): a forward start follows the first
// column, a reverse start the last.
void crop_start(Anchor& m, int64_t k) {
  m.len -= k;
  for (int q = 0; q < 2; ++q)
    if (m.s[q] > 0) m.s[q] += k;
}
void crop_end(Anchor& m, int64_t k) {
  m.len -= k;
  for (int q = 0; q < 2; ++q)
    if (m.s[q] < 0) m.s[q] -= k;
}

// EliminateOverlaps_v2 (eliminate_both = false) on one gap's two-sequence
// matches, then LengthFilter(12): per sequence, sort by left end and walk
// the overlaps, cropping (CropRight / CropLeft in that sequence's
// orientation) or deleting the shorter match; the cropped-off pieces are
// single-sequence matches, which processNewMatch drops.
int64_t filter_gap(Anchor* a, int64_t n, std::vector<Anchor*>& ml) {
  ml.resize(n);
  for (int64_t k = 0; k < n; ++k) ml[k] = a + k;
  if (n >= 2) {
    for (int q = 0; q < 2; ++q) {
      std::sort(ml.begin(), ml.end(), [q](const Anchor* x, const Anchor* y) { return left_end(*x, q) < left_end(*y, q); });
      bool any_deleted = false;
      const int64_t m = (int64_t)ml.size();
      for (int64_t i = 0; i < m; ++i) {
        if (!ml[i]) continue;
        for (int64_t j = i + 1; j < m; ++j) {
          if (!ml[j]) continue;
          const int64_t len_i = ml[i]->len;
          const int64_t over = len_i - (left_end(*ml[j], q) - left_end(*ml[i], q));
          if (over <= 0) break;
          if (ml[j]->len > len_i) {  // i is the shorter: crop its right end or delete it
            if (over >= len_i) {
              ml[i] = nullptr;
              any_deleted = true;
              break;  // the reference steps back to i, finds it deleted and moves on
            }
            if (ml[i]->s[q] > 0) crop_end(*ml[i], over);
            else crop_start(*ml[i], over);
          } else {  // j is: crop its left end or delete it
            if (over >= ml[j]->len) {
              ml[j] = nullptr;
              any_deleted = true;
            } else if (ml[j]->s[q] > 0) {
              crop_start(*ml[j], over);
            } else {
              crop_end(*ml[j], over);
            }
          }
        }
      }
      if (any_deleted) ml.erase(std::remove(ml.begin(), ml.end(), nullptr), ml.end());
    }
  }
  int64_t k = 0;
  std::vector<Anchor> kept;
  kept.reserve(ml.size());
  for (const Anchor* p : ml)
    if (p->len >= kGsMinAnchor) kept.push_back(*p);
  for (const Anchor& x : kept) a[k++] = x;
  return k;
}
}  // namespace

namespace {
// One chunk of a call's gaps: the searched gaps' device descriptors and
// caller indices, the device pass's rows and segment tables, and the host
// pass's filtered anchors.
struct GsChunk {
  std::vector<GapDev> gd;
  std::vector<uint32_t> gid;  // caller's gap index of each searched gap
  uint64_t words[2] = {0, 0}, keys[2] = {0, 0};
  std::vector<int64_t> rows;  // (start A, start B, length) per entry, GetMatchList order per gap
  std::vector<uint32_t> seg_gap, seg_n;
  std::vector<Anchor> anc;     // searched gap gi's survivors at [gap_r[gi], gap_r[gi] + nkept[gi])
  std::vector<size_t> gap_r;
  std::vector<int64_t> nkept;
};

// Runs fn(i) for i in [0, n) on up to nthreads host threads that claim runs
// of 16 indices from a counter.
template <class F>
void run_claimed(int n, int nthreads, F&& fn) {
  std::atomic<int> next{0};
  auto worker = [&]() {
    for (;;) {
      const int i0 = next.fetch_add(16);
      if (i0 >= n) break;
      for (int i = i0; i < std::min(n, i0 + 16); ++i) fn(i);
    }
  };
  if (nthreads > 1) {
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker);
    for (std::thread& th : pool) th.join();
  } else {
    worker();
  }
}

int host_threads_for(size_t items) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  return (int)std::min<uint64_t>(hw, std::max<uint64_t>(1, items / 20000));
}
}  // namespace

// Host plan of gaps [g0, g1) (already validated): seed weights, word and key
// ranges of the gaps that are searched.
static int gs_plan(const int64_t* gaps, uint64_t g0, uint64_t g1, GsChunk& ch) {
  for (uint64_t g = g0; g < g1; ++g) {
    const int64_t* q = gaps + 4 * g;
    const unsigned w = mvg_default_seed_weight((uint64_t)(q[1] + q[3]) / 2);
    if (w < (unsigned)kGsMinWeight) continue;  // the reference returns without searching
    if (w > 15)
      return report_error(MVG_ERR_ARG, "gap of mean length above 5.9 Mbp (seed weight above 15): search it with "
                                       "mvg_pairwise_matches and the rank-0 seed");
    const int L = mvg_seed_length(mvg_get_seed((int)w, 0));
    GapDev d{};
    d.w = (int32_t)w;
    for (int s = 0; s < 2; ++s) {
      const uint64_t len = (uint64_t)q[1 + 2 * s];
      d.src[s] = (uint64_t)q[2 * s];
      d.len[s] = (uint32_t)len;
      d.word[s] = ch.words[s];
      d.key[s] = ch.keys[s];
      ch.words[s] += packed_words(len);  // translate32's layout: two zero words after each gap
      ch.keys[s] += len >= (uint64_t)L ? len - L + 1 : 0;
    }
    ch.gd.push_back(d);
    ch.gid.push_back((uint32_t)g);
  }
  return 0;
}

// Device pass of one chunk, from packing to the emitted rows, which are
// copied to the host with the segment tables.  Synchronous.
static int gs_device(Ctx* c, const uint8_t* d_a, const uint8_t* d_b, GsChunk& ch) {
  const int ng = (int)ch.gd.size();
  if (ng == 0) return 0;
  const std::vector<GapDev>& gd = ch.gd;
  const uint64_t* words = ch.words;
  const uint64_t* keys = ch.keys;
  std::vector<int64_t>& rows = ch.rows;
  std::vector<uint32_t>& seg_gap = ch.seg_gap;
  std::vector<uint32_t>& seg_n = ch.seg_n;
  const uint64_t nkeys = keys[0] + keys[1];
  int rc = 0;
  if (nkeys >= (1ull << 31)) return report_error(MVG_ERR_ARG, "gaps hold more than 2^31 seed positions");
  Workspace& ws = c->ws;
  GapDev* d_gaps = (GapDev*)ws.get(c, kGsSlot + 0, gd.size() * sizeof(GapDev));
  uint32_t* pa = (uint32_t*)ws.get(c, kGsSlot + 1, words[0] * 4 + 64);
  uint32_t* pb = (uint32_t*)ws.get(c, kGsSlot + 2, words[1] * 4 + 64);
  uint64_t* k0 = (uint64_t*)ws.get(c, kGsSlot + 3, nkeys * 8);
  uint64_t* k1 = (uint64_t*)ws.get(c, kGsSlot + 4, nkeys * 8);
  uint32_t* v0 = (uint32_t*)ws.get(c, kGsSlot + 5, nkeys * 4);
  uint32_t* v1 = (uint32_t*)ws.get(c, kGsSlot + 6, nkeys * 4);
  int gbits = 1;
  while ((1ll << gbits) < ng) ++gbits;
  // (seed bits, strand, genome) below the gap index; a seed's bits are its
  // pattern's selected positions, which for some table entries exceed the
  // nominal weight (weight 11's rank-0 seed selects 12)
  int wmax = 0;
  for (const GapDev& d : gd) wmax = std::max(wmax, __builtin_popcountll(mvg_get_seed((int)d.w, 0)));
  const int kshift = 2 * wmax + 2;
  const int64_t ptiles = ((int64_t)nkeys + kPairTile - 1) / kPairTile;
  uint32_t* sscr = (uint32_t*)ws.get(c, kGsSlot + 7, sort_scratch_words((int64_t)nkeys, std::max(kshift, 16) + gbits) * 4);  // both sorts below
  uint32_t* tsum = (uint32_t*)ws.get(c, kGsSlot + 8, (ptiles + 4) * 4 + 64);
  if (!d_gaps || !pa || !pb || !k0 || !k1 || !v0 || !v1 || !sscr || !tsum)
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  uint32_t* d_npairs = tsum + ptiles + 2;
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  stage_mark(c, "gs_pack");
  MVG_CUDA_TRY(cudaMemcpyAsync(d_gaps, gd.data(), gd.size() * sizeof(GapDev), cudaMemcpyHostToDevice, c->stream));
  k_gs_pack<<<grid_for(words[0] + words[1], 256), 256, 0, c->stream>>>(d_a, d_b, d_gaps, ng, words[0], words[1],
                                                                        pa, pb, c->d_err);
  c->launches++;
  if (keys[0] == 0 || keys[1] == 0) {  // no seed in one genome's gaps: no match anywhere
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
  }
  stage_mark(c, "gs_keys");
  k_gs_keys<<<grid_for(nkeys, 256), 256, 0, c->stream>>>(pa, pb, d_gaps, ng, keys[0], keys[1], kshift, k0,
                                                         v0);
  c->launches++;
  stage_mark(c, "gs_seed_sort");
  int which = sort_pairs<uint64_t>(k0, v0, k1, v1, (int64_t)nkeys, kshift + gbits, sscr, c->stream, &c->launches,
                                   c->d_err);
  const uint64_t* sk = which ? k1 : k0;
  const uint32_t* sv = which ? v1 : v0;
  stage_mark(c, "gs_pairs");
  k_pair_count<uint64_t><<<(unsigned)ptiles, 256, 0, c->stream>>>(sk, (int64_t)nkeys, tsum);
  k_scan_bsums<<<1, 256, 0, c->stream>>>(tsum, ptiles, d_npairs);
  c->launches += 2;
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, d_npairs, 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if ((rc = check_device_error(c))) return rc;
  const int64_t npairs = (int64_t)(uint32_t)c->h_scalars[0];
  if (npairs > 0) {
    Mhe* mhe = (Mhe*)ws.get(c, kGsSlot + 9, npairs * sizeof(Mhe));
    Mhe* ent = (Mhe*)ws.get(c, kGsSlot + 10, npairs * sizeof(Mhe));
    uint64_t* bk0 = (uint64_t*)ws.get(c, kGsSlot + 11, npairs * 8);
    uint64_t* bk1 = (uint64_t*)ws.get(c, kGsSlot + 12, npairs * 8);
    uint32_t* o0 = (uint32_t*)ws.get(c, kGsSlot + 13, npairs * 4);
    uint32_t* o1 = (uint32_t*)ws.get(c, kGsSlot + 14, npairs * 4);
    // per entry: segment flag, segment index; per segment: start, gap, entries, output offset
    uint32_t* segtab = (uint32_t*)ws.get(c, kGsSlot + 15, (size_t)npairs * 4 * 6 + scan_scratch_words(npairs) * 8 + 256);
    if (!mhe || !ent || !bk0 || !bk1 || !o0 || !o1 || !segtab)
      return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    uint32_t* flag = segtab;
    uint32_t* sidx = flag + npairs;
    uint32_t* seg_start = sidx + npairs;
    uint32_t* d_seg_gap = seg_start + npairs;
    uint32_t* nent = d_seg_gap + npairs;
    uint32_t* ooff = nent + npairs;
    uint32_t* scr = ooff + npairs;
    uint32_t* totals = scr + scan_scratch_words(npairs) * 2;  // [0] segments, [1] entries, [2] counter
    k_gs_pair_emit<<<(unsigned)ptiles, 256, 0, c->stream>>>(sk, sv, (int64_t)nkeys, tsum, kshift, d_gaps, mhe, bk0,
                                                            o0);
    c->launches++;
    stage_mark(c, "gs_bucket_sort");
    which = sort_pairs<uint64_t>(bk0, o0, bk1, o1, npairs, 16 + gbits, sscr, c->stream, &c->launches, c->d_err);
    const uint64_t* sbk = which ? bk1 : bk0;
    const uint32_t* sorted = which ? o1 : o0;
    k_gs_seg_flags<<<grid_for(npairs, 256), 256, 0, c->stream>>>(sbk, npairs, flag);
    exclusive_scan(flag, sidx, npairs, scr, totals, c->stream, &c->launches);
    k_gs_seg_fill<<<grid_for(npairs, 256), 256, 0, c->stream>>>(sbk, npairs, flag, sidx, seg_start, d_seg_gap);
    c->launches += 2;
    MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, totals, 4, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaMemsetAsync(totals + 2, 0, 4, c->stream));
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const uint32_t nseg = (uint32_t)c->h_scalars[0];
    int sms = 0;
    MVG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    const uint32_t rblocks = std::min<uint32_t>((nseg + 7) / 8, (uint32_t)sms * 8);
    stage_mark(c, "gs_replay");
    k_gs_replay<<<rblocks, 256, 0, c->stream>>>(pa, pb, d_gaps, mhe, sorted, seg_start, d_seg_gap, nseg,
                                                (uint32_t)npairs, ent, nent, totals + 2);
    stage_mark(c, "gs_emit");
    exclusive_scan(nent, ooff, nseg, scr, totals + 1, c->stream, &c->launches);
    MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, totals + 1, 4, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const uint64_t nrows = (uint32_t)c->h_scalars[0];
    int64_t* d_rows = (int64_t*)ws.get(c, kGsSlot + 3, nrows * 24 + 24);  // the key buffer is free again
    if (!d_rows) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    k_gs_emit<<<grid_for((uint64_t)nseg * 32, 256), 256, 0, c->stream>>>(ent, seg_start, nent, ooff, nseg, d_rows);
    c->launches += 2;
    rows.resize(nrows * 3);
    seg_gap.resize(nseg);
    seg_n.resize(nseg);
    if (nrows) MVG_CUDA_TRY(cudaMemcpyAsync(rows.data(), d_rows, nrows * 24, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaMemcpyAsync(seg_gap.data(), d_seg_gap, (size_t)nseg * 4, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaMemcpyAsync(seg_n.data(), nent, (size_t)nseg * 4, cudaMemcpyDeviceToHost, c->stream));
    stage_mark(c, "gs_copy");
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if ((rc = check_device_error(c))) return rc;
  }
  return 0;
}

// Host pass of one chunk: per gap, overlap elimination and length filter,
// then genome coordinates.  Gaps are independent and their anchor counts
// differ by orders of magnitude, so host threads claim runs of gaps, each
// converting, filtering and shifting its gaps' rows in place.
static void gs_filter(GsChunk& ch) {
  const int ng = (int)ch.gd.size();
  ch.anc.resize(ch.rows.size() / 3);
  ch.gap_r.assign(ng + 1, 0);  // rows of searched gap gi: [gap_r[gi], gap_r[gi+1])
  for (size_t s = 0, r = 0, gi = 0; gi < (size_t)ng; ++gi) {
    while (s < ch.seg_gap.size() && ch.seg_gap[s] == (uint32_t)gi) r += ch.seg_n[s++];
    ch.gap_r[gi + 1] = r;
  }
  ch.nkept.assign(ng, 0);
  run_claimed(ng, host_threads_for(ch.anc.size()), [&](int gi) {
    thread_local std::vector<Anchor*> scratch;
    const size_t r0 = ch.gap_r[gi], r1 = ch.gap_r[gi + 1];
    for (size_t k = r0; k < r1; ++k)
      ch.anc[k] = Anchor{{ch.rows[3 * k], ch.rows[3 * k + 1]}, ch.rows[3 * k + 2]};
    const int64_t k = filter_gap(ch.anc.data() + r0, (int64_t)(r1 - r0), scratch);
    const GapDev& d = ch.gd[gi];
    for (int64_t u = 0; u < k; ++u)
      for (int q = 0; q < 2; ++q) {
        int64_t& x = ch.anc[r0 + u].s[q];
        x = x > 0 ? x + (int64_t)d.src[q] : x - (int64_t)d.src[q];
      }
    ch.nkept[gi] = k;
  });
}

// Gaps are searched in up to four chunks of about equal sequence: the host
// pass of one chunk runs on host threads while the device pass of the next
// runs on the GPU.
int gap_anchor_search_dev(Ctx* c, const uint8_t* d_a, uint64_t na, const uint8_t* d_b, uint64_t nb,
                          const int64_t* gaps, uint64_t ngaps, int64_t* out, uint64_t cap, uint64_t* gap_off,
                          uint64_t* count) {
  *count = 0;
  stage_begin_call(c);
  if (ngaps >= (1ull << 31)) return report_error(MVG_ERR_ARG, "too many gaps");
  int rc = gs_upload_tables(c->device);
  if (rc) return rc;
  uint64_t total_bases = 0;
  for (uint64_t g = 0; g < ngaps; ++g) {
    const int64_t* q = gaps + 4 * g;
    if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[3] < 0 || (uint64_t)(q[0] + q[1]) > na ||
        (uint64_t)(q[2] + q[3]) > nb)
      return report_error(MVG_ERR_RANGE, "gap outside its genome");
    if (q[1] >= (1ll << 31) || q[3] >= (1ll << 31)) return report_error(MVG_ERR_ARG, "gap longer than 2^31-1");
    total_bases += (uint64_t)(q[1] + q[3]);
  }
  const int nchunks = (int)std::max<uint64_t>(1, std::min<uint64_t>(4, total_bases / (32ull << 20)));
  std::vector<uint64_t> bound(nchunks + 1, ngaps);
  bound[0] = 0;
  for (uint64_t g = 0, acc = 0, k = 1; g < ngaps && k < (uint64_t)nchunks; ++g) {
    acc += (uint64_t)(gaps[4 * g + 1] + gaps[4 * g + 3]);
    if (acc * nchunks >= total_bases * k) bound[k++] = g + 1;
  }
  std::vector<GsChunk> chunks(nchunks);
  std::thread filt;  // the host pass of the previous chunk
  struct Joiner {
    std::thread& t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } joiner{filt};
  for (int k = 0; k < nchunks; ++k) {
    if ((rc = gs_plan(gaps, bound[k], bound[k + 1], chunks[k]))) return rc;
    if ((rc = gs_device(c, d_a, d_b, chunks[k]))) return rc;
    HostSpan wait(c, "gs_filter_wait");
    if (filt.joinable()) filt.join();
    filt = std::thread(gs_filter, std::ref(chunks[k]));
  }
  {
    HostSpan wait(c, "gs_filter_wait");
    filt.join();
  }
  stage_end(c);
  std::vector<uint64_t> per_gap(ngaps, 0);
  uint64_t total = 0;
  std::vector<std::pair<int, int>> where;  // (chunk, searched gap) in caller order
  std::vector<uint64_t> obase;             // output row of each searched gap's first survivor
  for (int k = 0; k < nchunks; ++k)
    for (size_t gi = 0; gi < chunks[k].gd.size(); ++gi) {
      const int64_t n = chunks[k].nkept[gi];
      per_gap[chunks[k].gid[gi]] = (uint64_t)n;
      where.push_back({k, (int)gi});
      obase.push_back(total);
      total += (uint64_t)n;
    }
  if (gap_off) {
    gap_off[0] = 0;
    for (uint64_t g = 0; g < ngaps; ++g) gap_off[g + 1] = gap_off[g] + per_gap[g];
  }
  *count = total;
  if (total > cap) return report_error(MVG_ERR_CAPACITY, "anchor output buffer too small");
  // searched-gap order is the caller's gap order
  run_claimed((int)where.size(), host_threads_for(total), [&](int i) {
    const GsChunk& ch = chunks[where[i].first];
    const int gi = where[i].second;
    for (int64_t u = 0; u < ch.nkept[gi]; ++u) {
      const Anchor& x = ch.anc[ch.gap_r[gi] + u];
      int64_t* o = out + 3 * (obase[i] + (uint64_t)u);
      o[0] = x.s[0];
      o[1] = x.s[1];
      o[2] = x.len;
    }
  });
  return 0;
}

}  // namespace mvg

using namespace mvg;

static Ctx* gs_ctx(mvg_handle h) { return reinterpret_cast<Ctx*>(h); }

extern "C" int mvg_gap_anchor_search_dev(mvg_handle h, const uint8_t* d_seq_a, uint64_t na, const uint8_t* d_seq_b,
                                         uint64_t nb, const int64_t* gaps, uint64_t ngaps, int64_t* out,
                                         uint64_t cap, uint64_t* gap_off, uint64_t* count) {
  if (!h || !count || (!gaps && ngaps) || (!out && cap) || (!d_seq_a && na) || (!d_seq_b && nb))
    return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = gs_ctx(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  return gap_anchor_search_dev(c, d_seq_a, na, d_seq_b, nb, gaps, ngaps, out, cap, gap_off, count);
}

extern "C" int mvg_gap_anchor_search(mvg_handle h, const uint8_t* seq_a, uint64_t na, const uint8_t* seq_b,
                                     uint64_t nb, const int64_t* gaps, uint64_t ngaps, int64_t* out, uint64_t cap,
                                     uint64_t* gap_off, uint64_t* count) {
  if (!h || !count || (!gaps && ngaps) || (!out && cap) || (!seq_a && na) || (!seq_b && nb))
    return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = gs_ctx(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  uint8_t* da = (uint8_t*)c->ws.get(c, 46, na + 16);
  uint8_t* db = (uint8_t*)c->ws.get(c, 47, nb + 16);
  if (!da || !db) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (na) MVG_CUDA_TRY(cudaMemcpyAsync(da, seq_a, na, cudaMemcpyHostToDevice, c->stream));
  if (nb) MVG_CUDA_TRY(cudaMemcpyAsync(db, seq_b, nb, cudaMemcpyHostToDevice, c->stream));
  return gap_anchor_search_dev(c, da, na, db, nb, gaps, ngaps, out, cap, gap_off, count);
}
