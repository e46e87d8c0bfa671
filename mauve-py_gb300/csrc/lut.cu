// Genome -> reference index LUT on the GPU.
//
// Construction from aligned blocks follows mauve/buildindex.py:112-130: per
// block, each side's index starts at start-1 and advances on a non-gap
// character; a column whose two characters are equal writes
// lut[genome_idx] = ref_idx when genome_idx < n (genome_idx == -1 wraps to
// n-1 as a numpy index does).  Later blocks and later columns overwrite
// earlier ones.
//
//   k_seg_count / scan / k_seg_fill  cut blocks into segments of kSegCols
//   k_lut_count                       per-segment non-gap counts of both rows
//   scan (x2)                         global exclusive prefix per segment
//   k_lut_walk                        per-column indices; each write is an
//                                     atomicMax of ((column+1) << 32 | value)
//                                     so the last writer in column order wins
//   k_lut_finish                      keys -> int32 LUT (-1 where unwritten)
//
// fillGaps / smoothEdges / findGaps (mauve/indexutils.pyx:47-139) run
// sequentially in place in the reference.  Their decisions depend only on
// the LUT as it was before the pass, except that a fill [g-1, u] hides every
// later gap start inside (g, u] (see the proof in k_fill_resolve).  So:
//
//   k_fill_flags / scan      gap starts of the unmodified LUT, compacted
//   k_fill_search            one warp per gap start: first partner u in
//                            (g, g+width] (ballot over 32 columns per step)
//   k_fill_resolve           gap starts that no earlier start's reach covers
//                            are certain; each walks its cluster forward
//   k_fill_apply             one warp per performed fill writes the run
#include "mvg_internal.h"
#include "prim.cuh"

namespace mvg {
namespace {

constexpr int kSegCols = 4096;     // columns per segment (256 threads x 16)
constexpr int kColsPerThread = 16;
constexpr int kLutThreads = 256;

// ------------------------------------------------------------ construction

__global__ void k_seg_count(const uint64_t* __restrict__ col_off, uint64_t nblocks, uint32_t* __restrict__ nseg,
                            uint32_t* err) {
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks;
       b += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t a = col_off[b], e = col_off[b + 1];
    if (e < a) {
      set_error(err, kDevRange);
      nseg[b] = 0;
      continue;
    }
    nseg[b] = (uint32_t)((e - a + kSegCols - 1) / kSegCols);
  }
}

__global__ void k_seg_fill(const uint32_t* __restrict__ nseg, const uint32_t* __restrict__ seg_start,
                           uint64_t nblocks, uint32_t* __restrict__ seg_block) {
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks;
       b += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s0 = seg_start[b], k = nseg[b];
    for (uint32_t q = 0; q < k; ++q) seg_block[s0 + q] = (uint32_t)b;
  }
}

struct SegRange {
  uint64_t begin, end;
  uint32_t block;
};

__device__ __forceinline__ SegRange seg_range(uint32_t seg, const uint32_t* seg_block, const uint32_t* seg_start,
                                              const uint64_t* col_off) {
  SegRange r;
  r.block = seg_block[seg];
  r.begin = col_off[r.block] + (uint64_t)(seg - seg_start[r.block]) * kSegCols;
  const uint64_t e = col_off[r.block + 1];
  r.end = r.begin + kSegCols < e ? r.begin + kSegCols : e;
  return r;
}

// Non-gap counts of this thread's columns, packed (genome | ref << 16).
__device__ __forceinline__ uint32_t thread_counts(const uint8_t* __restrict__ g, const uint8_t* __restrict__ r,
                                                  uint64_t c0, uint64_t c1) {
  uint32_t cg = 0, cr = 0;
  for (uint64_t c = c0; c < c1; ++c) {
    cg += g[c] != '-';
    cr += r[c] != '-';
  }
  return cg | (cr << 16);
}

__global__ void __launch_bounds__(kLutThreads) k_lut_count(const uint8_t* __restrict__ g, const uint8_t* __restrict__ r,
                                                           const uint32_t* __restrict__ seg_block,
                                                           const uint32_t* __restrict__ seg_start,
                                                           const uint64_t* __restrict__ col_off,
                                                           uint32_t* __restrict__ seg_g, uint32_t* __restrict__ seg_r) {
  const uint32_t seg = blockIdx.x;
  const SegRange sr = seg_range(seg, seg_block, seg_start, col_off);
  const uint64_t c0 = sr.begin + (uint64_t)threadIdx.x * kColsPerThread;
  const uint64_t c1 = c0 + kColsPerThread < sr.end ? c0 + kColsPerThread : sr.end;
  uint32_t v = c0 < sr.end ? thread_counts(g, r, c0, c1) : 0;
  __shared__ uint32_t stot;
  block_excl_scan256(v, &stot);
  if (threadIdx.x == 0) {
    seg_g[seg] = stot & 0xffffu;
    seg_r[seg] = stot >> 16;
  }
}

// Per column: indices after this column, and the keyed write.
__global__ void __launch_bounds__(kLutThreads) k_lut_walk(const uint8_t* __restrict__ g, const uint8_t* __restrict__ r,
                                                          const uint32_t* __restrict__ seg_block,
                                                          const uint32_t* __restrict__ seg_start,
                                                          const uint64_t* __restrict__ col_off,
                                                          const uint32_t* __restrict__ pre_g,
                                                          const uint32_t* __restrict__ pre_r,
                                                          const int64_t* __restrict__ g_start,
                                                          const int64_t* __restrict__ r_start, int64_t n,
                                                          unsigned long long* __restrict__ keys, uint32_t* err) {
  const uint32_t seg = blockIdx.x;
  const SegRange sr = seg_range(seg, seg_block, seg_start, col_off);
  const uint64_t c0 = sr.begin + (uint64_t)threadIdx.x * kColsPerThread;
  const uint64_t c1 = c0 + kColsPerThread < sr.end ? c0 + kColsPerThread : sr.end;
  const uint32_t v = c0 < sr.end ? thread_counts(g, r, c0, c1) : 0;
  __shared__ uint32_t stot;
  const uint32_t ex = block_excl_scan256(v, &stot);
  if (c0 >= sr.end) return;
  const uint32_t first = seg_start[sr.block];
  int64_t gi = g_start[sr.block] - 1 + (int64_t)(pre_g[seg] - pre_g[first]) + (int64_t)(ex & 0xffffu);
  int64_t ri = r_start[sr.block] - 1 + (int64_t)(pre_r[seg] - pre_r[first]) + (int64_t)(ex >> 16);
  for (uint64_t c = c0; c < c1; ++c) {
    const uint8_t gc = g[c], rc = r[c];
    gi += gc != '-';
    ri += rc != '-';
    if (gc == rc && gi < n) {
      const int64_t t = gi < 0 ? gi + n : gi;
      if (t < 0) {
        set_error(err, kDevRange);
        continue;
      }
      if (ri < INT32_MIN || ri > INT32_MAX) {
        set_error(err, kDevOverflow);
        continue;
      }
      const unsigned long long key = ((unsigned long long)(c + 1) << 32) | (uint32_t)(int32_t)ri;
      atomicMax(keys + t, key);
    }
  }
}

__global__ void k_lut_finish(const unsigned long long* __restrict__ keys, int64_t n, int32_t* __restrict__ lut) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    lut[i] = k ? (int32_t)(uint32_t)k : -1;
  }
}

// ------------------------------------------------------------ fixZeroIdx

// mauve/indexutils.pyx:27-44: if lut[0] == -1, the first index nx >= 10
// with lut[nx] != -1 gives ref_idx = lut[nx] - nx; lut[0] = ref_idx when
// ref_idx >= 0 and genome[0] == ref[ref_idx].  The Cython loop reads lut[nx]
// for every nx up to that index with bounds checks, so no such index (or a
// LUT of at most 10 entries) is an IndexError, as are an empty genome and
// ref_idx past the reference.  One CTA scans 256 indices per step.
__global__ void __launch_bounds__(256) k_fix_zero(int32_t* __restrict__ lut, int64_t n,
                                                  const uint8_t* __restrict__ genome, uint64_t glen,
                                                  const uint8_t* __restrict__ ref, uint64_t rlen, uint32_t* err) {
  if (lut[0] != -1) return;
  __shared__ int64_t found;
  if (threadIdx.x == 0) found = -1;
  __syncthreads();
  for (int64_t base = 10; base < n; base += 256) {
    const int64_t i = base + threadIdx.x;
    const bool hit = i < n && lut[i] != -1;
    const int any = __syncthreads_or(hit);
    if (any) {
      // lowest hitting index: one pass over the warps' ballots
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      __shared__ unsigned wb[8];
      if ((threadIdx.x & 31) == 0) wb[threadIdx.x >> 5] = bal;
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int w = 0; w < 8; ++w)
          if (wb[w]) {
            found = base + w * 32 + __ffs(wb[w]) - 1;
            break;
          }
      }
      __syncthreads();
      break;
    }
  }
  if (threadIdx.x != 0) return;
  if (found < 0) {
    set_error(err, kDevRange);
    return;
  }
  const int32_t ref_idx = (int32_t)((uint32_t)lut[found] - (uint32_t)found);
  if (ref_idx > -1) {
    if (glen == 0 || (uint64_t)ref_idx >= rlen) {
      set_error(err, kDevRange);
      return;
    }
    if (genome[0] == ref[ref_idx]) lut[0] = ref_idx;
  }
}

// ------------------------------------------------ fillGaps / smoothEdges

enum FillMode : int { kFill = 0, kSmooth = 1 };

__device__ __forceinline__ bool gap_start(const int32_t* lut, int64_t i, int mode) {
  const int32_t lo = lut[i - 1], m = lut[i];
  if (lo == -1) return false;
  return mode == kSmooth ? m != (int32_t)((uint32_t)lo + 1u) : m == -1;
}

__global__ void k_fill_flags(const int32_t* __restrict__ lut, int64_t n, int mode, uint32_t* __restrict__ flags) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flags[i] = i > 0 && gap_start(lut, i, mode);
}

__global__ void k_fill_compact(const int32_t* __restrict__ lut, int64_t n, int mode,
                               const uint32_t* __restrict__ pos, int32_t* __restrict__ cand) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (i > 0 && gap_start(lut, i, mode)) cand[pos[i]] = (int32_t)i;
}

// One warp per gap start g (lower = g-1, L = lut[lower]): the first u in
// g+1 .. min(n-1, g+width) with lut[u] - L == u - lower (int32 arithmetic),
// 32 columns per step.  reach = u, or g when there is none.
__global__ void k_fill_search(const int32_t* __restrict__ lut, int64_t n, int width,
                              const int32_t* __restrict__ cand, int64_t ncand, int32_t* __restrict__ reach) {
  const int lane = threadIdx.x & 31;
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ncand;
       k += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t gs = cand[k], lower = gs - 1;
    const int32_t L = lut[lower];
    int64_t last = gs + width;
    if (last > n - 1) last = n - 1;
    int32_t u = (int32_t)gs;
    for (int64_t base = gs + 1; base <= last; base += 32) {
      const int64_t up = base + lane;
      const bool ok = up <= last && (int32_t)((uint32_t)lut[up] - (uint32_t)L) == (int32_t)(up - lower);
      const unsigned bal = __ballot_sync(0xffffffffu, ok);
      if (bal) {
        u = (int32_t)(base + __ffs(bal) - 1);
        break;
      }
    }
    if (lane == 0) reach[k] = u;
  }
}

// Sequential semantics, restated: a fill from gap start g rewrites
// [g-1, u]; afterwards every position in (g, u] continues the run, so no
// gap start of the unmodified LUT inside (g, u] is one any more, while the
// value at u (the old lut[u]) and everything after u are untouched.  Hence
// a gap start is performed iff no PERFORMED earlier start reaches it, and
// the search of a performed start sees the unmodified LUT.  A start that no
// earlier start reaches at all (performed or not) is certainly performed:
// it heads a cluster.  Its thread walks the cluster: from a performed start
// the next performed one is the first start beyond its reach; the walk ends
// at the next cluster head.  reach(g) <= g + width, so heads are found by
// looking back over starts within width positions.
__device__ __forceinline__ bool cluster_head(const int32_t* cand, const int32_t* reach, int64_t k, int width) {
  const int64_t g = cand[k];
  for (int64_t j = k - 1; j >= 0 && (int64_t)cand[j] + width >= g; --j)
    if (reach[j] >= g) return false;
  return true;
}

__global__ void k_fill_heads(const int32_t* __restrict__ cand, const int32_t* __restrict__ reach, int64_t ncand,
                             int width, uint8_t* __restrict__ head) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ncand; k += (int64_t)gridDim.x * blockDim.x)
    head[k] = cluster_head(cand, reach, k, width);
}

__global__ void k_fill_resolve(const int32_t* __restrict__ cand, const int32_t* __restrict__ reach, int64_t ncand,
                               const uint8_t* __restrict__ head, uint8_t* __restrict__ active) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ncand; k += (int64_t)gridDim.x * blockDim.x) {
    if (!head[k]) continue;
    int64_t cur = k;
    active[cur] = 1;
    for (;;) {
      int64_t nx = cur + 1;
      while (nx < ncand && cand[nx] <= reach[cur]) active[nx++] = 0;
      if (nx >= ncand || head[nx]) break;
      cur = nx;
      active[cur] = 1;
    }
  }
}

// One warp per performed start with a partner: lut[g-1+t] = L + t for
// t = 0 .. u-(g-1).  Adjacent performed fills share at most their end
// position, where both write the same value.  gaps (findGaps) gets
// u-(g-1), or -1 for a performed start with no partner.
__global__ void k_fill_apply(int32_t* __restrict__ lut, const int32_t* __restrict__ cand,
                             const int32_t* __restrict__ reach, const int32_t* __restrict__ lval,
                             const uint8_t* __restrict__ active, int64_t ncand, int32_t* __restrict__ gaps) {
  const int lane = threadIdx.x & 31;
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ncand;
       k += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    if (!active[k]) continue;
    const int64_t gs = cand[k], u = reach[k], lower = gs - 1;
    if (u == gs) {
      if (gaps && lane == 0) gaps[gs] = -1;
      continue;
    }
    const int32_t L = lval[k];
    for (int64_t t = lane; t <= u - lower; t += 32) lut[lower + t] = (int32_t)((uint32_t)L + (uint32_t)t);
    if (gaps && lane == 0) gaps[gs] = (int32_t)(u - lower);
  }
}

__global__ void k_fill_lval(const int32_t* __restrict__ lut, const int32_t* __restrict__ cand, int64_t ncand,
                            int32_t* __restrict__ lval) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ncand; k += (int64_t)gridDim.x * blockDim.x)
    lval[k] = lut[cand[k] - 1];
}

// ------------------------------------------------------------ analysis

__global__ void k_find_edges(const int32_t* __restrict__ lut, int64_t n, uint8_t* __restrict__ edges) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    edges[i] = i == 0 ? 1 : ((uint32_t)lut[i] - (uint32_t)lut[i - 1] != 1u);
}

__global__ void k_find_mismatches(const int32_t* __restrict__ lut, int64_t n, const uint8_t* __restrict__ genome,
                                  int64_t glen, const uint8_t* __restrict__ ref, int64_t rlen,
                                  uint8_t* __restrict__ mism, uint32_t* err) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint8_t v = 0;
    if (i < glen) {
      const int32_t m = lut[i];
      if (m != -1) {
        if (m < 0 || m >= rlen)
          set_error(err, kDevRange);
        else
          v = genome[i] != ref[m];
      }
    }
    mism[i] = v;
  }
}

__global__ void k_lut_max(const int32_t* __restrict__ lut, int64_t n, int* __restrict__ mx) {
  int m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, lut[i]);
  for (int d = 16; d > 0; d >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

__global__ void k_lut_hist(const int32_t* __restrict__ lut, int64_t n, uint32_t* __restrict__ counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(counts + (lut[i] < 0 ? 0 : lut[i]), 1u);
}

__global__ void k_count_dups(const uint32_t* __restrict__ counts, int64_t nc, unsigned long long* __restrict__ dup) {
  unsigned long long d = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (int64_t)gridDim.x * blockDim.x)
    d += counts[i] > 1;
  for (int q = 16; q > 0; q >>= 1) d += __shfl_xor_sync(0xffffffffu, d, q);
  if ((threadIdx.x & 31) == 0 && d) atomicAdd(dup, d);
}

}  // namespace

// Workspace slots of this file.
enum : int {
  kWsSegN = 70, kWsSegStart, kWsSegBlock, kWsSegG, kWsSegR, kWsScan, kWsKeys, kWsFlags, kWsCand, kWsReach, kWsLval,
  kWsHead, kWsActive, kWsCounts, kWsMeta,
  // host-API staging
  kWsHLut, kWsHAux, kWsHGenome, kWsHRef, kWsHRowG, kWsHRowR, kWsHStarts, kWsHOff
};
static_assert(kWsHOff < Workspace::kSlots, "workspace slots");

static uint32_t* wsu32(Ctx* c, int slot, uint64_t n) { return (uint32_t*)c->ws.get(c, slot, n * 4 + 16); }

// Host reads of small device scalars through the pinned mirror.
static int read_u32(Ctx* c, const uint32_t* d, uint32_t* out) {
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, d, 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  *out = (uint32_t)(c->h_scalars[0] & 0xffffffffu);
  return 0;
}

int lut_from_blocks_dev(Ctx* c, const int64_t* d_gs, const int64_t* d_rs, const uint64_t* d_off,
                        const uint8_t* d_g, const uint8_t* d_r, uint64_t nblocks, uint64_t ncols, int32_t* d_lut,
                        int64_t n) {
  cudaStream_t st = c->stream;
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, st));
  unsigned long long* keys = (unsigned long long*)c->ws.get(c, kWsKeys, (size_t)n * 8 + 16);
  if (!keys) return report_error(MVG_ERR_NOMEM, "LUT key allocation failed");
  if (n > 0) MVG_CUDA_TRY(cudaMemsetAsync(keys, 0, (size_t)n * 8, st));
  if (nblocks > 0 && ncols > 0) {
    uint32_t* nseg = wsu32(c, kWsSegN, nblocks);
    uint32_t* sstart = wsu32(c, kWsSegStart, nblocks);
    uint32_t* scr = wsu32(c, kWsScan, scan_scratch_words((int64_t)nblocks) + 8);
    if (!nseg || !sstart || !scr) return report_error(MVG_ERR_NOMEM, "LUT segment allocation failed");
    k_seg_count<<<grid_for(nblocks, 256), 256, 0, st>>>(d_off, nblocks, nseg, c->d_err);
    uint32_t* d_tot = scr + scan_scratch_words((int64_t)nblocks) + 1;
    exclusive_scan(nseg, sstart, (int64_t)nblocks, scr, d_tot, st, &c->launches);
    c->launches++;
    uint32_t nsegs = 0;
    if (int rc = read_u32(c, d_tot, &nsegs)) return rc;
    if (int rc = check_device_error(c)) return rc;
    if (nsegs > 0) {
      uint32_t* sblock = wsu32(c, kWsSegBlock, nsegs);
      uint32_t* sg = wsu32(c, kWsSegG, nsegs);
      uint32_t* sr = wsu32(c, kWsSegR, nsegs);
      uint32_t* scr2 = wsu32(c, kWsFlags, scan_scratch_words(nsegs) + 8);
      if (!sblock || !sg || !sr || !scr2) return report_error(MVG_ERR_NOMEM, "LUT segment allocation failed");
      k_seg_fill<<<grid_for(nblocks, 256), 256, 0, st>>>(nseg, sstart, nblocks, sblock);
      k_lut_count<<<nsegs, kLutThreads, 0, st>>>(d_g, d_r, sblock, sstart, d_off, sg, sr);
      exclusive_scan(sg, sg, nsegs, scr2, nullptr, st, &c->launches);
      exclusive_scan(sr, sr, nsegs, scr2, nullptr, st, &c->launches);
      k_lut_walk<<<nsegs, kLutThreads, 0, st>>>(d_g, d_r, sblock, sstart, d_off, sg, sr, d_gs, d_rs, n, keys,
                                                c->d_err);
      c->launches += 3;
    }
  }
  if (n > 0) {
    k_lut_finish<<<grid_for((uint64_t)n, 256), 256, 0, st>>>(keys, n, d_lut);
    c->launches++;
  }
  MVG_CUDA_TRY(cudaGetLastError());
  return check_device_error(c);
}

int lut_fix_zero_dev(Ctx* c, int32_t* d_lut, int64_t n, const uint8_t* d_genome, uint64_t glen,
                     const uint8_t* d_ref, uint64_t rlen) {
  if (n <= 0) return report_error(MVG_ERR_RANGE, "fixZeroIdx: empty LUT");
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  k_fix_zero<<<1, 256, 0, c->stream>>>(d_lut, n, d_genome, glen, d_ref, rlen, c->d_err);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  return check_device_error(c);
}

int lut_fill_dev(Ctx* c, int32_t* d_lut, int64_t n, int width, int mode, int32_t* d_gaps) {
  cudaStream_t st = c->stream;
  if (d_gaps && n > 0) MVG_CUDA_TRY(cudaMemsetAsync(d_gaps, 0, (size_t)n * 4, st));
  if (n < 2 || width < 1) {  // the reference loops never find a partner
    MVG_CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
  }
  uint32_t* flags = wsu32(c, kWsFlags, (uint64_t)n);
  uint32_t* scr = wsu32(c, kWsScan, scan_scratch_words(n) + 8);
  if (!flags || !scr) return report_error(MVG_ERR_NOMEM, "LUT fill allocation failed");
  uint32_t* d_tot = scr + scan_scratch_words(n) + 1;
  k_fill_flags<<<grid_for((uint64_t)n, 256), 256, 0, st>>>(d_lut, n, mode, flags);
  exclusive_scan(flags, flags, n, scr, d_tot, st, &c->launches);
  c->launches++;
  uint32_t ncand = 0;
  if (int rc = read_u32(c, d_tot, &ncand)) return rc;  // synchronises the stream
  if (ncand == 0) return 0;
  int32_t* cand = (int32_t*)wsu32(c, kWsCand, ncand);
  int32_t* reach = (int32_t*)wsu32(c, kWsReach, ncand);
  int32_t* lval = (int32_t*)wsu32(c, kWsLval, ncand);
  uint8_t* head = (uint8_t*)c->ws.get(c, kWsHead, ncand + 16);
  uint8_t* active = (uint8_t*)c->ws.get(c, kWsActive, ncand + 16);
  if (!cand || !reach || !lval || !head || !active) return report_error(MVG_ERR_NOMEM, "LUT fill allocation failed");
  k_fill_compact<<<grid_for((uint64_t)n, 256), 256, 0, st>>>(d_lut, n, mode, flags, cand);
  k_fill_lval<<<grid_for(ncand, 256), 256, 0, st>>>(d_lut, cand, ncand, lval);
  k_fill_search<<<grid_for((uint64_t)ncand * 32, 256), 256, 0, st>>>(d_lut, n, width, cand, ncand, reach);
  k_fill_heads<<<grid_for(ncand, 256), 256, 0, st>>>(cand, reach, ncand, width, head);
  k_fill_resolve<<<grid_for(ncand, 256), 256, 0, st>>>(cand, reach, ncand, head, active);
  k_fill_apply<<<grid_for((uint64_t)ncand * 32, 256), 256, 0, st>>>(d_lut, cand, reach, lval, active, ncand, d_gaps);
  c->launches += 6;
  MVG_CUDA_TRY(cudaGetLastError());
  // like every entry point, return once the LUT is final (callers read it
  // on other streams)
  MVG_CUDA_TRY(cudaStreamSynchronize(st));
  return 0;
}

int lut_find_edges_dev(Ctx* c, const int32_t* d_lut, int64_t n, uint8_t* d_edges) {
  if (n <= 0) return 0;
  k_find_edges<<<grid_for((uint64_t)n, 256), 256, 0, c->stream>>>(d_lut, n, d_edges);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int lut_find_mismatches_dev(Ctx* c, const int32_t* d_lut, int64_t n, const uint8_t* d_genome, uint64_t glen,
                            const uint8_t* d_ref, uint64_t rlen, uint8_t* d_mism) {
  if (glen > (uint64_t)n) return report_error(MVG_ERR_RANGE, "findMismatches: genome longer than the LUT");
  if (n <= 0) return 0;
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  k_find_mismatches<<<grid_for((uint64_t)n, 256), 256, 0, c->stream>>>(d_lut, n, d_genome, (int64_t)glen, d_ref,
                                                                      (int64_t)rlen, d_mism, c->d_err);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  return check_device_error(c);
}

int lut_duplicate_mappings_dev(Ctx* c, const int32_t* d_lut, int64_t n, int64_t* result) {
  if (n <= 0) {
    *result = -1;
    return 0;
  }
  cudaStream_t st = c->stream;
  uint32_t* meta = wsu32(c, kWsMeta, 8);
  if (!meta) return report_error(MVG_ERR_NOMEM, "allocation failed");
  MVG_CUDA_TRY(cudaMemsetAsync(meta, 0, 32, st));
  k_lut_max<<<grid_for((uint64_t)n, 256), 256, 0, st>>>(d_lut, n, (int*)meta);
  c->launches++;
  uint32_t mx = 0;
  if (int rc = read_u32(c, meta, &mx)) return rc;
  const int64_t nc = (int64_t)mx + 1;
  uint32_t* counts = wsu32(c, kWsCounts, (uint64_t)nc);
  if (!counts) return report_error(MVG_ERR_NOMEM, "allocation failed");
  MVG_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)nc * 4, st));
  unsigned long long* dup = (unsigned long long*)(meta + 2);
  k_lut_hist<<<grid_for((uint64_t)n, 256), 256, 0, st>>>(d_lut, n, counts);
  k_count_dups<<<grid_for((uint64_t)nc, 256), 256, 0, st>>>(counts, nc, dup);
  c->launches += 2;
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, dup, 8, cudaMemcpyDeviceToHost, st));
  MVG_CUDA_TRY(cudaStreamSynchronize(st));
  *result = (int64_t)c->h_scalars[0] - 1;
  return 0;
}

}  // namespace mvg

// ------------------------------------------------------------------ C ABI

using namespace mvg;

namespace {

Ctx* ctx_of(mvg_handle h) { return reinterpret_cast<Ctx*>(h); }

// Host buffer -> workspace slot (async on the handle's stream).
template <typename T>
T* stage_in(Ctx* c, int slot, const T* host, uint64_t count) {
  T* d = (T*)c->ws.get(c, slot, count * sizeof(T) + 16);
  if (d && count) {
    if (cudaMemcpyAsync(d, host, count * sizeof(T), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) return nullptr;
  }
  return d;
}

int finish_out(Ctx* c, void* host, const void* dev, size_t bytes) {
  if (bytes) MVG_CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int check_lut_len(uint64_t n) {
  if (n > (uint64_t)INT32_MAX) return report_error(MVG_ERR_CAPACITY, "LUT longer than 2^31-1 entries");
  return 0;
}

int blocks_dev(Ctx* c, const int64_t* d_gs, const int64_t* d_rs, const uint64_t* d_off, const uint8_t* d_g,
               const uint8_t* d_r, uint64_t nblocks, uint64_t ncols, int32_t* d_lut, uint64_t n) {
  if (int rc = check_lut_len(n)) return rc;
  if (ncols >= 0xffffffffull) return report_error(MVG_ERR_CAPACITY, "more than 2^32-2 alignment columns");
  return lut_from_blocks_dev(c, d_gs, d_rs, d_off, d_g, d_r, nblocks, ncols, d_lut, (int64_t)n);
}

}  // namespace

extern "C" {

int mvg_lut_from_blocks_dev(mvg_handle h, const int64_t* d_genome_start, const int64_t* d_ref_start,
                            const uint64_t* d_col_off, const uint8_t* d_genome_rows, const uint8_t* d_ref_rows,
                            uint64_t nblocks, int32_t* d_lut, uint64_t n) {
  if (!h || (nblocks && (!d_genome_start || !d_ref_start || !d_col_off)) || (n && !d_lut))
    return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  uint64_t off[2] = {0, 0};
  if (nblocks) {
    MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, d_col_off, 8, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars + 1, d_col_off + nblocks, 8, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    off[0] = c->h_scalars[0];
    off[1] = c->h_scalars[1];
    if (off[1] < off[0]) return report_error(MVG_ERR_ARG, "column offsets decrease");
    if (off[1] && (!d_genome_rows || !d_ref_rows)) return report_error(MVG_ERR_ARG, "bad argument");
  }
  return blocks_dev(c, d_genome_start, d_ref_start, d_col_off, d_genome_rows, d_ref_rows, nblocks, off[1], d_lut, n);
}

int mvg_lut_from_blocks(mvg_handle h, const int64_t* genome_start, const int64_t* ref_start, const uint64_t* col_off,
                        const uint8_t* genome_rows, const uint8_t* ref_rows, uint64_t nblocks, int32_t* lut,
                        uint64_t n) {
  if (!h || (nblocks && (!genome_start || !ref_start || !col_off)) || (n && !lut))
    return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  uint64_t ncols = 0;
  if (nblocks) {
    for (uint64_t b = 0; b < nblocks; ++b)
      if (col_off[b + 1] < col_off[b]) return report_error(MVG_ERR_ARG, "column offsets decrease");
    ncols = col_off[nblocks];
    if (ncols && (!genome_rows || !ref_rows)) return report_error(MVG_ERR_ARG, "bad argument");
  }
  const int64_t* d_gs = stage_in(c, kWsHStarts, genome_start, nblocks);
  const int64_t* d_rs = stage_in(c, kWsHAux, ref_start, nblocks);
  const uint64_t* d_off = stage_in(c, kWsHOff, col_off, nblocks + 1);
  const uint8_t* d_g = stage_in(c, kWsHRowG, genome_rows, ncols);
  const uint8_t* d_r = stage_in(c, kWsHRowR, ref_rows, ncols);
  int32_t* d_lut = (int32_t*)c->ws.get(c, kWsHLut, n * 4 + 16);
  if (!d_gs || !d_rs || !d_off || !d_g || !d_r || !d_lut) return report_error(MVG_ERR_NOMEM, "staging failed");
  if (int rc = blocks_dev(c, d_gs, d_rs, d_off, d_g, d_r, nblocks, ncols, d_lut, n)) return rc;
  return finish_out(c, lut, d_lut, n * 4);
}

int mvg_lut_fix_zero_idx_dev(mvg_handle h, int32_t* d_lut, uint64_t n, const uint8_t* d_genome, uint64_t genome_len,
                             const uint8_t* d_ref, uint64_t ref_len) {
  if (!h || (n && !d_lut) || (genome_len && !d_genome) || (ref_len && !d_ref))
    return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  return lut_fix_zero_dev(c, d_lut, (int64_t)n, d_genome, genome_len, d_ref, ref_len);
}

int mvg_lut_fix_zero_idx(mvg_handle h, int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t genome_len,
                         const uint8_t* ref, uint64_t ref_len) {
  if (!h || (n && !lut) || (genome_len && !genome) || (ref_len && !ref)) return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  int32_t* d_lut = stage_in(c, kWsHLut, lut, n);
  const uint8_t* d_g = stage_in(c, kWsHGenome, genome, genome_len);
  const uint8_t* d_r = stage_in(c, kWsHRef, ref, ref_len);
  if (!d_lut || !d_g || !d_r) return report_error(MVG_ERR_NOMEM, "staging failed");
  if (int rc = lut_fix_zero_dev(c, d_lut, (int64_t)n, d_g, genome_len, d_r, ref_len)) return rc;
  return finish_out(c, lut, d_lut, 4);
}

static int fill_common(mvg_handle h, int32_t* lut, uint64_t n, int width, int mode, int32_t* gaps, bool host) {
  if (!h || (n && !lut)) return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  if (!host) return lut_fill_dev(c, lut, (int64_t)n, width, mode, gaps);
  int32_t* d_lut = stage_in(c, kWsHLut, lut, n);
  int32_t* d_gaps = gaps ? (int32_t*)c->ws.get(c, kWsHAux, n * 4 + 16) : nullptr;
  if (!d_lut || (gaps && !d_gaps)) return report_error(MVG_ERR_NOMEM, "staging failed");
  if (int rc = lut_fill_dev(c, d_lut, (int64_t)n, width, mode, d_gaps)) return rc;
  if (gaps && n) MVG_CUDA_TRY(cudaMemcpyAsync(gaps, d_gaps, n * 4, cudaMemcpyDeviceToHost, c->stream));
  return finish_out(c, lut, d_lut, n * 4);
}

int mvg_lut_fill_gaps(mvg_handle h, int32_t* lut, uint64_t n, int max_gap_width) {
  return fill_common(h, lut, n, max_gap_width, kFill, nullptr, true);
}
int mvg_lut_fill_gaps_dev(mvg_handle h, int32_t* d_lut, uint64_t n, int max_gap_width) {
  return fill_common(h, d_lut, n, max_gap_width, kFill, nullptr, false);
}
int mvg_lut_smooth_edges(mvg_handle h, int32_t* lut, uint64_t n, int smoothing_radius) {
  return fill_common(h, lut, n, smoothing_radius, kSmooth, nullptr, true);
}
int mvg_lut_smooth_edges_dev(mvg_handle h, int32_t* d_lut, uint64_t n, int smoothing_radius) {
  return fill_common(h, d_lut, n, smoothing_radius, kSmooth, nullptr, false);
}
int mvg_lut_find_gaps(mvg_handle h, int32_t* lut, uint64_t n, int32_t* gaps) {
  if (n && !gaps) return report_error(MVG_ERR_ARG, "bad argument");
  return fill_common(h, lut, n, 300, kFill, gaps, true);
}
int mvg_lut_find_gaps_dev(mvg_handle h, int32_t* d_lut, uint64_t n, int32_t* d_gaps) {
  if (n && !d_gaps) return report_error(MVG_ERR_ARG, "bad argument");
  return fill_common(h, d_lut, n, 300, kFill, d_gaps, false);
}

int mvg_lut_find_edges(mvg_handle h, const int32_t* lut, uint64_t n, uint8_t* edges) {
  if (!h || (n && (!lut || !edges))) return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  const int32_t* d_lut = stage_in(c, kWsHLut, lut, n);
  uint8_t* d_e = (uint8_t*)c->ws.get(c, kWsHAux, n + 16);
  if (!d_lut || !d_e) return report_error(MVG_ERR_NOMEM, "staging failed");
  if (int rc = lut_find_edges_dev(c, d_lut, (int64_t)n, d_e)) return rc;
  return finish_out(c, edges, d_e, n);
}

int mvg_lut_find_mismatches(mvg_handle h, const int32_t* lut, uint64_t n, const uint8_t* genome, uint64_t genome_len,
                            const uint8_t* ref, uint64_t ref_len, uint8_t* mismatches) {
  if (!h || (n && (!lut || !mismatches)) || (genome_len && !genome) || (ref_len && !ref))
    return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  const int32_t* d_lut = stage_in(c, kWsHLut, lut, n);
  const uint8_t* d_g = stage_in(c, kWsHGenome, genome, genome_len);
  const uint8_t* d_r = stage_in(c, kWsHRef, ref, ref_len);
  uint8_t* d_m = (uint8_t*)c->ws.get(c, kWsHAux, n + 16);
  if (!d_lut || !d_g || !d_r || !d_m) return report_error(MVG_ERR_NOMEM, "staging failed");
  if (int rc = lut_find_mismatches_dev(c, d_lut, (int64_t)n, d_g, genome_len, d_r, ref_len, d_m)) return rc;
  return finish_out(c, mismatches, d_m, n);
}

int mvg_lut_find_duplicate_mappings(mvg_handle h, const int32_t* lut, uint64_t n, int64_t* result) {
  if (!h || !result || (n && !lut)) return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  const int32_t* d_lut = stage_in(c, kWsHLut, lut, n);
  if (!d_lut) return report_error(MVG_ERR_NOMEM, "staging failed");
  return lut_duplicate_mappings_dev(c, d_lut, (int64_t)n, result);
}

int mvg_build_index_lut_dev(mvg_handle h, const int64_t* d_genome_start, const int64_t* d_ref_start,
                            const uint64_t* d_col_off, const uint8_t* d_genome_rows, const uint8_t* d_ref_rows,
                            uint64_t nblocks, const uint8_t* d_genome, uint64_t genome_len, const uint8_t* d_ref,
                            uint64_t ref_len, int fill_gaps, int max_gap_width, int smooth_edges,
                            int smoothing_radius, int32_t* d_lut, uint64_t n) {
  if (fill_gaps && ((genome_len && !d_genome) || (ref_len && !d_ref))) return report_error(MVG_ERR_ARG, "bad argument");
  if (int rc = mvg_lut_from_blocks_dev(h, d_genome_start, d_ref_start, d_col_off, d_genome_rows, d_ref_rows, nblocks,
                                       d_lut, n))
    return rc;
  Ctx* c = ctx_of(h);
  if (fill_gaps) {
    if (int rc = lut_fix_zero_dev(c, d_lut, (int64_t)n, d_genome, genome_len, d_ref, ref_len)) return rc;
    if (int rc = lut_fill_dev(c, d_lut, (int64_t)n, max_gap_width, kFill, nullptr)) return rc;
  }
  if (smooth_edges)
    if (int rc = lut_fill_dev(c, d_lut, (int64_t)n, smoothing_radius, kSmooth, nullptr)) return rc;
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int mvg_build_index_lut(mvg_handle h, const int64_t* genome_start, const int64_t* ref_start, const uint64_t* col_off,
                        const uint8_t* genome_rows, const uint8_t* ref_rows, uint64_t nblocks, const uint8_t* genome,
                        uint64_t genome_len, const uint8_t* ref, uint64_t ref_len, int fill_gaps, int max_gap_width,
                        int smooth_edges, int smoothing_radius, int32_t* lut, uint64_t n) {
  if (!h || (nblocks && (!genome_start || !ref_start || !col_off)) || (n && !lut))
    return report_error(MVG_ERR_ARG, "bad argument");
  if (fill_gaps && ((genome_len && !genome) || (ref_len && !ref))) return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = ctx_of(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  if (int rc = check_lut_len(n)) return rc;
  uint64_t ncols = 0;
  if (nblocks) {
    for (uint64_t b = 0; b < nblocks; ++b)
      if (col_off[b + 1] < col_off[b]) return report_error(MVG_ERR_ARG, "column offsets decrease");
    ncols = col_off[nblocks];
    if (ncols && (!genome_rows || !ref_rows)) return report_error(MVG_ERR_ARG, "bad argument");
  }
  const int64_t* d_gs = stage_in(c, kWsHStarts, genome_start, nblocks);
  const int64_t* d_rs = stage_in(c, kWsHAux, ref_start, nblocks);
  const uint64_t* d_off = stage_in(c, kWsHOff, col_off, nblocks + 1);
  const uint8_t* d_gr = stage_in(c, kWsHRowG, genome_rows, ncols);
  const uint8_t* d_rr = stage_in(c, kWsHRowR, ref_rows, ncols);
  const uint8_t* d_g = fill_gaps ? stage_in(c, kWsHGenome, genome, genome_len) : nullptr;
  const uint8_t* d_r = fill_gaps ? stage_in(c, kWsHRef, ref, ref_len) : nullptr;
  int32_t* d_lut = (int32_t*)c->ws.get(c, kWsHLut, n * 4 + 16);
  if (!d_gs || !d_rs || !d_off || !d_gr || !d_rr || !d_lut || (fill_gaps && (!d_g || !d_r)))
    return report_error(MVG_ERR_NOMEM, "staging failed");
  if (int rc = blocks_dev(c, d_gs, d_rs, d_off, d_gr, d_rr, nblocks, ncols, d_lut, n)) return rc;
  if (fill_gaps) {
    if (int rc = lut_fix_zero_dev(c, d_lut, (int64_t)n, d_g, genome_len, d_r, ref_len)) return rc;
    if (int rc = lut_fill_dev(c, d_lut, (int64_t)n, max_gap_width, kFill, nullptr)) return rc;
  }
  if (smooth_edges)
    if (int rc = lut_fill_dev(c, d_lut, (int64_t)n, smoothing_radius, kSmooth, nullptr)) return rc;
  return finish_out(c, lut, d_lut, n * 4);
}

}  // extern "C"
