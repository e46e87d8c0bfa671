// Windowed traceback for long paths (included by gapdp.cu).
//
// BitTraceBack (MU/bittraceback.cpp:138-210) is a serial walk from (LA, LB)
// to (0, 0); walked one thread per problem, every step is a dependent global
// load, and the longest path of a batch sets the traceback's time.  Both
// traceback layouts (strips, gapdp_kernel.cuh; ring, gapdp_ring.cuh) store
// 128-byte rows of 32 lane words, and the walk visits rows in non-increasing
// order.  So one warp walks one long path: all lanes run the same walk, the
// rows come through shared memory in windows of kTbRows rows, the window
// below the current one is prefetched with cp.async while the walk runs, and
// lane 0 writes the path.  Short paths keep the thread-per-problem walker.
#pragma once
#include "band.h"

namespace mvg {

constexpr int kTbRows = 64;                 // rows per window (8 KB)
constexpr int kTbWarps = 4;                 // warps per block
constexpr int kTbLongPath = 1024;           // LA + LB at which a path gets a warp
constexpr size_t kTbSmem = (size_t)kTbWarps * 2 * kTbRows * 32 * 4;  // two windows per warp

// Strip layout: strip k (32*rows rows) starts at word base_k; cell (i, j)
// with i-1 = k*srows + t*rows + r is nibble (j - lo_k + t)*rows + r of lane t.
struct StripMap {
  Band band;
  int rows, srows, cur_k, cur_lo;
  int64_t base;
  __device__ void init(int LA, int LB, const int32_t* delta, const int32_t* half, uint32_t p, int rows_) {
    rows = rows_;
    srows = 32 * rows;
    band = delta ? make_band(LA, LB, delta[p], half[p], srows) : make_full(LA, LB, srows);
    cur_k = (LA - 1) / srows;
    base = 0;
    for (int k = 0; k < cur_k; ++k)
      base += (int64_t)band_words_per_lane(band_hi(band, k) - band_lo(band, k) + 1, rows) * 32;
    cur_lo = band_lo(band, cur_k);
  }
  __device__ bool map(int pa, int pb, int64_t& X, int& t, int& sh) {
    const int i0 = pa - 1;
    const int lr = __ffs(rows) - 1;  // rows is 1, 2, 4 or 8
    const int k = i0 >> (lr + 5), rem = i0 & (srows - 1);
    while (cur_k > k) {
      --cur_k;
      base -= (int64_t)band_words_per_lane(band_hi(band, cur_k) - band_lo(band, cur_k) + 1, rows) * 32;
      cur_lo = band_lo(band, cur_k);
    }
    t = rem >> lr;
    const int r = rem & (rows - 1);
    const int s = pb - cur_lo + t;
    if (s < t) return false;
    const int64_t nib = (int64_t)s * rows + r;
    X = base / 32 + (nib >> 3);
    sh = 4 * (int)(nib & 7);
    return true;
  }
};

// Ring layout: group g = (i-1)/R computes column j at step j + g - lo_0;
// row r of the group is nibble r of that step in lane g mod 32 (ring_tb_at).
struct RingMap {
  RingBand b;
  int gc, loc;
  __device__ void init(int LA, int LB, const int32_t* delta, const int32_t* half, uint32_t p, int R) {
    b = make_ring_band(LA, LB, delta[p], half[p], R);
    gc = -1;
    loc = 0;
  }
  __device__ bool map(int pa, int pb, int64_t& X, int& t, int& sh) {
    const int g = (pa - 1) / b.R, r = (pa - 1) - g * b.R;
    if (g != gc) {
      gc = g;
      loc = ring_lo(b, g);
    }
    if (pb < loc || pb > loc + b.W - 1) return false;
    ring_tb_at(b.R, (int64_t)(pb + g - b.lo0), r, X, sh);
    t = g & 31;
    return true;
  }
};

__device__ __forceinline__ void tb_copy_rows(uint32_t* dst, const uint32_t* T, int64_t row0, int nrows) {
  // nrows rows of 128 bytes as 16-byte cp.async chunks, spread over the lanes
  const int lane = threadIdx.x & 31;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(dst);
  for (int c = lane; c < nrows * 8; c += 32) {
    const uint32_t* g = T + (row0 + (c >> 3)) * 32 + (c & 7) * 4;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sbase + (uint32_t)c * 16u), "l"(g) : "memory");
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void tb_wait_copies() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncwarp();
}

// One warp walks problem slot w; Map gives (row, lane, shift) per cell.
template <class Map>
__device__ void tb_walk_warp(Map& map, const uint32_t* T, uint32_t* win0, uint32_t* win1, int LA, int LB, char cur,
                             char* out_end, int64_t* len_out, uint32_t* err, int32_t* env_out) {
  const int lane = threadIdx.x & 31;
  uint32_t* bc = win0;  // window the walk reads
  uint32_t* bo = win1;  // the other window (prefetch target)
  int64_t lc = INT64_MAX, lo_o = INT64_MAX;  // first row each holds (none yet)
  bool pending = false;
  char* out = out_end;
  int pa = LA, pb = LB;
  int64_t n = 0;
  const int64_t limit = (int64_t)LA + LB;
  int32_t dev_lo = INT32_MAX, dev_hi = INT32_MIN;
  for (;;) {
    if (n >= limit) {
      if (lane == 0) set_error(err, kDevCapacity);
      break;
    }
    --out;
    if (lane == 0) *out = cur;
    ++n;
    if (env_out && pa >= 1) {
      const int32_t dv = pb - (int32_t)((int64_t)pa * LB / LA);
      dev_lo = min(dev_lo, dv);
      dev_hi = max(dev_hi, dv);
    }
    uint32_t bits = 0;
    if (pa >= 1 && pb >= 1) {
      int64_t X;
      int t, sh;
      if (!map.map(pa, pb, X, t, sh)) {
        if (lane == 0) set_error(err, kDevCapacity);
        break;
      }
      if (X < lc) {
        if (pending) tb_wait_copies();
        pending = false;
        if (X < lo_o) {  // a jump below the prefetched window: load the window ending at X
          const int64_t r0 = X - (kTbRows - 1) > 0 ? X - (kTbRows - 1) : 0;
          __syncwarp();
          tb_copy_rows(bo, T, r0, (int)(X - r0 + 1));
          tb_wait_copies();
          lo_o = r0;
        }
        uint32_t* tp = bc;
        bc = bo;
        bo = tp;
        lc = lo_o;
        // prefetch the window below into the other buffer
        if (lc > 0) {
          const int64_t r1 = lc - kTbRows > 0 ? lc - kTbRows : 0;
          __syncwarp();
          tb_copy_rows(bo, T, r1, (int)(lc - r1));
          lo_o = r1;
          pending = true;
        } else {
          lo_o = INT64_MAX;
        }
      }
      bits = (bc[(X - lc) * 32 + t] >> sh) & 15u;
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
      if (lane == 0) set_error(err, kDevCapacity);
      break;
    }
    cur = next;
  }
  if (pending) tb_wait_copies();
  if (lane == 0) {
    *len_out = n;
    if (env_out) {
      env_out[0] = dev_lo;
      env_out[1] = dev_hi;
    }
  }
}

// The long paths of a wave, one warp each: slots[0..nslots) index the
// wave's arrays and are claimed through a counter, largest first.
// rows_of == nullptr: strip layout with `rows` rows per lane, else the ring
// layout with rows_of[w] rows per group.
__global__ void __launch_bounds__(kTbWarps * 32) k_traceback_win(
    const uint64_t* __restrict__ oa, const uint64_t* __restrict__ ob, const uint32_t* __restrict__ order,
    const uint64_t* __restrict__ tb_off, const uint32_t* __restrict__ slots, int nslots,
    const uint32_t* __restrict__ tb, const uint8_t* __restrict__ end_edge, const int32_t* __restrict__ band_delta,
    const int32_t* __restrict__ band_half, const uint8_t* __restrict__ accept, const uint64_t* __restrict__ path_off,
    char* __restrict__ paths, int64_t* __restrict__ path_len, uint32_t* err, int rows,
    const uint8_t* __restrict__ rows_of, int32_t* __restrict__ env, unsigned* counter) {
  extern __shared__ __align__(16) uint32_t tb_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* win0 = tb_smem + (size_t)wib * 2 * kTbRows * 32;
  uint32_t* win1 = win0 + kTbRows * 32;
  for (;;) {
    int q = 0;
    if (lane == 0) q = (int)atomicAdd(counter, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nslots) break;
    const int w = (int)slots[q];
    const uint32_t p = order[w];
    if (accept && !accept[p]) continue;
    const int LA = (int)(oa[p + 1] - oa[p]), LB = (int)(ob[p + 1] - ob[p]);
    const uint32_t* T = tb + tb_off[w] / 4;
    char* out_end = paths + path_off[p] + (LA + LB);
    int32_t* e = env ? env + 2 * p : nullptr;
    if (rows_of) {
      RingMap m;
      m.init(LA, LB, band_delta, band_half, p, rows_of[w]);
      tb_walk_warp(m, T, win0, win1, LA, LB, (char)end_edge[p], out_end, path_len + p, err, e);
    } else {
      StripMap m;
      m.init(LA, LB, band_delta, band_half, p, rows);
      tb_walk_warp(m, T, win0, win1, LA, LB, (char)end_edge[p], out_end, path_len + p, err, e);
    }
  }
}

}  // namespace mvg
