// Traceback of checkpointed full-DP passes (included by gapdp.cu after
// gapdp_kernel.cuh).
//
// One warp per problem, problems claimed from a counter in slot order
// (largest first).  The path is walked from (LA, LB) towards (0, 0) as in
// k_traceback (MU/bittraceback.cpp:138-210), but the traceback bits are not
// stored: for the block of the matrix the walk is in (strip k of 32*R rows,
// column block b of kCkCols columns) the warp recomputes them from the
// forward pass's checkpoints, with the same wavefront and the same
// recurrence code (dp_column), so every bit equals the one a stored-bits
// pass would have written:
//   top row      the previous strip's bottom-row checkpoint (row 0's fixed
//                values for strip 0),
//   left column  the column checkpoint left of the block (the matrix's
//                column-0 state for block 0).
// Only columns up to the walk's current one are recomputed: the cells right
// of it cannot be on the path.  The bits go to shared memory (one word per
// column and lane), and the walk continues inside the block until it leaves
// it upwards or to the left.  Steps along row 0 or column 0 need no bits.
#pragma once

namespace mvg {

constexpr int kCkWarps = 4;
constexpr size_t kCkSmem = (size_t)kCkWarps * kCkCols * 32 * sizeof(uint32_t);  // 64 KB

template <int R>
__global__ void __launch_bounds__(kCkWarps * 32) k_tb_ck(const uint8_t* __restrict__ sa,
                                                          const uint64_t* __restrict__ oa,
                                                          const uint8_t* __restrict__ sb,
                                                          const uint64_t* __restrict__ ob,
                                                          const uint32_t* __restrict__ order,
                                                          const uint64_t* __restrict__ ck_off, int nwork,
                                                          const uint32_t* __restrict__ arena,
                                                          const uint8_t* __restrict__ end_edge,
                                                          const uint64_t* __restrict__ path_off, char* __restrict__ paths,
                                                          int64_t* __restrict__ path_len, uint32_t* err,
                                                          int32_t* __restrict__ env, unsigned* counter) {
  constexpr int SR = 32 * R;
  extern __shared__ __align__(16) uint32_t ck_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* nib = ck_smem + (size_t)wib * kCkCols * 32;  // [column in block][lane]
  for (;;) {
    int q = 0;
    if (lane == 0) q = (int)atomicAdd(counter, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nwork) break;
    const uint32_t p = order[q];
    const int LA = (int)(oa[p + 1] - oa[p]), LB = (int)(ob[p + 1] - ob[p]);
    const uint8_t* A = sa + oa[p];
    const uint8_t* B = sb + ob[p];
    const int4* ck = reinterpret_cast<const int4*>(arena + ck_off[q] / 4);
    char* out = paths + path_off[p] + (LA + LB);  // writes go backwards from here
    int pa = LA, pb = LB;
    char cur = (char)end_edge[p];
    int64_t n = 0;
    const int64_t limit = (int64_t)LA + LB;
    int32_t dev_lo = INT32_MAX, dev_hi = INT32_MIN;
    bool done = false, fail = false;
    // one step of the walk with the bits of the current cell (0 off the matrix)
    auto walk_step = [&](uint32_t bits) {
      if (n >= limit) {
        fail = true;
        return;
      }
      if (lane == 0) *(out - 1) = cur;
      --out;
      ++n;
      if (env && pa >= 1) {
        const int32_t dv = pb - (int32_t)((int64_t)pa * LB / LA);
        dev_lo = min(dev_lo, dv);
        dev_hi = max(dev_hi, dv);
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
      if (pa == 0 && pb == 0) {
        done = true;
        return;
      }
      if (pa < 0 || pb < 0) {
        fail = true;
        return;
      }
      cur = next;
    };
    while (!done && !fail) {
      if (pa < 1 || pb < 1) {  // along row 0 or column 0
        walk_step(0u);
        continue;
      }
      const int k = (pa - 1) / SR, b = (pb - 1) / kCkCols;
      const int row0 = k * SR, c0 = b * kCkCols + 1;
      const int Wb = pb - c0 + 1;  // columns c0 .. pb
      // ---- recompute the block's bits
      DpLane<R> L;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = row0 + lane * R + r + 1;
        L.arow[r] = c_score_rows[(i <= LA ? A[i - 1] : 0u) & 3u];
      }
      if (b == 0) {  // column 0: (M, D, I) = (-inf, 0, -inf), M carried as Mg
#pragma unroll
        for (int r = 0; r < R; ++r) {
          L.lM[r] = kNeg + kGap;
          L.lD[r] = 0;
          L.lI[r] = kNeg;
        }
      } else {
        const int4* col = ck + ck_col_entry(LA, LB, R, k, b) + lane * R;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int4 v = col[r];
          L.lM[r] = v.x;
          L.lD[r] = v.y;
          L.lI[r] = v.z;
        }
      }
      // the row above the strip at column x (the forward pass's above())
      auto above = [&](int x) -> int4 {
        if (k == 0) return x == 0 ? make_int4(kGap, kNeg, kNeg, 0) : make_int4(kNeg, kNeg, 0, 0);
        if (x >= 1) return ck[(int64_t)(k - 1) * LB + x - 1];
        return make_int4(kNeg + kGap, 0, kNeg, 0);
      };
      const int4 dg0 = above(c0 - 1);
      int32_t pubM = L.lM[R - 1], pubD = L.lD[R - 1], pubI = L.lI[R - 1];
      int32_t upM = kNeg, upD = kNeg, upI = kNeg;
      for (int s = 0; s < Wb + 31; ++s) {
        const int jj = s - lane;
        const int j = c0 + jj;
        const int32_t rM = __shfl_up_sync(0xffffffffu, pubM, 1);
        const int32_t rD = __shfl_up_sync(0xffffffffu, pubD, 1);
        const int32_t rI = __shfl_up_sync(0xffffffffu, pubI, 1);
        int4 v = make_int4(0, 0, 0, 0);
        if (lane == 0 && s < Wb) v = above(c0 + s);
        int32_t dgM = upM, dgD = upD, dgI = upI;
        if (s == 0 && lane == 0) {
          dgM = dg0.x;
          dgD = dg0.y;
          dgI = dg0.z;
        }
        upM = lane == 0 ? v.x : rM;
        upD = lane == 0 ? v.y : rD;
        upI = lane == 0 ? v.z : rI;
        if (jj >= 0 && jj < Wb) {
          const uint32_t bsel = (uint32_t)B[j - 1] | 0x4440u;
          uint32_t nibs = dp_column<R, true>(L, upM, upD, dgM, dgD, dgI, bsel, j == 1 ? -kGap : 0);
          if (s == 0 && lane == 0 && k == 0 && LA == 1 && c0 == 1) {
            // NWSmall's last-row special case with LA == 1 (as in dp_solve)
            L.lM[0] = (int32_t)__byte_perm(L.arow[0], 0u, bsel) - kScoreBias + 2 * kGap;
            nibs = (nibs & ~3u) | TB_DM;
          }
          pubM = L.lM[R - 1];
          pubD = L.lD[R - 1];
          pubI = L.lI[R - 1];
          nib[jj * 32 + lane] = nibs;
        }
      }
      __syncwarp();
      // ---- walk inside the block (every lane walks; lane 0 writes)
      while (!done && !fail && pa > row0 && pb >= c0) {
        const int rem = pa - 1 - row0;
        const uint32_t word = nib[(pb - c0) * 32 + rem / R];
        walk_step((word >> (4 * (rem % R))) & 15u);
      }
      __syncwarp();  // the next block's recompute overwrites the bits
    }
    if (fail && lane == 0) set_error(err, kDevCapacity);
    if (lane == 0) {
      path_len[p] = n;
      if (env) {
        env[2 * p] = dev_lo;
        env[2 * p + 1] = dev_hi;
      }
    }
  }
}

}  // namespace mvg
