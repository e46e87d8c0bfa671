// Exclusive scan over uint32 (three passes: tile sums, scan of sums, tiles).
#include "prim.cuh"

namespace mvg {

__global__ void k_scan_reduce(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ bsum) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
  for (int k = 0; k < kScanTile / 256; ++k) {
    int64_t i = base + k * 256 + threadIdx.x;
    if (i < n) s += in[i];
  }
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  __shared__ uint32_t ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; ++w) t += ws[w];
    bsum[blockIdx.x] = t;
  }
}

__global__ void k_scan_bsums(uint32_t* __restrict__ bsum, int64_t nb, uint32_t* __restrict__ total) {
  __shared__ uint32_t ctot;
  uint32_t carry = 0;
  for (int64_t c = 0; c < nb; c += 256 * 8) {  // 8 consecutive sums per thread
    const int64_t i0 = c + (int64_t)threadIdx.x * 8;
    uint32_t v[8], sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      v[k] = i0 + k < nb ? bsum[i0 + k] : 0u;
      sum += v[k];
    }
    uint32_t run = carry + block_excl_scan256(sum, &ctot);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (i0 + k < nb) bsum[i0 + k] = run;
      run += v[k];
    }
    carry += ctot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_down(const uint32_t* in, int64_t n, const uint32_t* __restrict__ bsum, uint32_t* out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  __shared__ uint32_t carry;
  __shared__ uint32_t ctot;
  if (threadIdx.x == 0) carry = bsum[blockIdx.x];
  __syncthreads();
  for (int k = 0; k < kScanTile / 256; ++k) {
    int64_t i = base + k * 256 + threadIdx.x;
    uint32_t v = i < n ? in[i] : 0;
    uint32_t ex = block_excl_scan256(v, &ctot);
    if (i < n) out[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += ctot;
    __syncthreads();
  }
}

void exclusive_scan(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* scratch, uint32_t* d_total,
                    cudaStream_t st, uint64_t* launches) {
  if (n <= 0) {
    if (d_total) cudaMemsetAsync(d_total, 0, sizeof(uint32_t), st);
    return;
  }
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  k_scan_reduce<<<(unsigned)nb, 256, 0, st>>>(in, n, scratch);
  k_scan_bsums<<<1, 256, 0, st>>>(scratch, nb, d_total);
  k_scan_down<<<(unsigned)nb, 256, 0, st>>>(in, n, scratch, out);
  if (launches) *launches += 3;
}

// Block c of nchunks, 1024 threads: thread (q, d) takes digit d over every
// fourth chunk sum (from q) and over quarter q of chunk c's tiles.
//   offset(t, d) = start(d) + sum of d's counts in chunks before c
//                + sum of d's counts in tiles of chunk c before t
// where start(d) is the number of keys with a smaller digit.
__global__ void __launch_bounds__(1024) k_rts_offsets(uint32_t* __restrict__ counts, int64_t ntiles,
                                                      const uint32_t* __restrict__ csum, int64_t ctiles,
                                                      int64_t nchunks) {
  const int d = threadIdx.x & 255, q = threadIdx.x >> 8;
  const int64_t c = blockIdx.x;
  __shared__ uint32_t s_before[4][256], s_tot[4][256], s_part[4][256];
  __shared__ uint32_t wtot[8];
  uint32_t tot = 0, before = 0;
#pragma unroll 8
  for (int64_t cc = q; cc < nchunks; cc += 4) {
    const uint32_t v = csum[cc * 256 + d];
    tot += v;
    before += cc < c ? v : 0u;
  }
  const int64_t per = (ctiles + 3) / 4;
  const int64_t t0 = c * ctiles + q * per;
  const int64_t t1 = min(ntiles, min(c * ctiles + ctiles, t0 + per));
  uint32_t part = 0;
#pragma unroll 8
  for (int64_t t = t0; t < t1; ++t) part += counts[t * 256 + d];
  s_before[q][d] = before;
  s_tot[q][d] = tot;
  s_part[q][d] = part;
  __syncthreads();
  uint32_t T = 0, inc = 0;
  if (q == 0) {
    T = s_tot[0][d] + s_tot[1][d] + s_tot[2][d] + s_tot[3][d];
    inc = warp_incl_scan(T);
    if ((d & 31) == 31) wtot[d >> 5] = inc;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const uint32_t x = threadIdx.x < 8 ? wtot[threadIdx.x] : 0u;
    const uint32_t y = warp_incl_scan(x);
    if (threadIdx.x < 8) wtot[threadIdx.x] = y - x;
  }
  __syncthreads();
  if (q == 0) s_tot[0][d] = wtot[d >> 5] + inc - T;  // start(d)
  __syncthreads();
  uint32_t run = s_tot[0][d] + s_before[0][d] + s_before[1][d] + s_before[2][d] + s_before[3][d];
  for (int k = 0; k < q; ++k) run += s_part[k][d];
#pragma unroll 8
  for (int64_t t = t0; t < t1; ++t) {
    const uint32_t x = counts[t * 256 + d];
    counts[t * 256 + d] = run;
    run += x;
  }
}

}  // namespace mvg
