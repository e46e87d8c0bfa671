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
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t c = 0; c < nb; c += 256) {
    int64_t i = c + threadIdx.x;
    uint32_t v = i < nb ? bsum[i] : 0;
    uint32_t tot;
    __shared__ uint32_t ctot;
    uint32_t ex = block_excl_scan256(v, &ctot);
    (void)tot;
    if (i < nb) bsum[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += ctot;
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

__global__ void __launch_bounds__(256) k_os_scan(uint32_t* __restrict__ ghist) {
  uint32_t* g = ghist + blockIdx.x * 256;
  const uint32_t v = g[threadIdx.x];
  const uint32_t ex = block_excl_scan256(v, nullptr);
  g[threadIdx.x] = ex;
}

// Block d: offsets[d][t] = gstart[d] + counts[d][0] + ... + counts[d][t-1].
__global__ void __launch_bounds__(256) k_rts_rowscan(uint32_t* __restrict__ counts, int64_t ntiles,
                                                     const uint32_t* __restrict__ gstart) {
  uint32_t* row = counts + (int64_t)blockIdx.x * ntiles;
  __shared__ uint32_t tot;
  uint32_t carry = gstart[blockIdx.x];
  for (int64_t c = 0; c < ntiles; c += 256 * 8) {
    const int64_t i0 = c + (int64_t)threadIdx.x * 8;
    uint32_t v[8];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      v[k] = i0 + k < ntiles ? row[i0 + k] : 0u;
      sum += v[k];
    }
    uint32_t run = carry + block_excl_scan256(sum, &tot);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (i0 + k < ntiles) row[i0 + k] = run;
      run += v[k];
    }
    carry += tot;
    __syncthreads();
  }
}

}  // namespace mvg
