// Shared definitions for the GB300 (sm_103a) pairwise anchoring and gap-
// alignment kernels.  Everything here is device-side plumbing: error codes,
// the spaced-seed description, 2-bit window extraction and a few warp/grid
// helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mauve_gb300.h"

namespace mvg {

constexpr int kWarp = 32;

// Status words written by kernels (device-side error flag, first error wins).
enum DevError : uint32_t {
  kDevOk = 0,
  kDevGapChar = 1,      // '-' in a genome sequence (translate32 throws on it)
  kDevBadBase = 2,      // DP input code outside 0..3
  kDevCapacity = 3,     // an internal capacity bound was exceeded
  kDevWatchdog = 4,     // a bounded wait gave up
  kDevRange = 5,        // LUT: an index outside the LUT or a sequence
  kDevOverflow = 6,     // LUT: a value outside int32
};

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t code) {
  if (err) atomicCAS(err, 0u, code);
}

// A spaced seed: pattern bits (bit L-1 = leftmost base), length L, weight w,
// and the pattern decomposed into runs of consecutive 1 bits so a seed mer is
// gathered with one shift/mask per run instead of one per base.
struct SeedDesc {
  uint64_t pattern;
  uint64_t seed_mask;  // top 2w bits
  int L, w;
  int nruns;
  // the pattern reads the same reversed (every rank-0 seed of weight >= 5
  // and the coding seed): the reverse complement of a mer is then the mer
  // of the reverse-complement window
  int sym;
  // run r covers bases [run_start[r], run_start[r] + run_len[r]) of the window
  // and lands at output bit offset run_out[r] (from the MSB of the 2w-bit mer).
  int8_t run_start[32], run_len[32], run_out[32];
};

SeedDesc make_seed_desc(uint64_t pattern);

// 64-bit big-endian window of 32 bases starting at base pos, from 2-bit
// MSB-first packed words (with at least two readable words after pos/16).
__device__ __forceinline__ uint64_t window64(const uint32_t* __restrict__ g, uint64_t pos) {
  uint64_t w = pos >> 4;
  uint32_t bit = (uint32_t)(pos & 15) * 2;
  uint64_t m = ((uint64_t)__ldg(g + w) << 32) | __ldg(g + w + 1);
  if (bit) m = (m << bit) | (__ldg(g + w + 2) >> (32 - bit));
  return m;
}

// Pattern-selected bases of a 32-base window, left-aligned in 64 bits.
__device__ __forceinline__ uint64_t gather_seed(uint64_t win, const SeedDesc& s) {
  uint64_t out = 0;
#pragma unroll 4
  for (int r = 0; r < s.nruns; ++r) {
    int len2 = 2 * s.run_len[r];
    uint64_t part = (win << (2 * s.run_start[r])) >> (64 - len2);
    out |= part << (64 - 2 * s.run_out[r] - len2);
  }
  return out;
}

// Reverse complement of a left-aligned 2w-bit mer, left-aligned, with the low
// bit set as the strand marker.
__device__ __forceinline__ uint64_t revcomp_mer(uint64_t mer, int w) {
  uint64_t r = __brevll(~mer);  // groups reversed, bits inside groups swapped
  r = ((r >> 1) & 0x5555555555555555ull) | ((r & 0x5555555555555555ull) << 1);
  return (r << (64 - 2 * w)) | 1ull;
}

__device__ __forceinline__ uint64_t canonical_mer(const uint32_t* __restrict__ g, uint64_t pos, const SeedDesc& s) {
  uint64_t f = gather_seed(window64(g, pos), s);
  uint64_t r = revcomp_mer(f, s.w);
  return f < r ? f : r;
}

// The seed gather as a table: window byte c (bases 4c .. 4c+3) maps to its
// selected bases already at their place in the left-aligned mer, so a mer is
// the OR of one lookup per window byte.  Built by the whole block in shared
// memory (8 x 256 entries); seed_bytes(s) = ceil(L / 4) bytes are used.
__device__ __forceinline__ int seed_bytes(const SeedDesc& s) { return (s.L + 3) >> 2; }

__device__ __forceinline__ void seed_lut_build(const SeedDesc& s, uint64_t (*lut)[256]) {
  const int nb = seed_bytes(s);
  for (int e = threadIdx.x; e < nb * 256; e += blockDim.x) {
    const int c = e >> 8, b = e & 255;
    uint64_t v = 0;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const int k = 4 * c + kk;  // window base
      if (k < s.L && ((s.pattern >> (s.L - 1 - k)) & 1ull)) {
        const int o = k == 0 ? 0 : __popcll(s.pattern >> (s.L - k));  // selected bases before k
        v |= (uint64_t)((b >> (6 - 2 * kk)) & 3) << (62 - 2 * o);
      }
    }
    lut[c][b] = v;
  }
}

__device__ __forceinline__ uint64_t canonical_mer_lut(const uint32_t* __restrict__ g, uint64_t pos,
                                                      const uint64_t (*lut)[256], int nb, int w) {
  const uint64_t win = window64(g, pos);
  uint64_t f = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c)
    if (c < nb) f |= lut[c][(uint32_t)(win >> (56 - 8 * c)) & 255u];
  const uint64_t r = revcomp_mer(f, w);
  return f < r ? f : r;
}

// The same table for seeds of weight w <= 15: the mer left-aligned in 32
// bits (the top 2w bits), so a lookup is one 4-byte word.
__device__ __forceinline__ void seed_lut_build32(const SeedDesc& s, uint32_t (*lut)[256]) {
  const int nb = seed_bytes(s);
  for (int e = threadIdx.x; e < nb * 256; e += blockDim.x) {
    const int c = e >> 8, b = e & 255;
    uint32_t v = 0;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const int k = 4 * c + kk;
      if (k < s.L && ((s.pattern >> (s.L - 1 - k)) & 1ull)) {
        const int o = k == 0 ? 0 : __popcll(s.pattern >> (s.L - k));
        v |= (uint32_t)((b >> (6 - 2 * kk)) & 3) << (30 - 2 * o);
      }
    }
    lut[c][b] = v;
  }
}

// revcomp_mer in 32 bits (w <= 15): the reverse complement left-aligned,
// bit 0 set as the reverse-strand flag; min(f, revcomp32(f)) orders exactly
// as the 64-bit pair does.
__device__ __forceinline__ uint32_t revcomp_mer32(uint32_t mer, int w) {
  uint32_t r = __brev(~mer);
  r = ((r >> 1) & 0x55555555u) | ((r & 0x55555555u) << 1);
  return (r << (32 - 2 * w)) | 1u;
}

// The forward mer of the position u bases into a 64-bit window (u + L <= 32).
__device__ __forceinline__ uint32_t gather_mer32(uint64_t win, int u, const uint32_t (*lut)[256], int nb) {
  uint32_t f = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c)
    if (c < nb) f |= lut[c][(uint32_t)(win >> (56 - 8 * c - 2 * u)) & 255u];
  return f;
}

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace mvg

#define MVG_CUDA_TRY(expr)                                      \
  do {                                                          \
    cudaError_t _e = (expr);                                    \
    if (_e != cudaSuccess) return ::mvg::report_cuda(_e, #expr); \
  } while (0)

namespace mvg {
int report_cuda(cudaError_t e, const char* what);
int report_error(int code, const char* msg);
}  // namespace mvg
