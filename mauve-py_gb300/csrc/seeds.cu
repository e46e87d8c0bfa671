// Seed path: 2-bit packing, spaced-seed canonical mers and the sorted mer
// list (SML) build.
//
//   k_pack          ASCII bases -> 2-bit MSB-first uint32 words, 16 bases per
//                   thread from one 128-bit load (translate32,
//                   LM/SortedMerList.cpp:425-459; table :29-47).
//   k_seed_keys     canonical spaced-seed mer of every position
//                   (GetSeedMer/RevCompMer/GetDnaSeedMer, :597-615, 726-769),
//                   emitted as a compact sort key: the 2w seed bits then the
//                   strand bit, (2w+1) bits in all, which orders exactly like
//                   the reference's 64-bit bmer.mer.
//   radix sort      stable LSD over those 2w+1 bits (prim.cuh).
//   k_seed_keys_pair  the pairwise matcher's keys: both genomes in one array,
//                   a genome bit below the SML key, sorted once.
#include <string.h>

#include <algorithm>

#include "mvg_internal.h"
#include "prim.cuh"

namespace mvg {

// translate32's table (LM/SortedMerList.cpp:29-47): every byte not listed
// maps to 0 (A).  Bit 7 of an entry flags '-', which the reference rejects.
__constant__ uint8_t c_base_table[256];

static void init_base_table_host(uint8_t* t) {
  memset(t, 0, 256);
  const char* c1 = "cCbByY";
  const char* c2 = "gGsSkK";
  for (const char* p = c1; *p; ++p) t[(uint8_t)*p] = 1;
  for (const char* p = c2; *p; ++p) t[(uint8_t)*p] = 2;
  t[(uint8_t)'t'] = 3;
  t[(uint8_t)'T'] = 3;
  t[(uint8_t)'-'] = 0x80;
}

int upload_base_table() {
  uint8_t t[256];
  init_base_table_host(t);
  MVG_CUDA_TRY(cudaMemcpyToSymbol(c_base_table, t, 256));
  return 0;
}

SeedDesc make_seed_desc(uint64_t pattern) {
  SeedDesc s;
  memset(&s, 0, sizeof(s));
  s.pattern = pattern;
  s.L = pattern ? 64 - __builtin_clzll(pattern) - __builtin_ctzll(pattern) : 0;
  s.w = __builtin_popcountll(pattern);
  s.seed_mask = s.w ? (~0ull << (64 - 2 * s.w)) : 0;
  uint64_t rev = 0;
  for (int k = 0; k < s.L; ++k) rev = (rev << 1) | ((pattern >> k) & 1ull);
  s.sym = s.L > 0 && rev == pattern;
  int out = 0;
  for (int k = 0; k < s.L;) {
    if (pattern & (1ull << (s.L - 1 - k))) {
      int st = k;
      while (k < s.L && (pattern & (1ull << (s.L - 1 - k)))) ++k;
      s.run_start[s.nruns] = (int8_t)st;
      s.run_len[s.nruns] = (int8_t)(k - st);
      s.run_out[s.nruns] = (int8_t)out;
      out += k - st;
      s.nruns++;
    } else {
      ++k;
    }
  }
  return s;
}

// One thread per output word: 16 bases, one 128-bit load when aligned.
__global__ void k_pack(const uint8_t* __restrict__ seq, uint64_t n, uint32_t* __restrict__ out, uint64_t words,
                       uint32_t* err) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const bool aligned = (((uintptr_t)seq) & 15) == 0;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += stride) {
    const uint64_t b0 = w * 16;
    uint32_t word = 0, bad = 0;
    if (b0 + 16 <= n && aligned) {
      uint4 v = __ldg(reinterpret_cast<const uint4*>(seq + b0));
      uint32_t parts[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          uint32_t t = c_base_table[(parts[q] >> (8 * k)) & 255u];
          bad |= t;
          word |= (t & 3u) << (30 - 2 * (q * 4 + k));
        }
      }
    } else {
      for (int k = 0; k < 16; ++k) {
        uint64_t i = b0 + k;
        if (i < n) {
          uint32_t t = c_base_table[seq[i]];
          bad |= t;
          word |= (t & 3u) << (30 - 2 * k);
        }
      }
    }
    if (bad & 0x80u) set_error(err, kDevGapChar);
    out[w] = word;
  }
}

// Canonical mer per position -> (2w+1)-bit key and the position.
template <typename K>
__global__ void k_seed_keys(const uint32_t* __restrict__ g, uint64_t count, SeedDesc s, K* __restrict__ keys,
                            uint32_t* __restrict__ pos) {
  __shared__ uint64_t lut[8][256];
  seed_lut_build(s, lut);
  __syncthreads();
  const int nb = seed_bytes(s);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const int shift = 64 - 2 * s.w;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < count; p += stride) {
    uint64_t m = canonical_mer_lut(g, p, lut, nb, s.w);
    keys[p] = (K)(((m >> shift) << 1) | (m & 1ull));
    pos[p] = (uint32_t)p;
  }
}

// Both genomes' keys in one array for the pairwise matcher: the SML key
// (seed bits, strand bit) followed by a genome bit (A = 0, B = 1); values are
// positions.  Sorted stably, every seed's occurrences in the two genomes are
// adjacent, each genome's in position order.  Blocks build the seed's gather
// table once and then take sort tiles of os::kTile positions in turn.  With
// 32-bit keys (weight <= 15) a thread makes the keys of 4 consecutive
// positions from one window and stores them as one 16-byte word.  Unless
// counts0 is null, each tile's first-pass digit counts are written as its
// count row (counts0) and added into its chunk's sums (csum0), the layout
// rts_sort_pairs reads when told the keys come counted.
template <typename K>
__global__ void __launch_bounds__(256) k_seed_keys_pair(const uint32_t* __restrict__ ga, uint64_t ca,
                                                        const uint32_t* __restrict__ gb, uint64_t cb, SeedDesc s,
                                                        K* __restrict__ keys, uint32_t* __restrict__ pos,
                                                        uint32_t* __restrict__ counts0, uint32_t* __restrict__ csum0,
                                                        int64_t ntiles, int64_t ctiles) {
  constexpr bool k32 = sizeof(K) == 4;
  __shared__ uint32_t h[8][256];
  __shared__ __align__(8) uint32_t lutw[k32 ? 8 * 256 : 2 * 8 * 256];
  const int tid = threadIdx.x, wid = tid >> 5;
  const bool count = counts0 != nullptr;
  auto lut32 = reinterpret_cast<uint32_t(*)[256]>(lutw);
  auto lut64 = reinterpret_cast<uint64_t(*)[256]>(lutw);
  if constexpr (k32)
    seed_lut_build32(s, lut32);
  else
    seed_lut_build(s, lut64);
#pragma unroll
  for (int w = 0; w < 8; ++w) h[w][tid] = 0;
  __syncthreads();
  const int nb = seed_bytes(s);
  const uint64_t n = ca + cb;
  // four positions from one 32-base window: u + L <= 32 and no byte shift
  // below zero (8 nb + 6 <= 64)
  const bool quad = nb <= 7;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t base = (uint64_t)tile * os::kTile;
    if constexpr (k32) {
      const int sh = 32 - 2 * s.w;
#pragma unroll
      for (int j = 0; j < os::kTile / 1024; ++j) {
        const uint64_t p0 = base + (uint64_t)j * 1024 + 4 * tid;
        if (p0 >= n) break;
        if (quad && p0 + 4 <= n && (p0 + 4 <= ca || p0 >= ca)) {
          const bool in_b = p0 >= ca;
          const uint64_t q0 = in_b ? p0 - ca : p0;
          const uint64_t win = window64(in_b ? gb : ga, q0);
          uint32_t kk[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const uint32_t f = gather_mer32(win, u, lut32, nb);
            const uint32_t r = revcomp_mer32(f, s.w);
            const uint32_t m = f < r ? f : r;
            kk[u] = ((((m >> sh) << 1) | (m & 1u)) << 1) | (in_b ? 1u : 0u);
          }
          *reinterpret_cast<uint4*>(keys + p0) = make_uint4(kk[0], kk[1], kk[2], kk[3]);
          *reinterpret_cast<uint4*>(pos + p0) =
              make_uint4((uint32_t)q0, (uint32_t)q0 + 1, (uint32_t)q0 + 2, (uint32_t)q0 + 3);
          if (count) {
#pragma unroll
            for (int u = 0; u < 4; ++u) atomicAdd(&h[wid][kk[u] & 255u], 1u);
          }
        } else {
          for (int u = 0; u < 4; ++u) {
            const uint64_t p = p0 + u;
            if (p >= n) break;
            const bool in_b = p >= ca;
            const uint64_t q = in_b ? p - ca : p;
            const uint32_t f = gather_mer32(window64(in_b ? gb : ga, q), 0, lut32, nb);
            const uint32_t r = revcomp_mer32(f, s.w);
            const uint32_t m = f < r ? f : r;
            const uint32_t key = ((((m >> sh) << 1) | (m & 1u)) << 1) | (in_b ? 1u : 0u);
            keys[p] = (K)key;
            pos[p] = (uint32_t)q;
            if (count) atomicAdd(&h[wid][key & 255u], 1u);
          }
        }
      }
    } else {
      const int shift = 64 - 2 * s.w;
#pragma unroll 2
      for (int k = 0; k < os::kItems; ++k) {
        const uint64_t p = base + (uint64_t)k * 256 + tid;
        if (p >= n) break;
        const bool in_b = p >= ca;
        const uint64_t q = in_b ? p - ca : p;
        const uint64_t m = canonical_mer_lut(in_b ? gb : ga, q, lut64, nb, s.w);
        const K key = (K)(((((m >> shift) << 1) | (m & 1ull)) << 1) | (in_b ? 1ull : 0ull));
        keys[p] = key;
        pos[p] = (uint32_t)q;
        if (count) atomicAdd(&h[wid][(uint32_t)key & 255u], 1u);
      }
    }
    if (count) {
      __syncthreads();
      uint32_t sum = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) {
        sum += h[w][tid];
        h[w][tid] = 0;
      }
      counts0[tile * 256 + tid] = sum;
      if (sum) atomicAdd(&csum0[(tile / ctiles) * 256 + tid], sum);
      __syncthreads();
    }
  }
}

template <typename K>
__global__ void k_key_to_mer(const K* __restrict__ keys, uint64_t count, int w, uint64_t* __restrict__ mer) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    uint64_t k = (uint64_t)keys[i];
    mer[i] = ((k >> 1) << (64 - 2 * w)) | (k & 1ull);
  }
}

int grid_for(uint64_t n, int threads) {
  uint64_t b = (n + threads - 1) / threads;
  const uint64_t cap = 152ull * 16;  // 16 resident blocks per SM on 152 SMs
  if (b > cap) b = cap;
  return (int)(b ? b : 1);
}

int pack_sequence(Ctx* c, const uint8_t* d_seq, uint64_t n, uint32_t* d_packed) {
  const uint64_t words = packed_words(n);
  k_pack<<<grid_for(words, 256), 256, 0, c->stream>>>(d_seq, n, d_packed, words, c->d_err);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename K>
static int sml_sort_impl(Ctx* c, const uint32_t* d_packed, uint64_t count, const SeedDesc& s, uint32_t* d_pos_out,
                         uint64_t* d_mer_out, SmlKeys* keep, int sb) {
  const int nbits = 2 * s.w + 1;
  Workspace& ws = c->ws;
  K* k0 = (K*)ws.get(c, sb + 0, count * sizeof(K));
  K* k1 = (K*)ws.get(c, sb + 1, count * sizeof(K));
  uint32_t* v0 = (uint32_t*)ws.get(c, sb + 2, count * sizeof(uint32_t));
  uint32_t* v1 = (uint32_t*)ws.get(c, sb + 3, count * sizeof(uint32_t));
  uint32_t* scr = (uint32_t*)ws.get(c, sb + 4, sort_scratch_words(count, nbits) * sizeof(uint32_t));
  if (!k0 || !k1 || !v0 || !v1 || !scr) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  k_seed_keys<K><<<grid_for(count, 256), 256, 0, c->stream>>>(d_packed, count, s, k0, v0);
  c->launches++;
  int which = sort_pairs<K>(k0, v0, k1, v1, (int64_t)count, nbits, scr, c->stream, &c->launches, c->d_err);
  K* ks = which ? k1 : k0;
  uint32_t* vs = which ? v1 : v0;
  if (d_pos_out) MVG_CUDA_TRY(cudaMemcpyAsync(d_pos_out, vs, count * sizeof(uint32_t), cudaMemcpyDeviceToDevice, c->stream));
  if (d_mer_out) {
    k_key_to_mer<K><<<grid_for(count, 256), 256, 0, c->stream>>>(ks, count, s.w, d_mer_out);
    c->launches++;
  }
  if (keep) {
    keep->keys = ks;
    keep->pos = vs;
    keep->wide = sizeof(K) == 8;
    keep->count = count;
  }
  MVG_CUDA_TRY(cudaGetLastError());
  return 0;
}

// The whole SML build on caller-provided device buffers (no workspace, no
// allocation): pack, seed keys, radix sort, positions and mers out.
// packed: packed_words(n) words; k0/k1: count keys of sml_key_bytes(s) each;
// v0/v1: count uint32; scr: radix_scratch_words(count) words.
template <typename K>
static int sml_build_into_impl(const uint8_t* d_seq, uint64_t n, uint64_t count, const SeedDesc& s, uint32_t* packed,
                               void* k0, void* k1, uint32_t* v0, uint32_t* v1, uint32_t* scr, uint32_t* d_pos_out,
                               uint64_t* d_mer_out, cudaStream_t st, uint32_t* d_err, uint64_t* launches) {
  const uint64_t words = packed_words(n);
  k_pack<<<grid_for(words, 256), 256, 0, st>>>(d_seq, n, packed, words, d_err);
  ++*launches;
  if (count == 0) return 0;
  k_seed_keys<K><<<grid_for(count, 256), 256, 0, st>>>(packed, count, s, (K*)k0, v0);
  ++*launches;
  const int which = radix_sort_pairs<K>((K*)k0, v0, (K*)k1, v1, (int64_t)count, 2 * s.w + 1, scr, st, launches);
  K* ks = which ? (K*)k1 : (K*)k0;
  uint32_t* vs = which ? v1 : v0;
  if (d_pos_out) MVG_CUDA_TRY(cudaMemcpyAsync(d_pos_out, vs, count * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  if (d_mer_out) {
    k_key_to_mer<K><<<grid_for(count, 256), 256, 0, st>>>(ks, count, s.w, d_mer_out);
    ++*launches;
  }
  MVG_CUDA_TRY(cudaGetLastError());
  return 0;
}

size_t sml_key_bytes(const SeedDesc& s) { return 2 * s.w + 1 <= 32 ? 4 : 8; }

int sml_build_into(const uint8_t* d_seq, uint64_t n, uint64_t count, const SeedDesc& s, uint32_t* packed, void* k0,
                   void* k1, uint32_t* v0, uint32_t* v1, uint32_t* scr, uint32_t* d_pos_out, uint64_t* d_mer_out,
                   cudaStream_t st, uint32_t* d_err, uint64_t* launches) {
  if (sml_key_bytes(s) == 4)
    return sml_build_into_impl<uint32_t>(d_seq, n, count, s, packed, k0, k1, v0, v1, scr, d_pos_out, d_mer_out, st,
                                         d_err, launches);
  return sml_build_into_impl<uint64_t>(d_seq, n, count, s, packed, k0, k1, v0, v1, scr, d_pos_out, d_mer_out, st,
                                       d_err, launches);
}

template <typename K>
static int pair_sort_impl(Ctx* c, const uint32_t* ga, uint64_t ca, const uint32_t* gb, uint64_t cb,
                          const SeedDesc& s, SmlKeys* out) {
  const uint64_t count = ca + cb;
  const int nbits = 2 * s.w + 2;
  Workspace& ws = c->ws;
  K* k0 = (K*)ws.get(c, 0, count * sizeof(K));
  K* k1 = (K*)ws.get(c, 1, count * sizeof(K));
  uint32_t* v0 = (uint32_t*)ws.get(c, 2, count * sizeof(uint32_t));
  uint32_t* v1 = (uint32_t*)ws.get(c, 3, count * sizeof(uint32_t));
  uint32_t* scr = (uint32_t*)ws.get(c, 4, sort_scratch_words(count, nbits) * sizeof(uint32_t));
  if (!k0 || !k1 || !v0 || !v1 || !scr) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  const RtsGeom g = rts_geom((int64_t)count, nbits);
  const unsigned grid = (unsigned)std::min<int64_t>(g.ntiles, 152 * 4);
  int which;
  if ((int64_t)count < (1ll << 31)) {  // the sort_pairs range of the reduce-then-scan sort
    uint32_t* csum = rts_csum(scr, g);
    MVG_CUDA_TRY(cudaMemsetAsync(csum, 0, (size_t)g.npass * g.nchunks * 256 * 4, c->stream));
    k_seed_keys_pair<K><<<grid, 256, 0, c->stream>>>(ga, ca, gb, cb, s, k0, v0, rts_counts(scr), csum, g.ntiles,
                                                      g.ctiles);
    c->launches++;
    which = rts_sort_pairs<K>(k0, v0, k1, v1, (int64_t)count, nbits, scr, c->stream, &c->launches, true);
  } else {
    k_seed_keys_pair<K><<<grid, 256, 0, c->stream>>>(ga, ca, gb, cb, s, k0, v0, nullptr, nullptr, g.ntiles, 1);
    c->launches++;
    which = sort_pairs<K>(k0, v0, k1, v1, (int64_t)count, nbits, scr, c->stream, &c->launches, c->d_err);
  }
  out->keys = which ? k1 : k0;
  out->pos = which ? v1 : v0;
  out->wide = sizeof(K) == 8;
  out->count = count;
  MVG_CUDA_TRY(cudaGetLastError());
  return 0;
}

int pair_sort(Ctx* c, const uint32_t* ga, uint64_t ca, const uint32_t* gb, uint64_t cb, const SeedDesc& s,
              SmlKeys* out) {
  if (2 * s.w + 2 <= 32) return pair_sort_impl<uint32_t>(c, ga, ca, gb, cb, s, out);
  return pair_sort_impl<uint64_t>(c, ga, ca, gb, cb, s, out);
}

int sml_sort(Ctx* c, const uint32_t* d_packed, uint64_t count, const SeedDesc& s, uint32_t* d_pos_out,
             uint64_t* d_mer_out, SmlKeys* keep, int slot_base) {
  if (2 * s.w + 1 <= 32) return sml_sort_impl<uint32_t>(c, d_packed, count, s, d_pos_out, d_mer_out, keep, slot_base);
  return sml_sort_impl<uint64_t>(c, d_packed, count, s, d_pos_out, d_mer_out, keep, slot_base);
}

}  // namespace mvg
