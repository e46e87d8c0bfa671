// C ABI (include/mauve_gb300.h): handle lifetime, host-buffer wrappers,
// error reporting and the grow-only device workspace.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mvg_internal.h"

namespace mvg {

static thread_local char g_last_error[512] = "";

int report_error(int code, const char* msg) {
  snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
  return code;
}

int report_cuda(cudaError_t e, const char* what) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? MVG_ERR_NOMEM : MVG_ERR_CUDA;
}

void* Workspace::get(Ctx* c, int slot, size_t bytes) {
  if (slot < 0 || slot >= kSlots) return nullptr;
  if (bytes == 0) bytes = 16;
  if (size[slot] >= bytes) return ptr[slot];
  if (ptr[slot]) {
    cudaStreamSynchronize(c->stream);
    cudaFree(ptr[slot]);
    ptr[slot] = nullptr;
    size[slot] = 0;
  }
  size_t want = bytes + bytes / 8 + 256;  // headroom so near-equal sizes reuse
  if (cudaMalloc(&ptr[slot], want) != cudaSuccess) {
    cudaGetLastError();
    ptr[slot] = nullptr;
    return nullptr;
  }
  size[slot] = want;
  return ptr[slot];
}

void Workspace::release() {
  for (int i = 0; i < kSlots; ++i) {
    if (ptr[i]) cudaFree(ptr[i]);
    ptr[i] = nullptr;
    size[i] = 0;
  }
}

int check_device_error(Ctx* c) {
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_err, c->d_err, 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  switch (*c->h_err) {
    case kDevOk:
      return 0;
    case kDevGapChar:
      return report_error(MVG_ERR_GAP_CHAR, "gap character '-' in genome sequence");
    case kDevBadBase:
      return report_error(MVG_ERR_BAD_BASE, "gap-DP base code outside 0..3");
    case kDevCapacity:
      return report_error(MVG_ERR_DEVICE, "device capacity bound exceeded");
    case kDevRange:
      return report_error(MVG_ERR_RANGE, "index out of range");
    case kDevOverflow:
      return report_error(MVG_ERR_OVERFLOW, "LUT value does not fit int32");
    default:
      return report_error(MVG_ERR_DEVICE, "device kernel reported an error");
  }
}

int upload_base_table();
int upload_score_table();

}  // namespace mvg

using namespace mvg;

struct mvg_context : public mvg::Ctx {};

// Resolved seed patterns (weights 3..31, ranks 0..5): getSeed() over the
// tables of LM/SeedMasks.h:44-260 with its solid fallbacks applied.
static const uint64_t kSeedTable[29][6] = {
    {0xb, 0x7, 0x7, 0x7, 0x7, 0x7},
    {0x3b, 0xf, 0xf, 0xf, 0xf, 0xf},
    {0x6b, 0x139, 0x193, 0x6b, 0x1f, 0x1f},
    {0x58d, 0x653, 0x1ab, 0xdb, 0x3f, 0x3f},
    {0x1953, 0x588d, 0x688b, 0x17d, 0x164d, 0x7f},
    {0x3927, 0x1ca7, 0x6553, 0xb6d, 0xff, 0xff},
    {0x7497, 0x1c927, 0x72a7, 0x6fb, 0x16ed, 0x1ff},
    {0x1d297, 0x3a497, 0xe997, 0x6d5b, 0x3ff, 0x3ff},
    {0x7954f, 0x75257, 0x1c9527, 0x5bed, 0x5b26d, 0x7ff},
    {0x7954f, 0x3d32f, 0x768b7, 0x5b56d, 0xfff, 0xfff},
    {0x792a4f, 0x1d64d7, 0x1d3597, 0x1b7db, 0x75ad7, 0x1fff},
    {0x1e6acf, 0xf59af, 0x3d4caf, 0x35ad6b, 0x3fff, 0x3fff},
    {0x7ac9af, 0x7b2a6f, 0x79aacf, 0x16df6d, 0x6b5d6b, 0x7fff},
    {0xf599af, 0xee5a77, 0x7cd59f, 0xeb5ad7, 0xffff, 0xffff},
    {0x6dbedb, 0x1ffff, 0x1ffff, 0x1ffff, 0x1ffff, 0x1ffff},
    {0x3e6b59f, 0x3eb335f, 0x7b3566f, 0x3ffff, 0x3ffff, 0x3ffff},
    {0x7b974ef, 0x7d6735f, 0x1edd74f, 0x7ffff, 0x7ffff, 0x7ffff},
    {0x1f59b35f, 0x3edcedf, 0xfae675f, 0xfffff, 0xfffff, 0xfffff},
    {0x7ddaddf, 0xaeb3f, 0x7eb76bf, 0x1fffff, 0x1fffff, 0x1fffff},
    {0x3fffff, 0x3fffff, 0x3fffff, 0x3fffff, 0x3fffff, 0x3fffff},
    {0x7fffff, 0x7fffff, 0x7fffff, 0x7fffff, 0x7fffff, 0x7fffff},
    {0xffffff, 0xffffff, 0xffffff, 0xffffff, 0xffffff, 0xffffff},
    {0x1ffffff, 0x1ffffff, 0x1ffffff, 0x1ffffff, 0x1ffffff, 0x1ffffff},
    {0x3ffffff, 0x3ffffff, 0x3ffffff, 0x3ffffff, 0x3ffffff, 0x3ffffff},
    {0x7ffffff, 0x7ffffff, 0x7ffffff, 0x7ffffff, 0x7ffffff, 0x7ffffff},
    {0xfffffff, 0xfffffff, 0xfffffff, 0xfffffff, 0xfffffff, 0xfffffff},
    {0x1fffffff, 0x1fffffff, 0x1fffffff, 0x1fffffff, 0x1fffffff, 0x1fffffff},
    {0x3fffffff, 0x3fffffff, 0x3fffffff, 0x3fffffff, 0x3fffffff, 0x3fffffff},
    {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff},
};

namespace mvg {

int stage_reserve(Ctx* c, size_t need) {
  for (cudaStream_t st : {c->stream, c->aux, c->aux2, c->aux3, c->aux4, c->aux5})
    if (st) MVG_CUDA_TRY(cudaStreamSynchronize(st));
  c->h_stage_used = 0;
  if (c->h_stage_cap >= need) return 0;
  if (c->h_stage) cudaFreeHost(c->h_stage);
  c->h_stage = nullptr;
  c->h_stage_cap = 0;
  const size_t want = need + need / 4 + (1 << 20);
  if (cudaMallocHost(&c->h_stage, want) != cudaSuccess) {
    cudaGetLastError();
    c->h_stage = nullptr;
    return 0;  // copies fall back to pageable sources
  }
  c->h_stage_cap = want;
  return 0;
}

int h2d_async(Ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return 0;
  const size_t off = (c->h_stage_used + 255) & ~(size_t)255;
  if (c->h_stage && off + bytes <= c->h_stage_cap) {
    memcpy(c->h_stage + off, src, bytes);
    c->h_stage_used = off + bytes;
    MVG_CUDA_TRY(cudaMemcpyAsync(dst, c->h_stage + off, bytes, cudaMemcpyHostToDevice, st));
    return 0;
  }
  MVG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
  return 0;
}

}  // namespace mvg

namespace mvg {

// bytes from the device into host memory through the handle's pinned
// buffer (one synchronisation, no pageable staging).
int pinned_d2h(Ctx* c, void* dst, const void* d_src, size_t bytes) {
  if (bytes == 0) return 0;
  if (c->h_off_cap < bytes) {
    if (c->h_off) cudaFreeHost(c->h_off);
    c->h_off = nullptr;
    c->h_off_cap = 0;
    MVG_CUDA_TRY(cudaMallocHost(&c->h_off, bytes + bytes / 4));
    c->h_off_cap = bytes + bytes / 4;
  }
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_off, d_src, bytes, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  memcpy(dst, c->h_off, bytes);
  return 0;
}

// Both offset arrays of a device gap-DP batch to the host, through a
// pinned buffer (one synchronisation, no pageable staging).
static int offsets_to_host(Ctx* c, const uint64_t* d_a, const uint64_t* d_b, int64_t nprob,
                           std::vector<uint64_t>& oa, std::vector<uint64_t>& ob) {
  const size_t bytes = (size_t)(nprob + 1) * 8;
  if (c->h_off_cap < 2 * bytes) {
    if (c->h_off) cudaFreeHost(c->h_off);
    c->h_off = nullptr;
    c->h_off_cap = 0;
    MVG_CUDA_TRY(cudaMallocHost(&c->h_off, 2 * bytes + bytes / 4));
    c->h_off_cap = 2 * bytes + bytes / 4;
  }
  uint8_t* hb = (uint8_t*)c->h_off;
  MVG_CUDA_TRY(cudaMemcpyAsync(hb, d_a, bytes, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(hb + bytes, d_b, bytes, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  oa.assign((const uint64_t*)hb, (const uint64_t*)hb + nprob + 1);
  ob.assign((const uint64_t*)(hb + bytes), (const uint64_t*)(hb + bytes) + nprob + 1);
  return 0;
}

}  // namespace mvg

extern "C" {

const char* mvg_last_error(void) { return g_last_error; }

int mvg_create(mvg_handle* out, int device) {
  if (!out) return report_error(MVG_ERR_ARG, "null handle pointer");
  *out = nullptr;
  MVG_CUDA_TRY(cudaSetDevice(device));
  mvg_context* c = new mvg_context();
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux3, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork3, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join3, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux4, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux5, cudaStreamNonBlocking);
  for (cudaEvent_t* ev : {&c->fork4, &c->join4, &c->fork5, &c->join5})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_err, 64);
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_err, 64);
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_scalars, 64);
  if (e != cudaSuccess) {
    delete c;
    return report_cuda(e, "mvg_create");
  }
  int rc = upload_base_table();
  if (!rc) rc = upload_score_table();
  if (rc) {
    delete c;
    return rc;
  }
  MVG_CUDA_TRY(cudaMemset(c->d_err, 0, 64));
  *out = c;
  return 0;
}

int mvg_destroy(mvg_handle h) {
  if (!h) return 0;
  cudaSetDevice(h->device);
  for (cudaStream_t st : {h->stream, h->aux, h->aux2, h->aux3, h->aux4, h->aux5})
    if (st) cudaStreamSynchronize(st);
  mlp_release(h);
  for (cudaGraphExec_t& g : h->dp_exec)
    if (g) cudaGraphExecDestroy(g);
  for (cudaEvent_t ev : h->ev)
    if (ev) cudaEventDestroy(ev);
  h->ws.release();
  if (h->d_err) cudaFree(h->d_err);
  if (h->h_err) cudaFreeHost(h->h_err);
  if (h->h_scalars) cudaFreeHost(h->h_scalars);
  if (h->h_stage) cudaFreeHost(h->h_stage);
  if (h->h_off) cudaFreeHost(h->h_off);
  for (cudaEvent_t ev : {h->fork, h->join, h->fork2, h->join2, h->fork3, h->join3, h->fork4, h->join4, h->fork5,
                         h->join5})
    if (ev) cudaEventDestroy(ev);
  for (cudaStream_t st : {h->aux5, h->aux4, h->aux3, h->aux2, h->aux, h->stream})
    if (st) cudaStreamDestroy(st);
  delete h;
  return 0;
}

void* mvg_stream(mvg_handle h) { return h ? (void*)h->stream : nullptr; }

uint64_t mvg_kernel_launches(mvg_handle h) { return h ? h->launches : 0; }

uint64_t mvg_get_seed(int weight, int rank) {
  if (weight > 31) return 0xffffffffull;
  if (rank > 5 || rank < 0) return (1ull << weight) - 1;  // includes SOLID_SEED = INT_MAX
  if (weight < 3) return 0;
  return kSeedTable[weight - 3][rank];
}

unsigned mvg_default_seed_weight(uint64_t avg_len) {
  unsigned w = (unsigned)ceil((log((double)avg_len) / log(2.0)) / 1.5);
  if (!(w & 1)) ++w;
  w = w < 5 ? 0 : w;
  if (avg_len == 0) w = 0;
  return w > 31 ? 31 : w;
}

int mvg_seed_length(uint64_t seed) { return seed ? 64 - __builtin_clzll(seed) - __builtin_ctzll(seed) : 0; }
int mvg_seed_weight(uint64_t seed) { return __builtin_popcountll(seed); }

int mvg_sml_build_dev(mvg_handle h, const uint8_t* d_seq, uint64_t n, uint64_t seed, uint32_t* d_pos_out,
                      uint64_t* d_mer_out, uint64_t cap, uint64_t* count) {
  if (!h || !count || (!d_seq && n)) return report_error(MVG_ERR_ARG, "null argument");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  const SeedDesc s = make_seed_desc(seed);
  if (s.L == 0 || s.L > 31) return report_error(MVG_ERR_ARG, "invalid seed pattern");
  if (n >= 0xffffffffull) return report_error(MVG_ERR_ARG, "sequence longer than 2^32-1");
  const uint64_t cnt = n >= (uint64_t)s.L ? n - s.L + 1 : 0;
  *count = cnt;
  if (cnt > cap) return report_error(MVG_ERR_CAPACITY, "SML output buffer too small");
  uint32_t* g = (uint32_t*)h->ws.get(h, 20, packed_words(n) * 4);
  if (!g) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemsetAsync(h->d_err, 0, 4, h->stream));
  int rc = pack_sequence(h, d_seq, n, g);
  if (rc) return rc;
  if (cnt) {
    rc = sml_sort(h, g, cnt, s, d_pos_out, d_mer_out, nullptr, 0);
    if (rc) return rc;
  }
  return check_device_error(h);
}

int mvg_sml_build(mvg_handle h, const uint8_t* seq, uint64_t n, uint64_t seed, uint32_t* pos_out, uint64_t* mer_out,
                  uint64_t cap, uint64_t* count) {
  if (!h || !count || (!seq && n)) return report_error(MVG_ERR_ARG, "null argument");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  const int L = mvg_seed_length(seed);
  const uint64_t cnt = (L && n >= (uint64_t)L) ? n - L + 1 : 0;
  *count = cnt;
  if (cnt > cap) return report_error(MVG_ERR_CAPACITY, "SML output buffer too small");
  uint8_t* d_seq = (uint8_t*)h->ws.get(h, 46, n + 16);
  uint32_t* d_pos = (uint32_t*)h->ws.get(h, 47, cnt * 4 + 16);
  uint64_t* d_mer = mer_out ? (uint64_t*)h->ws.get(h, 9, cnt * 8 + 16) : nullptr;
  if (!d_seq || !d_pos || (mer_out && !d_mer)) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemcpyAsync(d_seq, seq, n, cudaMemcpyHostToDevice, h->stream));
  int rc = mvg_sml_build_dev(h, d_seq, n, seed, d_pos, d_mer, cap, count);
  if (rc) return rc;
  if (pos_out) MVG_CUDA_TRY(cudaMemcpyAsync(pos_out, d_pos, cnt * 4, cudaMemcpyDeviceToHost, h->stream));
  if (mer_out) MVG_CUDA_TRY(cudaMemcpyAsync(mer_out, d_mer, cnt * 8, cudaMemcpyDeviceToHost, h->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return 0;
}

int mvg_pairwise_matches_dev(mvg_handle h, const uint8_t* d_seq_a, uint64_t na, const uint8_t* d_seq_b, uint64_t nb,
                             uint64_t seed, int64_t* d_out, uint64_t cap, uint64_t* count) {
  if (!h || !count || (!d_seq_a && na) || (!d_seq_b && nb) || (!d_out && cap))
    return report_error(MVG_ERR_ARG, "null argument");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  return pairwise_matches_dev(h, d_seq_a, na, d_seq_b, nb, seed, d_out, cap, count);
}

int mvg_pairwise_matches(mvg_handle h, const uint8_t* seq_a, uint64_t na, const uint8_t* seq_b, uint64_t nb,
                         uint64_t seed, int64_t* out, uint64_t cap, uint64_t* count) {
  if (!h || !count || (!seq_a && na) || (!seq_b && nb) || (!out && cap)) return report_error(MVG_ERR_ARG, "null argument");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  uint8_t* da = (uint8_t*)h->ws.get(h, 46, na + 16);
  uint8_t* db = (uint8_t*)h->ws.get(h, 47, nb + 16);
  const uint64_t dcap = std::max<uint64_t>(cap, 1);
  int64_t* dout = (int64_t*)h->ws.get(h, 57, dcap * 24);
  if (!da || !db || !dout) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemcpyAsync(da, seq_a, na, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(db, seq_b, nb, cudaMemcpyHostToDevice, h->stream));
  int rc = pairwise_matches_dev(h, da, na, db, nb, seed, dout, cap, count);
  if (rc && rc != MVG_ERR_CAPACITY) return rc;
  const uint64_t nout = std::min<uint64_t>(*count, cap);
  if (nout) MVG_CUDA_TRY(cudaMemcpyAsync(out, dout, nout * 24, cudaMemcpyDeviceToHost, h->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return rc;
}

int mvg_pairwise_stats(mvg_handle h, uint64_t stats[4]) {
  if (!h || !stats) return report_error(MVG_ERR_ARG, "null argument");
  stats[0] = h->stats.pairs;
  stats[1] = h->stats.collisions;
  stats[2] = h->stats.matches;
  stats[3] = h->stats.buckets;
  return 0;
}

int mvg_gapdp_batch_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                        const uint64_t* d_off_b, int64_t nprob, int32_t* d_scores, char* d_paths,
                        const uint64_t* d_path_off, int64_t* d_path_len) {
  if (!h || nprob < 0 || (nprob && (!d_off_a || !d_off_b || !d_scores)) || (d_paths && (!d_path_off || !d_path_len)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  std::vector<uint64_t> oa, ob;
  if (int rc = offsets_to_host(h, d_off_a, d_off_b, nprob, oa, ob)) return rc;
  return gapdp_batch_dev(h, d_seq_a, d_off_a, d_seq_b, d_off_b, nprob, d_scores, d_paths, d_path_off, d_path_len,
                         oa.data(), ob.data());
}

int mvg_gapdp_batch(mvg_handle h, const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                    const uint64_t* off_b, int64_t nprob, int32_t* scores, char* paths, const uint64_t* path_off,
                    int64_t* path_len) {
  if (!h || nprob < 0 || (nprob && (!off_a || !off_b || !scores || !seq_a || !seq_b)) ||
      (paths && (!path_off || !path_len)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  const uint64_t na = off_a[nprob], nb = off_b[nprob];
  const uint64_t np = paths ? path_off[nprob] : 0;
  uint8_t* dsa = (uint8_t*)h->ws.get(h, 46, na + 16);
  uint8_t* dsb = (uint8_t*)h->ws.get(h, 47, nb + 16);
  uint64_t* doa = (uint64_t*)h->ws.get(h, 5, (nprob + 1) * 8);
  uint64_t* dob = (uint64_t*)h->ws.get(h, 6, (nprob + 1) * 8);
  int32_t* dsc = (int32_t*)h->ws.get(h, 7, nprob * 4);
  char* dpa = paths ? (char*)h->ws.get(h, 9, np + 16) : nullptr;
  uint64_t* dpo = paths ? (uint64_t*)h->ws.get(h, 8, (nprob + 1) * 8) : nullptr;
  int64_t* dpl = paths ? (int64_t*)h->ws.get(h, 22, nprob * 8) : nullptr;
  if (!dsa || !dsb || !doa || !dob || !dsc || (paths && (!dpa || !dpo || !dpl)))
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemcpyAsync(dsa, seq_a, na, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dsb, seq_b, nb, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(doa, off_a, (nprob + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dob, off_b, (nprob + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  if (paths) MVG_CUDA_TRY(cudaMemcpyAsync(dpo, path_off, (nprob + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  int rc = gapdp_batch_dev(h, dsa, doa, dsb, dob, nprob, dsc, dpa, dpo, dpl, off_a, off_b);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemcpyAsync(scores, dsc, nprob * 4, cudaMemcpyDeviceToHost, h->stream));
  if (paths) {
    MVG_CUDA_TRY(cudaMemcpyAsync(paths, dpa, np, cudaMemcpyDeviceToHost, h->stream));
    MVG_CUDA_TRY(cudaMemcpyAsync(path_len, dpl, nprob * 8, cudaMemcpyDeviceToHost, h->stream));
  }
  MVG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return 0;
}

int mvg_gapdp_envelope_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                           const uint64_t* d_off_b, int64_t nprob, int32_t* d_scores, int32_t* d_env) {
  if (!h || nprob < 0 || (nprob && (!d_off_a || !d_off_b || !d_scores || !d_env)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  std::vector<uint64_t> oa, ob;
  if (int rc = offsets_to_host(h, d_off_a, d_off_b, nprob, oa, ob)) return rc;
  return gapdp_batch_dev(h, d_seq_a, d_off_a, d_seq_b, d_off_b, nprob, d_scores, nullptr, nullptr, nullptr, oa.data(),
                         ob.data(), d_env);
}

int mvg_gapdp_banded_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                         const uint64_t* d_off_b, int64_t nprob, const int32_t* band_delta, const int32_t* band_half,
                         int32_t* d_scores, char* d_paths, const uint64_t* d_path_off, int64_t* d_path_len,
                         uint8_t* used_band, uint64_t* cells) {
  if (!h || nprob < 0 || (nprob && (!d_off_a || !d_off_b || !d_scores || !band_delta || !band_half)) ||
      (d_paths && (!d_path_off || !d_path_len)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  std::vector<uint64_t> oa, ob;
  if (int rc = offsets_to_host(h, d_off_a, d_off_b, nprob, oa, ob)) return rc;
  return gapdp_banded_dev(h, d_seq_a, d_off_a, d_seq_b, d_off_b, nprob, band_delta, band_half, d_scores, d_paths,
                          d_path_off, d_path_len, used_band, oa.data(), ob.data(), cells);
}

int mvg_gapdp_banded(mvg_handle h, const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                     const uint64_t* off_b, int64_t nprob, const int32_t* band_delta, const int32_t* band_half,
                     int32_t* scores, char* paths, const uint64_t* path_off, int64_t* path_len, uint8_t* used_band,
                     uint64_t* cells) {
  if (!h || nprob < 0 || (nprob && (!off_a || !off_b || !scores || !seq_a || !seq_b || !band_delta || !band_half)) ||
      (paths && (!path_off || !path_len)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  const uint64_t na = off_a[nprob], nb = off_b[nprob];
  const uint64_t np = paths ? path_off[nprob] : 0;
  uint8_t* dsa = (uint8_t*)h->ws.get(h, 46, na + 16);
  uint8_t* dsb = (uint8_t*)h->ws.get(h, 47, nb + 16);
  uint64_t* doa = (uint64_t*)h->ws.get(h, 5, (nprob + 1) * 8);
  uint64_t* dob = (uint64_t*)h->ws.get(h, 6, (nprob + 1) * 8);
  int32_t* dsc = (int32_t*)h->ws.get(h, 7, nprob * 4);
  char* dpa = paths ? (char*)h->ws.get(h, 9, np + 16) : nullptr;
  uint64_t* dpo = paths ? (uint64_t*)h->ws.get(h, 8, (nprob + 1) * 8) : nullptr;
  int64_t* dpl = paths ? (int64_t*)h->ws.get(h, 22, nprob * 8) : nullptr;
  if (!dsa || !dsb || !doa || !dob || !dsc || (paths && (!dpa || !dpo || !dpl)))
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemcpyAsync(dsa, seq_a, na, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dsb, seq_b, nb, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(doa, off_a, (nprob + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dob, off_b, (nprob + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  if (paths) MVG_CUDA_TRY(cudaMemcpyAsync(dpo, path_off, (nprob + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  int rc = gapdp_banded_dev(h, dsa, doa, dsb, dob, nprob, band_delta, band_half, dsc, dpa, dpo, dpl, used_band, off_a,
                            off_b, cells);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemcpyAsync(scores, dsc, nprob * 4, cudaMemcpyDeviceToHost, h->stream));
  if (paths) {
    MVG_CUDA_TRY(cudaMemcpyAsync(paths, dpa, np, cudaMemcpyDeviceToHost, h->stream));
    MVG_CUDA_TRY(cudaMemcpyAsync(path_len, dpl, nprob * 8, cudaMemcpyDeviceToHost, h->stream));
  }
  MVG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return 0;
}

int mvg_set_tb_arena(mvg_handle h, uint64_t bytes) {
  if (!h || bytes < (1ull << 20)) return report_error(MVG_ERR_ARG, "arena must be at least 1 MiB");
  h->tb_arena = bytes;
  return 0;
}

int mvg_set_dp_rows(mvg_handle h, int full_rows, int band_rows) {
  if (!h || (full_rows != 4 && full_rows != 8) ||
      (band_rows != 1 && band_rows != 2 && band_rows != 4 && band_rows != 8))
    return report_error(MVG_ERR_ARG, "rows per lane: full DP 4 or 8, banded 1, 2, 4 or 8");
  h->dp_rows = full_rows;
  h->band_rows = band_rows;
  return 0;
}

int mvg_set_band_whole_fraction(mvg_handle h, double fraction) {
  if (!h || !(fraction > 0.0) || fraction > 1.0) return report_error(MVG_ERR_ARG, "fraction must be in (0, 1]");
  h->band_whole = fraction;
  return 0;
}

int mvg_set_band_ring(mvg_handle h, int on) {
  if (!h || (on != 0 && on != 1)) return report_error(MVG_ERR_ARG, "on must be 0 or 1");
  h->band_ring = on;
  return 0;
}

int mvg_set_dp_spin_limit(mvg_handle h, long long polls) {
  if (!h || polls < 1) return report_error(MVG_ERR_ARG, "spin limit must be at least 1");
  h->dp_spin_limit = polls;
  return 0;
}

int mvg_set_profiling(mvg_handle h, int on) {
  if (!h) return report_error(MVG_ERR_ARG, "null handle");
  h->profiling = on != 0;
  if (h->profiling) {  // created here, not at the first mark: marks may be recorded into a graph
    MVG_CUDA_TRY(cudaSetDevice(h->device));
    for (int k = 0; k <= kMaxStages; ++k)
      if (!h->ev[k]) MVG_CUDA_TRY(cudaEventCreate(&h->ev[k]));
  }
  return 0;
}

int mvg_set_dp_coop_strips(mvg_handle h, int strips) {
  if (!h || strips < 2 || strips > 1 << 20) return report_error(MVG_ERR_ARG, "strips must be in 2 .. 2^20");
  h->dp_coop_strips = strips;
  return 0;
}

int mvg_set_ring_max_rows(mvg_handle h, int rows) {
  if (!h || rows < 0 || rows > 32) return report_error(MVG_ERR_ARG, "rows must be in 0..32");
  h->ring_max_rows = rows;
  return 0;
}

int mvg_set_band_whole_full_rows(mvg_handle h, int64_t rows) {
  if (!h || rows < 1) return report_error(MVG_ERR_ARG, "rows must be at least 1");
  h->whole_full_rows = rows;
  return 0;
}

int mvg_set_dp_checkpoint(mvg_handle h, int on) {
  if (!h || (on != 0 && on != 1)) return report_error(MVG_ERR_ARG, "on must be 0 or 1");
  h->dp_ckpt = on;
  return 0;
}

int mvg_set_dp_graph(mvg_handle h, int on) {
  if (!h || (on != 0 && on != 1)) return report_error(MVG_ERR_ARG, "on must be 0 or 1");
  h->dp_graph = on;
  return 0;
}

int mvg_stage_times(mvg_handle h, char* names, size_t names_cap, double* ms, int cap, int* n) {
  if (!h || !n || (cap && !ms) || (names_cap && !names)) return report_error(MVG_ERR_ARG, "null argument");
  *n = 0;
  if (names_cap) names[0] = 0;
  size_t used = 0;
  auto add = [&](const char* prefix, const char* name, double t) {
    if (*n >= cap) return;
    ms[*n] = t;
    const size_t lp = strlen(prefix), len = strlen(name);
    if (names_cap && used + lp + len + 2 < names_cap) {
      if (used) names[used++] = ',';
      memcpy(names + used, prefix, lp);
      memcpy(names + used + lp, name, len);
      used += lp + len;
      names[used] = 0;
    }
    *n += 1;
  };
  if (h->nstage >= 2) {
    MVG_CUDA_TRY(cudaEventSynchronize(h->ev[h->nstage - 1]));
    for (int k = 0; k + 1 < h->nstage; ++k) {
      float t = 0;
      MVG_CUDA_TRY(cudaEventElapsedTime(&t, h->ev[k], h->ev[k + 1]));
      add("", h->stage_name[k], t);
    }
  }
  // host planning sections, after the device stages
  for (int k = 0; k < h->nhost; ++k) add("host_", h->host_name[k], h->host_ms[k]);
  return 0;
}

int mvg_probe_int32_peak(mvg_handle h, double* ops_per_s) {
  if (!h || !ops_per_s) return report_error(MVG_ERR_ARG, "null argument");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  return probe_int32_peak(h, ops_per_s);
}

}  // extern "C"
