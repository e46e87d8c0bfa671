// Host-side internals shared by the translation units of libmauve_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>

#include "mvg_common.cuh"

namespace mvg {

struct Ctx;

// Grow-only device buffers, one per slot, owned by the handle.  Calls reuse
// them, so steady-state calls allocate nothing.
struct Workspace {
  static constexpr int kSlots = 96;
  void* ptr[kSlots] = {};
  size_t size[kSlots] = {};
  void* get(Ctx* c, int slot, size_t bytes);
  void release();
};

struct MatchStats {
  uint64_t pairs = 0, collisions = 0, matches = 0, buckets = 0;
};

// Optional per-stage CUDA-event timing on the handle's stream (off by default).
constexpr int kMaxStages = 256;  // a many-wave gap-DP call marks three stages per wave

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;       // second stream for work that runs beside the main stream's
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaStream_t aux2 = nullptr, aux3 = nullptr;  // side streams of work already on two streams
  cudaEvent_t fork2 = nullptr, join2 = nullptr, fork3 = nullptr, join3 = nullptr;
  cudaStream_t aux4 = nullptr, aux5 = nullptr;  // a third lane of banded work and its side stream
  cudaEvent_t fork4 = nullptr, join4 = nullptr, fork5 = nullptr, join5 = nullptr;
  uint32_t* d_err = nullptr;     // device error word
  uint32_t* h_err = nullptr;     // pinned mirror
  uint64_t* h_scalars = nullptr; // pinned scalars for small device->host reads
  uint8_t* h_stage = nullptr;    // pinned staging of one call's host->device copies (bump allocated)
  size_t h_stage_cap = 0, h_stage_used = 0;
  void* h_off = nullptr;         // pinned buffer for gap-DP offsets read back from the device
  size_t h_off_cap = 0;
  uint64_t launches = 0;
  uint64_t tb_arena = ~0ull;  // capped per call at 60% of free device memory
  int dp_rows = 8;            // full gap-DP rows per lane (4 or 8)
  int band_rows = 4;          // banded gap-DP rows per lane (1, 2, 4 or 8)
  double band_whole = 0.5;    // bands covering at least this share of their matrix run whole
  int band_ring = 1;          // banded problems on the ring schedule where it is valid
  int band_gate = 0;          // band proposals: divergence gate window threshold (0 = off)
  int pair_bucket_cap = 3072;  // seed-join buckets sorted in shared memory up to this size
  long long dp_spin_limit = 1ll << 26;  // polls before a whole-CTA gap-DP wait gives up (about a second)
  int dp_graph = 1;                      // gap-DP passes launched as one recorded CUDA graph
  int dp_ckpt = 1;                       // full-DP passes keep checkpoints, the traceback recomputes blocks
  int64_t whole_full_rows = 512;         // banded calls: whole-matrix problems from this many rows go to the full DP
  int ring_max_rows = 32;                // banded calls: tallest ring group height used
  int dp_coop_strips = 16;               // full-DP problems of at least this many strips use a whole CTA
  cudaGraphExec_t dp_exec[2] = {};       // the executable graph of each DP lane, updated per call
  uint64_t graph_launches = 0;
  int mlp_tc = 1;              // MLP forward hidden layers on tcgen05 (else mma.sync)
  uint64_t mlp_tc_passes = 0;  // forward passes that ran on tcgen05
  Workspace ws;
  MatchStats stats;
  bool profiling = false;
  cudaEvent_t ev[kMaxStages + 1] = {};
  const char* stage_name[kMaxStages] = {};
  int nstage = -1;  // -1: no stage recorded yet in this call
  // host-side planning time of the call, by name (summed), when profiling
  static constexpr int kMaxHost = 12;
  double host_ms[kMaxHost] = {};
  const char* host_name[kMaxHost] = {};
  int nhost = 0;
};

// Marks the start of a named stage (and the end of the previous one).
inline void stage_mark(Ctx* c, const char* name) {
  if (!c->profiling) return;
  if (c->nstage < 0) c->nstage = 0;
  if (c->nstage >= kMaxStages) return;
  if (!c->ev[c->nstage]) cudaEventCreate(&c->ev[c->nstage]);
  // inside a recorded graph the mark must be an event-record node of its own
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(c->stream, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(c->ev[c->nstage], c->stream, cudaEventRecordExternal);
  else
    cudaEventRecord(c->ev[c->nstage], c->stream);
  c->stage_name[c->nstage] = name;
  c->nstage++;
}
inline void stage_begin_call(Ctx* c) {
  c->nstage = -1;
  c->nhost = 0;
}

// Wall time of a host-side section, added to the call's host stage `name`.
struct HostSpan {
  Ctx* c;
  const char* name;
  std::chrono::steady_clock::time_point t0;
  HostSpan(Ctx* c_, const char* n) : c(c_), name(n), t0(std::chrono::steady_clock::now()) {}
  ~HostSpan() {
    if (!c->profiling) return;
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (int k = 0; k < c->nhost; ++k)
      if (c->host_name[k] == name) {
        c->host_ms[k] += ms;
        return;
      }
    if (c->nhost < Ctx::kMaxHost) {
      c->host_name[c->nhost] = name;
      c->host_ms[c->nhost++] = ms;
    }
  }
};
inline void stage_end(Ctx* c) { stage_mark(c, "end"); }

// Sorted keys kept on the device for the join.
struct SmlKeys {
  const void* keys = nullptr;  // uint32 or uint64 compact keys: (seed bits << 1) | strand [, genome bit]
  const uint32_t* pos = nullptr;
  bool wide = false;
  uint64_t count = 0;
};

inline uint64_t packed_words(uint64_t n) { return (n * 2) / 32 + (((n * 2) % 32) ? 1 : 0) + 2; }

int upload_base_table();
int grid_for(uint64_t n, int threads);
int pack_sequence(Ctx* c, const uint8_t* d_seq, uint64_t n, uint32_t* d_packed);
int sml_sort(Ctx* c, const uint32_t* d_packed, uint64_t count, const SeedDesc& s, uint32_t* d_pos_out,
             uint64_t* d_mer_out, SmlKeys* keep, int slot_base);
// Both genomes' keys ((seed bits, strand, genome) with A = 0) sorted in one array.
// The bucketed seed join (pair_buckets.cu) for 32-bit keys and at most
// kPairBucketMaxKeys keys: pairs staged per bucket in mer order.
constexpr uint64_t kPairBucketMaxKeys = 1ull << 25;
struct PairBucketGeom {
  int bbits, nbuckets, npass, dbits, lbits, spass, sbits;
  int64_t tile, ntiles, nchunks;
};
PairBucketGeom pair_bucket_geom(uint64_t n, int w);
struct PairStage {
  const uint2* stage = nullptr;   // bucket b's pairs at stage[bstart[b] ..]: (pos A, pos B | reverse << 31)
  const uint32_t* bstart = nullptr;
  uint32_t* pcount = nullptr;     // pairs per bucket
  uint32_t* pbase = nullptr;      // room for their exclusive scan
  int nbuckets = 0;
};
int pair_buckets(Ctx* c, const uint32_t* ga, uint64_t ca, const uint32_t* gb, uint64_t cb, const SeedDesc& s,
                 PairStage* out);
// Exclusive scan of n <= 16384 counts in one launch; *total gets the sum.
void pair_scan_small(const uint32_t* in, int n, uint32_t* out, uint32_t* total, cudaStream_t st);
int pair_sort(Ctx* c, const uint32_t* ga, uint64_t ca, const uint32_t* gb, uint64_t cb, const SeedDesc& s,
              SmlKeys* out);
int check_device_error(Ctx* c);
// Pinned staging for a call's host->device copies: stage_reserve waits for
// the handle's streams, makes room for `need` bytes and starts the call's
// allocation over; h2d_async copies through it (a truly asynchronous copy,
// so the host goes on planning while the stream is busy), or straight from
// the pageable source when the staging is full.
int stage_reserve(Ctx* c, size_t need);
int h2d_async(Ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t st);
// bytes from the device to host memory through a pinned buffer, waiting
// for the handle's stream.
int pinned_d2h(Ctx* c, void* dst, const void* d_src, size_t bytes);
size_t sml_key_bytes(const SeedDesc& s);
int sml_build_into(const uint8_t* d_seq, uint64_t n, uint64_t count, const SeedDesc& s, uint32_t* packed, void* k0,
                   void* k1, uint32_t* v0, uint32_t* v1, uint32_t* scr, uint32_t* d_pos_out, uint64_t* d_mer_out,
                   cudaStream_t st, uint32_t* d_err, uint64_t* launches);

int pairwise_matches_dev(Ctx* c, const uint8_t* d_a, uint64_t na, const uint8_t* d_b, uint64_t nb, uint64_t seed,
                         int64_t* d_out, uint64_t cap, uint64_t* count);
int gapdp_batch_dev(Ctx* c, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb, const uint64_t* d_ob,
                    int64_t nprob, int32_t* d_scores, char* d_paths, const uint64_t* d_path_off, int64_t* d_path_len,
                    const uint64_t* h_oa, const uint64_t* h_ob, int32_t* d_env = nullptr);
int gapdp_banded_dev(Ctx* c, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb, const uint64_t* d_ob,
                     int64_t nprob, const int32_t* h_delta, const int32_t* h_half, int32_t* d_scores, char* d_paths,
                     const uint64_t* d_path_off, int64_t* d_path_len, uint8_t* h_used_band, const uint64_t* h_oa,
                     const uint64_t* h_ob, uint64_t* banded_cells);
int probe_int32_peak(Ctx* c, double* ops);
void mlp_release(const void* h);

}  // namespace mvg
