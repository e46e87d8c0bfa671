// Batched gap-alignment DP: muscle NWSmall (MU/nwsmall.cpp:500-670) for two
// single DNA sequences, in int32, bit-exact in score and traceback; plus the
// banded variant with its exactness check and full-DP fallback.
//
// Scoring with MUSCLE's DNA defaults, all integer-valued in the reference's
// float arithmetic: match matrix NUC_SP + 60 (MU/nucmx.cpp:8-25), gap open
// -400 split into -200 open / -200 close per position
// (MU/profilefrommsa.cpp:291-292), extend 0, and TERMGAPS_Half
// (MU/termgaps.cpp:6-38), which zeroes the first position's open.  (The
// zeroed last close is never read by NWSmall's recurrences.)  The reference's
// -1e37 sentinel (MU/intmath.h:46) is represented by kNeg = -2^29: finite
// scores stay above -1.3e7 for 20 kbp inputs, and the only comparisons
// between two sentinel-derived values (D in row 1, I in column 1) see equal
// operands exactly as the float code does, so every traceback bit matches.
//
// Kernels: k_gapdp_t (gapdp_kernel.cuh) fills the traceback arena;
// k_traceback walks each problem's bits from (LA, LB) like BitTraceBack
// (MU/bittraceback.cpp:138-210); k_path_compact moves paths to slot heads.
// Full-DP passes run checkpointed by default: the forward kernel keeps
// strip rows and block columns instead of traceback bits, and k_tb_ck
// (traceback_ck.cuh) recomputes the bits of the blocks each path crosses.
#include <limits.h>

#include <algorithm>
#include <memory>
#include <cmath>
#include <functional>
#include <numeric>
#include <thread>
#include <vector>

#include "gapdp_kernel.cuh"
#include "traceback_win.cuh"
#include "traceback_ck.cuh"
#include "gapdp_ring.cuh"
#include "mvg_internal.h"

namespace mvg {

// Best score of each base code, biased, one byte per code (the banded
// kernel's bound).  The matrix is symmetric, so row and column maxima agree.
static uint32_t g_base_max = 0;

static bool score_rows_host(uint32_t* rows) {
  const int sp[4][4] = {{91, -114, -31, -123}, {-114, 100, -125, -31}, {-31, -125, 100, -114}, {-123, -31, -114, 91}};
  uint32_t bm = 0;
  for (int a = 0; a < 4; ++a) {
    uint32_t r = 0;
    int best = -1000;
    for (int b = 0; b < 4; ++b) {
      const int v = sp[a][b] + 60 + kScoreBias;
      if (v < 0 || v > 255) return false;
      if (sp[a][b] != sp[b][a]) return false;
      r |= (uint32_t)v << (8 * b);
      best = best > v ? best : v;
    }
    // the bound sums these maxima over unused bases too: they must be >= 0
    if (best - kScoreBias < 0) return false;
    rows[a] = r;
    bm |= (uint32_t)best << (8 * a);
  }
  g_base_max = bm;
  return true;
}

int upload_score_table() {
  uint32_t rows[4];
  if (!score_rows_host(rows)) return report_error(MVG_ERR_ARG, "score table does not fit the packed byte layout");
  MVG_CUDA_TRY(cudaMemcpyToSymbol(c_score_rows, rows, sizeof(rows)));
  return 0;
}

template __global__ void k_gapdp_t<false, 4>(DpJob);
template __global__ void k_gapdp_t<true, 4>(DpJob);
template __global__ void k_gapdp_t<false, 8>(DpJob);
template __global__ void k_gapdp_t<true, 8>(DpJob);
template __global__ void k_gapdp_t<true, 2>(DpJob);
template __global__ void k_gapdp_t<true, 1>(DpJob);
template __global__ void k_gapdp_t<false, 4, true>(DpJob);
template __global__ void k_gapdp_t<false, 8, true>(DpJob);
template __global__ void k_tb_ck<4>(const uint8_t*, const uint64_t*, const uint8_t*, const uint64_t*, const uint32_t*,
                                    const uint64_t*, int, const uint32_t*, const uint8_t*, const uint64_t*, char*,
                                    int64_t*, uint32_t*, int32_t*, unsigned*);
template __global__ void k_tb_ck<8>(const uint8_t*, const uint64_t*, const uint8_t*, const uint64_t*, const uint32_t*,
                                    const uint64_t*, int, const uint32_t*, const uint8_t*, const uint64_t*, char*,
                                    int64_t*, uint32_t*, int32_t*, unsigned*);
template __global__ void k_gapdp_ring<4>(RingJob);
template __global__ void k_gapdp_ring<6>(RingJob);
template __global__ void k_gapdp_ring<8>(RingJob);
template __global__ void k_gapdp_ring<12>(RingJob);
template __global__ void k_gapdp_ring<16>(RingJob);
template __global__ void k_gapdp_ring<24>(RingJob);
template __global__ void k_gapdp_ring<32>(RingJob);

// The group heights the ring schedule offers, smallest first.
static const int kRingRows[] = {4, 6, 8, 12, 16, 24, 32};
constexpr int kRingHeights = (int)(sizeof(kRingRows) / sizeof(kRingRows[0]));

// Runs f(begin, end, t) over [0, n) in up to 16 contiguous chunks on host
// threads (one chunk below 20,000 items), chunk t covering items before
// chunk t + 1's; returns the number of chunks.
// Indices 0..n-1 ordered by key (ascending, ties in index order): a stable
// LSD radix sort with 11-bit digits over the key's used bits.
static std::vector<uint32_t> radix_order(const std::vector<uint64_t>& key) {
  const size_t n = key.size();
  std::vector<uint32_t> a(n), b(n);
  for (size_t i = 0; i < n; ++i) a[i] = (uint32_t)i;
  uint64_t all = 0;
  for (uint64_t k : key) all |= k;
  for (int shift = 0; shift < 64 && (all >> shift) != 0; shift += 11) {
    uint32_t count[2049] = {};
    for (size_t i = 0; i < n; ++i) ++count[((key[a[i]] >> shift) & 2047u) + 1];
    for (int d = 0; d < 2048; ++d) count[d + 1] += count[d];
    for (size_t i = 0; i < n; ++i) b[count[(key[a[i]] >> shift) & 2047u]++] = a[i];
    a.swap(b);
  }
  return a;
}

template <class F>
static int host_chunks(int64_t n, F f) {
  int nt = 1;
  if (n >= 20000) {
    const unsigned hw = std::thread::hardware_concurrency();
    nt = (int)std::min<int64_t>(std::min<unsigned>(hw ? hw : 1, 16u), n / 5000);
    if (nt < 1) nt = 1;
  }
  if (nt == 1) {
    f((int64_t)0, n, 0);
    return 1;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) th.emplace_back(f, n * t / nt, n * (t + 1) / nt, t);
  for (auto& x : th) x.join();
  return nt;
}

static void (*ring_kernel(int R))(RingJob) {
  switch (R) {
    case 4: return k_gapdp_ring<4>;
    case 6: return k_gapdp_ring<6>;
    case 8: return k_gapdp_ring<8>;
    case 12: return k_gapdp_ring<12>;
    case 16: return k_gapdp_ring<16>;
    case 24: return k_gapdp_ring<24>;
    default: return k_gapdp_ring<32>;
  }
}

// BitTraceBack from (LA, LB); writes the path reversed at the end of the
// problem's path slot and its length.  Banded problems index their strips
// through the band geometry (only accepted ones are traced).
__global__ void k_traceback(const uint64_t* __restrict__ oa, const uint64_t* __restrict__ ob,
                            const uint32_t* __restrict__ order, const uint64_t* __restrict__ tb_off, int nwork,
                            const uint32_t* __restrict__ tb, const uint8_t* __restrict__ end_edge,
                            const int32_t* __restrict__ band_delta, const int32_t* __restrict__ band_half,
                            const uint8_t* __restrict__ accept, const uint64_t* __restrict__ path_off,
                            char* __restrict__ paths, int64_t* __restrict__ path_len, uint32_t* err,
                            int rows, int32_t* __restrict__ env, int long_path) {
  const int srows = 32 * rows;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += gridDim.x * blockDim.x) {
    const uint32_t p = order[w];
    if (accept && !accept[p]) continue;
    const int LA = (int)(oa[p + 1] - oa[p]), LB = (int)(ob[p + 1] - ob[p]);
    if (LA + LB >= long_path) continue;  // k_traceback_win walks it
    const uint32_t* T = tb + tb_off[w] / 4;
    const bool banded = band_delta != nullptr;
    const Band band = banded ? make_band(LA, LB, band_delta[p], band_half[p], srows) : make_full(LA, LB, srows);
    // strip k's word base and first column; strips are walked bottom-up
    int cur_k = (LA - 1) / srows;
    int64_t base = 0;
    for (int k = 0; k < cur_k; ++k)
      base += (int64_t)band_words_per_lane(band_hi(band, k) - band_lo(band, k) + 1, rows) * 32;
    int cur_lo = band_lo(band, cur_k);
    char* out = paths + path_off[p] + (LA + LB);  // writes go backwards from here
    int pa = LA, pb = LB;
    char cur = (char)end_edge[p];
    int64_t n = 0;
    const int64_t limit = (int64_t)LA + LB;
    // path envelope: extreme deviations of the visited cells (rows >= 1) from
    // the diagonal j = i*LB/LA, the quantity a band must cover
    int32_t dev_lo = INT32_MAX, dev_hi = INT32_MIN;
    for (;;) {
      if (n >= limit) {
        set_error(err, kDevCapacity);
        break;
      }
      *(--out) = cur;
      ++n;
      if (env && pa >= 1) {
        const int32_t dv = pb - (int32_t)((int64_t)pa * LB / LA);
        dev_lo = min(dev_lo, dv);
        dev_hi = max(dev_hi, dv);
      }
      uint32_t bits = 0;
      if (pa >= 1 && pb >= 1) {
        const int i0 = pa - 1;
        const int k = i0 / srows, rem = i0 % srows;
        while (cur_k > k) {  // move the strip window up
          --cur_k;
          base -= (int64_t)band_words_per_lane(band_hi(band, cur_k) - band_lo(band, cur_k) + 1, rows) * 32;
          cur_lo = band_lo(band, cur_k);
        }
        const int t = rem / rows, r = rem % rows;
        const int s = pb - cur_lo + t;
        if (s < t) {  // left of the strip: outside an accepted band cannot happen
          set_error(err, kDevCapacity);
          break;
        }
        const int nib = s * rows + r;
        bits = (T[base + (nib >> 3) * 32 + t] >> (4 * (nib & 7))) & 15u;
        // start fetching the word of the cell 8 steps further along the
        // diagonal (most steps are matches): 8 rows up in this strip, which
        // is another lane's stream (each step's word is otherwise a
        // dependent miss)
        if (rem >= 8 && pb > 8) {
          const int t8 = (rem - 8) / rows, r8 = (rem - 8) % rows;
          const int s8 = (pb - 8) - cur_lo + t8;
          if (s8 >= t8) {
            const int nib8 = s8 * rows + r8;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(T + base + (nib8 >> 3) * 32 + t8));
          }
        }
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
        set_error(err, kDevCapacity);
        break;
      }
      cur = next;
    }
    path_len[p] = n;
    if (env) {
      env[2 * p] = dev_lo;
      env[2 * p + 1] = dev_hi;
    }
  }
}

// Moves each path from the tail of its slot to the head (warp per problem).
__global__ void k_path_compact(const uint64_t* __restrict__ oa, const uint64_t* __restrict__ ob,
                               const uint32_t* __restrict__ order, int nwork, const uint8_t* __restrict__ accept,
                               const uint64_t* __restrict__ path_off, char* paths,
                               const int64_t* __restrict__ path_len) {
  const int lane = threadIdx.x & 31;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwork; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t p = order[w];
    if (accept && !accept[p]) continue;
    const int64_t slot = (int64_t)(oa[p + 1] - oa[p]) + (int64_t)(ob[p + 1] - ob[p]);
    const int64_t n = path_len[p];
    char* dst = paths + path_off[p];
    const char* src = dst + (slot - n);
    if (src == dst) continue;
    for (int64_t c = 0; c < n; c += 32) {
      char v = 0;
      if (c + lane < n) v = src[c + lane];
      __syncwarp();
      if (c + lane < n) dst[c + lane] = v;
      __syncwarp();
    }
  }
}

struct DpInputs {
  const uint8_t* sa;
  const uint64_t* oa;
  const uint8_t* sb;
  const uint64_t* ob;
  int32_t* scores;
  char* paths;
  const uint64_t* path_off;
  int64_t* path_len;
  int32_t* env = nullptr;  // optional path envelope output [2 * nprob]
};

// Starts the long-path walker for one wave on the aux stream (joined by
// tb_long_join), beside the thread walker on the main stream.  A warp walks
// a path about ten times faster than a thread but far fewer warps than
// threads run at once, so warps take the longest paths only: those with
// LA + LB >= kTbLongPath, at most one round of the walker's warps, longest
// first.  *long_path receives the length from which paths go to warps.
// The streams one DP pass runs on: its own, and the side stream its
// long-path walker forks to, with the events and workspace slots for that.
struct TbLanes {
  cudaStream_t st, side;
  cudaEvent_t fork, join;
  int slot_list, slot_ctr;
};

static TbLanes main_lanes(Ctx* c) { return TbLanes{c->stream, c->aux, c->fork, c->join, 62, 63}; }

// Host side of the long-path walker: the slots (of this wave's order) whose
// paths go to warps, longest first, and the length from which they do.
static int tb_long_plan(Ctx* c, const std::vector<uint32_t>& slot_len, std::vector<uint32_t>* long_slots,
                        int* long_path, int* grid) {
  long_slots->clear();
  *long_path = INT_MAX;
  *grid = 0;
  static bool attr = false;  // once per process: more than 48 KB of shared memory
  static int cap = 0;
  int sms = 0;
  MVG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  if (!attr) {
    MVG_CUDA_TRY(cudaFuncSetAttribute(k_traceback_win, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTbSmem));
    int bps = 0;
    MVG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_traceback_win, kTbWarps * 32, kTbSmem));
    cap = std::max(1, bps) * kTbWarps;
    attr = true;
  }
  const size_t round = (size_t)cap * (size_t)sms;
  std::vector<uint32_t> lens;
  for (uint32_t L : slot_len)
    if (L >= (uint32_t)kTbLongPath) lens.push_back(L);
  if (lens.empty()) return 0;
  uint32_t thr = kTbLongPath;
  if (lens.size() > round) {
    std::nth_element(lens.begin(), lens.begin() + (round - 1), lens.end(), std::greater<uint32_t>());
    thr = std::max<uint32_t>(thr, lens[round - 1]);
  }
  std::vector<std::pair<uint32_t, uint32_t>> sel;  // (length, slot)
  for (size_t q = 0; q < slot_len.size(); ++q)
    if (slot_len[q] >= thr) sel.push_back({slot_len[q], (uint32_t)q});
  std::sort(sel.begin(), sel.end(), [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
    return a.first != b.first ? a.first > b.first : a.second < b.second;
  });
  long_slots->resize(sel.size());
  for (size_t q = 0; q < sel.size(); ++q) (*long_slots)[q] = sel[q].second;
  const int n = (int)long_slots->size();
  *grid = std::min(sms * (cap / kTbWarps), (n + kTbWarps - 1) / kTbWarps);
  *long_path = (int)thr;
  return 0;
}

// Device side: the walker's launch on the side stream, forked from and
// joined back to the pass's stream (tb_long_join).  Stream operations only,
// so a pass's launches can be recorded into a CUDA graph.
static int tb_long_launch(Ctx* c, const TbLanes& L, const DpInputs& in, const uint32_t* d_order,
                          const uint64_t* d_tboff, const uint32_t* tb, const uint8_t* d_edge, const int32_t* d_delta,
                          const int32_t* d_half, const uint8_t* d_accept, int rows, const uint8_t* d_rows,
                          const uint32_t* d_slots, int n, int grid, unsigned* d_ctr) {
  MVG_CUDA_TRY(cudaMemsetAsync(d_ctr, 0, 4, L.st));
  MVG_CUDA_TRY(cudaEventRecord(L.fork, L.st));
  MVG_CUDA_TRY(cudaStreamWaitEvent(L.side, L.fork, 0));
  k_traceback_win<<<grid, kTbWarps * 32, kTbSmem, L.side>>>(in.oa, in.ob, d_order, d_tboff, d_slots, n, tb, d_edge,
                                                            d_delta, d_half, d_accept, in.path_off, in.paths,
                                                            in.path_len, c->d_err, rows, d_rows, in.env, d_ctr);
  MVG_CUDA_TRY(cudaEventRecord(L.join, L.side));
  c->launches++;
  return 0;
}

static int tb_long_fork(Ctx* c, const TbLanes& L, const DpInputs& in, const std::vector<uint32_t>& slot_len,
                        const uint32_t* d_order, const uint64_t* d_tboff, const uint32_t* tb, const uint8_t* d_edge,
                        const int32_t* d_delta, const int32_t* d_half, const uint8_t* d_accept, int rows,
                        const uint8_t* d_rows, int* long_path, bool* forked) {
  *forked = false;
  std::vector<uint32_t> long_slots;
  int grid = 0;
  if (int e = tb_long_plan(c, slot_len, &long_slots, long_path, &grid)) return e;
  if (long_slots.empty()) return 0;
  const int n = (int)long_slots.size();
  uint32_t* d_slots = (uint32_t*)c->ws.get(c, L.slot_list, (size_t)n * 4 + 16);
  unsigned* d_ctr = (unsigned*)c->ws.get(c, L.slot_ctr, 64);
  if (!d_slots || !d_ctr) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (int e = h2d_async(c, d_slots, long_slots.data(), (size_t)n * 4, L.st)) return e;
  if (int e = tb_long_launch(c, L, in, d_order, d_tboff, tb, d_edge, d_delta, d_half, d_accept, rows, d_rows,
                             d_slots, n, grid, d_ctr))
    return e;
  *forked = true;
  return 0;
}

static int tb_long_join(const TbLanes& L, bool forked) {
  if (forked) MVG_CUDA_TRY(cudaStreamWaitEvent(L.st, L.join, 0));
  return 0;
}

// Records the stream work issued between begin() and launch() into a CUDA
// graph (stream capture in thread-local mode, so only this thread's calls
// are restricted) and launches it as one graph; the executable graph is
// kept by the caller and updated in place from the next recording when the
// shape is unchanged (kernel arguments and grid sizes may differ), else
// instantiated anew.  With recording off, or when the caller's stream is
// already being captured, the work is issued directly and launch() does
// nothing.  An error while recording ends the capture and discards it.
class GraphRecorder {
 public:
  GraphRecorder(Ctx* c, cudaStream_t st, bool on) : c_(c), st_(st), on_(on) {}
  ~GraphRecorder() { discard(); }
  int begin() {
    if (!on_) return 0;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    MVG_CUDA_TRY(cudaStreamIsCapturing(st_, &cs));
    if (cs != cudaStreamCaptureStatusNone) return 0;
    MVG_CUDA_TRY(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
    active_ = true;
    return 0;
  }
  int check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    discard();
    return report_cuda(e, what);
  }
  int check(int rc) {
    if (rc) discard();
    return rc;
  }
  int launch(cudaGraphExec_t* exec) {
    if (!active_) return 0;
    active_ = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st_, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return report_cuda(e, "cudaStreamEndCapture");
    }
    if (*exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(*exec, g, &info) != cudaSuccess) {
        cudaGetLastError();  // a different shape: instantiate below
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
      }
    }
    if (!*exec && (e = cudaGraphInstantiate(exec, g, 0)) != cudaSuccess) {
      *exec = nullptr;
      cudaGraphDestroy(g);
      return report_cuda(e, "cudaGraphInstantiate");
    }
    cudaGraphDestroy(g);
    MVG_CUDA_TRY(cudaGraphLaunch(*exec, st_));
    c_->graph_launches++;
    return 0;
  }

 private:
  void discard() {
    if (!active_) return;
    active_ = false;
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(st_, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
  }
  Ctx* c_;
  cudaStream_t st_;
  bool on_;
  bool active_ = false;
};

// Runs the DP for the problems in `ids` (full, or banded with per-problem
// delta/half on the device): LPT order, size-mixed waves that fit the
// traceback arena, then traceback and path compaction per wave.
// Workspace slots of one run_dp lane: row buffers, order, traceback
// offsets, claim counter, traceback arena.
struct DpSlots {
  int rowbuf, order, tboff, counter, arena;
};
constexpr DpSlots kDpSlots{10, 11, 12, 14, 18};
constexpr DpSlots kDpSlotsLane2{49, 50, 51, 52, 53};

static int run_dp(Ctx* c, const DpInputs& in, const std::vector<uint32_t>& ids, const std::vector<int64_t>& la,
                  const std::vector<int64_t>& lb, const int32_t* d_delta, const int32_t* d_half,
                  const std::vector<int32_t>* h_delta, const std::vector<int32_t>* h_half, uint8_t* d_accept,
                  const TbLanes* lanes = nullptr, const DpSlots& sl = kDpSlots) {
  const TbLanes L = lanes ? *lanes : main_lanes(c);
  const int64_t nwork = (int64_t)ids.size();
  if (nwork == 0) return 0;
  std::unique_ptr<HostSpan> span(new HostSpan(c, "dp_plan"));
  const bool banded = d_delta != nullptr;
  // banded passes may use shorter strips: the staircase of a narrow band
  // widens by the diagonal's drift over one strip
  const int rows = banded ? c->band_rows : c->dp_rows;
  // full passes keep checkpoints instead of traceback bits (traceback_ck.cuh)
  const bool ckpt = !banded && c->dp_ckpt && (rows == 4 || rows == 8);
  std::unique_ptr<HostSpan> sub(new HostSpan(c, "dp_sizes"));
  std::vector<uint64_t> bytes(nwork), cells(nwork);
  int64_t maxlb = 0;
  for (int64_t w = 0; w < nwork; ++w) {
    const uint32_t p = ids[w];
    const Band b = banded ? make_band((int)la[p], (int)lb[p], (*h_delta)[p], (*h_half)[p], 32 * rows)
                          : make_full((int)la[p], (int)lb[p], 32 * rows);
    const uint64_t slot = ckpt ? (uint64_t)ck_entries((int)la[p], (int)lb[p], rows) * sizeof(int4)
                               : band_tb_words(b, rows) * 4;
    cells[w] = banded ? band_cells(b) : (uint64_t)la[p] * (uint64_t)lb[p];
    bytes[w] = (slot + 255) & ~255ull;
    maxlb = std::max(maxlb, lb[p]);
  }
  // Whole-CTA (pipelined) mode for problems with many strips.  A banded
  // strip can only start once the previous one has passed the next strip's
  // first column (about one strip height of drift plus the 64-column
  // prefetch), so narrow bands would leave the pipeline nearly serial: they
  // stay on one warp unless their strips are at least 8 strip heights wide.
  std::vector<char> is_big(nwork);
  for (int64_t w = 0; w < nwork; ++w) {
    const int64_t a = la[ids[w]];
    const bool many = (a + 32 * rows - 1) / (32 * rows) >= (banded ? kCoopMinStrips : c->dp_coop_strips);
    is_big[w] = many && (!banded || cells[w] >= (uint64_t)a * 8 * 32 * rows);
  }
  // largest first, ties in input order: one sort of packed (cells, index) keys
  sub.reset(new HostSpan(c, "dp_sort"));
  std::vector<uint32_t> idx;
  {
    constexpr uint64_t kMax = (1ull << 40) - 1;  // at most 1e6 x 1e6 cells
    std::vector<uint64_t> key(nwork);
    for (int64_t w = 0; w < nwork; ++w) key[w] = kMax - std::min(cells[w], kMax);
    idx = radix_order(key);
  }

  uint64_t arena = c->tb_arena;
  {
    size_t free_b = 0, total_b = 0;
    HostSpan mem_span(c, "meminfo");
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
      const size_t have = c->ws.size[sl.arena] + free_b;  // the arena slot itself may be re-allocated
      const uint64_t cap = (uint64_t)(have * 0.6);
      if (arena > cap) arena = cap;
    }
  }
  uint64_t total_tb = 0, max_tb = 0;
  for (int64_t w = 0; w < nwork; ++w) {
    total_tb += bytes[w];
    max_tb = std::max(max_tb, bytes[w]);
  }
  if (max_tb > arena) return report_error(MVG_ERR_CAPACITY, "one gap-DP problem exceeds the traceback arena");
  sub.reset(new HostSpan(c, "dp_waves"));
  // Waves: deal the size-sorted problems round-robin, so every wave holds the
  // same mix of sizes and stays largest-first inside.
  // at least one wave: checkpointed slots of problems within one block hold nothing
  int64_t nwaves = std::max<int64_t>(1, (int64_t)((total_tb + arena - 1) / arena));
  std::vector<uint32_t> order;
  std::vector<uint64_t> tboff;
  std::vector<int64_t> wave_begin, wave_nbig;
  uint64_t arena_need = 0;
  for (;;) {
    order.clear();
    tboff.clear();
    wave_begin.clear();
    wave_nbig.clear();
    arena_need = 0;
    bool fits = true;
    for (int64_t v = 0; v < nwaves && fits; ++v) {
      wave_begin.push_back((int64_t)order.size());
      uint64_t acc = 0;
      // large problems (solved by a whole CTA) first, then the rest; each part largest first
      int64_t nb = 0;
      for (int pass = 0; pass < 2; ++pass)
        for (int64_t q = v; q < nwork; q += nwaves) {
          const bool big = is_big[idx[q]];
          if (big != (pass == 0)) continue;
          order.push_back(ids[idx[q]]);
          tboff.push_back(acc);
          acc += bytes[idx[q]];
          nb += big;
        }
      wave_nbig.push_back(nb);
      if (acc > arena) fits = false;
      arena_need = std::max(arena_need, acc);
    }
    if (fits) break;
    ++nwaves;
  }
  wave_begin.push_back(nwork);

  sub.reset(new HostSpan(c, "dp_copy"));
  int dev_sms = 0;
  MVG_CUDA_TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  void (*kern)(DpJob) = ckpt        ? (rows == 8 ? k_gapdp_t<false, 8, true> : k_gapdp_t<false, 4, true>)
                        : rows == 8 ? (banded ? k_gapdp_t<true, 8> : k_gapdp_t<false, 8>)
                        : rows == 4 ? (banded ? k_gapdp_t<true, 4> : k_gapdp_t<false, 4>)
                        : rows == 2 ? k_gapdp_t<true, 2>
                                    : k_gapdp_t<true, 1>;
  int bps = 0;
  MVG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, kDpThreads, 0));
  if (bps < 1) bps = 1;
  const int grid = dev_sms * bps;
  const int64_t nwarps = (int64_t)grid * (kDpThreads / 32);
  Workspace& ws = c->ws;
  const int64_t rb_stride = maxlb + 2;
  int4* rowbuf = (int4*)ws.get(c, sl.rowbuf, (size_t)nwarps * rb_stride * sizeof(int4));
  uint32_t* d_order = (uint32_t*)ws.get(c, sl.order, (size_t)nwork * 4);
  uint64_t* d_tboff = (uint64_t*)ws.get(c, sl.tboff, (size_t)nwork * 8);
  uint8_t* d_edge = (uint8_t*)ws.get(c, 13, (size_t)(la.size()) + 16);  // per problem, shared by all lanes
  unsigned* d_counter = (unsigned*)ws.get(c, sl.counter, 64);
  uint32_t* tb = (uint32_t*)ws.get(c, sl.arena, std::max<uint64_t>(arena_need, 256));
  if (!rowbuf || !d_order || !d_tboff || !d_edge || !d_counter || !tb)
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (int e = h2d_async(c, d_order, order.data(), (size_t)nwork * 4, L.st)) return e;
  if (int e = h2d_async(c, d_tboff, tboff.data(), (size_t)nwork * 8, L.st)) return e;
  // the long-path walkers of all waves: slot lists concatenated, one counter each
  const size_t nwaves_run = wave_begin.size() - 1;
  std::vector<int> long_path(nwaves_run, INT_MAX), long_n(nwaves_run, 0), long_grid(nwaves_run, 0);
  std::vector<size_t> long_at(nwaves_run, 0);
  std::vector<uint32_t> all_long;
  for (size_t wv = 0; wv < nwaves_run; ++wv) {
    const int64_t w0 = wave_begin[wv], w1 = wave_begin[wv + 1];
    std::vector<uint32_t> slot_len(w1 - w0), ls;
    for (int64_t q = w0; q < w1; ++q) slot_len[q - w0] = (uint32_t)(la[order[q]] + lb[order[q]]);
    if (!ckpt)  // checkpointed passes walk every path on a warp
      if (int e = tb_long_plan(c, slot_len, &ls, &long_path[wv], &long_grid[wv])) return e;
    long_at[wv] = all_long.size();
    long_n[wv] = (int)ls.size();
    all_long.insert(all_long.end(), ls.begin(), ls.end());
  }
  int ck_grid = 0;
  if (ckpt) {
    static bool ck_attr[2] = {false, false};  // once per process and kernel: more than 48 KB of shared memory
    void (*tbk)(const uint8_t*, const uint64_t*, const uint8_t*, const uint64_t*, const uint32_t*, const uint64_t*,
                int, const uint32_t*, const uint8_t*, const uint64_t*, char*, int64_t*, uint32_t*, int32_t*,
                unsigned*) = rows == 8 ? k_tb_ck<8> : k_tb_ck<4>;
    if (!ck_attr[rows == 8]) {
      MVG_CUDA_TRY(cudaFuncSetAttribute(tbk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCkSmem));
      ck_attr[rows == 8] = true;
    }
    int cbps = 0;
    MVG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cbps, tbk, kCkWarps * 32, kCkSmem));
    ck_grid = dev_sms * std::max(1, cbps);
  }
  uint32_t* d_long = (uint32_t*)ws.get(c, L.slot_list, all_long.size() * 4 + 16);
  unsigned* d_long_ctr = (unsigned*)ws.get(c, L.slot_ctr, nwaves_run * 4 + 64);
  if (!d_long || !d_long_ctr) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (!all_long.empty())
    if (int e = h2d_async(c, d_long, all_long.data(), all_long.size() * 4, L.st)) return e;
  sub.reset();
  span.reset();
  // Every wave's launches (claim counters, the persistent DP kernel, the two
  // traceback walkers, path compaction) are recorded into one CUDA graph and
  // launched at once; the executable graph is kept per lane and updated in
  // place when the next call has the same shape.
  const int lane_id = sl.arena == kDpSlots.arena ? 0 : 1;
  GraphRecorder rec(c, L.st, c->dp_graph != 0);
  if (int e = rec.begin()) return e;
  for (size_t wv = 0; wv < nwaves_run; ++wv) {
    const int64_t w0 = wave_begin[wv], w1 = wave_begin[wv + 1];
    DpJob J;
    J.sa = in.sa;
    J.oa = in.oa;
    J.sb = in.sb;
    J.ob = in.ob;
    J.order = d_order + w0;
    J.tb_off = d_tboff + w0;
    J.nwork = (int)(w1 - w0);
    J.nbig = (int)wave_nbig[wv];
    J.tb = tb;
    J.rowbuf = rowbuf;
    J.rowbuf_stride = rb_stride;
    J.scores = in.scores;
    J.end_edge = d_edge;
    J.band_delta = d_delta;
    J.band_half = d_half;
    J.accept = d_accept;
    J.base_max = g_base_max;
    J.counter = d_counter;
    J.err = c->d_err;
    J.spin_limit = c->dp_spin_limit;
    if (int e = rec.check(cudaMemsetAsync(d_counter, 0, 8, L.st), "cudaMemsetAsync")) return e;
    stage_mark(c, banded ? "dp_banded" : "dp");
    kern<<<grid, kDpThreads, 0, L.st>>>(J);
    stage_mark(c, "traceback");
    if (ckpt) {
      unsigned* ctr = d_long_ctr + wv;
      if (int e = rec.check(cudaMemsetAsync(ctr, 0, 4, L.st), "cudaMemsetAsync")) return e;
      if (rows == 8)
        k_tb_ck<8><<<ck_grid, kCkWarps * 32, kCkSmem, L.st>>>(in.sa, in.oa, in.sb, in.ob, J.order, J.tb_off, J.nwork,
                                                               tb, d_edge, in.path_off, in.paths, in.path_len,
                                                               c->d_err, in.env, ctr);
      else
        k_tb_ck<4><<<ck_grid, kCkWarps * 32, kCkSmem, L.st>>>(in.sa, in.oa, in.sb, in.ob, J.order, J.tb_off, J.nwork,
                                                               tb, d_edge, in.path_off, in.paths, in.path_len,
                                                               c->d_err, in.env, ctr);
      stage_mark(c, "path_compact");
      k_path_compact<<<grid_for((int64_t)J.nwork * 32, 256), 256, 0, L.st>>>(
          in.oa, in.ob, J.order, J.nwork, d_accept, in.path_off, in.paths, in.path_len);
      c->launches += 3;
      if (int e = rec.check(cudaGetLastError(), "kernel launch")) return e;
      continue;
    }
    const bool forked = long_n[wv] > 0;
    if (forked)
      if (int e = rec.check(tb_long_launch(c, L, in, J.order, J.tb_off, tb, d_edge, d_delta, d_half, d_accept, rows,
                                           nullptr, d_long + long_at[wv], long_n[wv], long_grid[wv],
                                           d_long_ctr + wv)))
        return e;
    k_traceback<<<grid_for(J.nwork, 128), 128, 0, L.st>>>(in.oa, in.ob, J.order, J.tb_off, J.nwork, tb, d_edge,
                                                                d_delta, d_half, d_accept, in.path_off, in.paths,
                                                                in.path_len, c->d_err, rows, in.env, long_path[wv]);
    if (int e = rec.check(tb_long_join(L, forked))) return e;
    stage_mark(c, "path_compact");
    k_path_compact<<<grid_for((int64_t)J.nwork * 32, 256), 256, 0, L.st>>>(
        in.oa, in.ob, J.order, J.nwork, d_accept, in.path_off, in.paths, in.path_len);
    c->launches += 3;
    if (int e = rec.check(cudaGetLastError(), "kernel launch")) return e;
  }
  return rec.launch(&c->dp_exec[lane_id]);
}

// Ring-scheduled banded problems (gapdp_ring.cuh): rsel[w] is the group
// height R of ids[w].  Slots are ordered by R, each class most expensive
// first, and cut into waves that fit the traceback arena; per wave one
// k_gapdp_ring<R> launch per class, then traceback and path compaction.
static int run_ring(Ctx* c, const TbLanes& L, const DpInputs& in, const std::vector<uint32_t>& ids,
                    const std::vector<uint8_t>& rsel, const std::vector<int64_t>& la, const std::vector<int64_t>& lb,
                    const std::vector<int32_t>& dv, const std::vector<int32_t>& hv, const int32_t* d_delta,
                    const int32_t* d_half, uint8_t* d_accept, unsigned long long* d_cells) {
  const int64_t nwork = (int64_t)ids.size();
  if (nwork == 0) return 0;
  std::unique_ptr<HostSpan> span(new HostSpan(c, "ring_plan"));
  std::vector<uint64_t> bytes(nwork), cost(nwork);
  host_chunks(nwork, [&](int64_t w0, int64_t w1, int) {
    for (int64_t w = w0; w < w1; ++w) {
      const uint32_t p = ids[w];
      const RingBand b = make_ring_band((int)la[p], (int)lb[p], dv[p], hv[p], rsel[w]);
      bytes[w] = (ring_tb_words(b) * 4 + 255) & ~255ull;
      cost[w] = (uint64_t)b.steps * (uint64_t)(rsel[w] * 18 + 50);
    }
  });
  // by group height, each class most expensive first, ties in input order
  std::vector<uint32_t> idx;
  {
    constexpr uint64_t kMax = (1ull << 40) - 1;
    std::vector<uint64_t> key(nwork);
    for (int64_t w = 0; w < nwork; ++w) {
      int q = 0;
      while (q + 1 < kRingHeights && kRingRows[q] != rsel[w]) ++q;
      key[w] = ((uint64_t)q << 40) | (kMax - std::min(cost[w], kMax));
    }
    idx = radix_order(key);
  }
  uint64_t arena = c->tb_arena;
  {
    size_t free_b = 0, total_b = 0;
    HostSpan mem_span(c, "meminfo");
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
      const uint64_t cap = (uint64_t)((c->ws.size[67] + free_b) * 0.6);
      if (arena > cap) arena = cap;
    }
  }
  std::vector<uint32_t> order(nwork);
  std::vector<uint8_t> rows_of(nwork);
  std::vector<uint64_t> tboff(nwork);
  std::vector<int64_t> wave_begin;
  uint64_t acc = 0, arena_need = 0;
  for (int64_t q = 0; q < nwork; ++q) {
    const uint32_t w = idx[q];
    if (bytes[w] > arena) return report_error(MVG_ERR_CAPACITY, "one gap-DP problem exceeds the traceback arena");
    if (q == 0 || acc + bytes[w] > arena) {
      wave_begin.push_back(q);
      acc = 0;
    }
    order[q] = ids[w];
    rows_of[q] = rsel[w];
    tboff[q] = acc;
    acc += bytes[w];
    arena_need = std::max(arena_need, acc);
  }
  wave_begin.push_back(nwork);
  Workspace& ws = c->ws;
  uint32_t* d_order = (uint32_t*)ws.get(c, 64, (size_t)nwork * 4);
  uint64_t* d_tboff = (uint64_t*)ws.get(c, 65, (size_t)nwork * 8);
  uint8_t* d_edge = (uint8_t*)ws.get(c, 13, la.size() + 16);
  unsigned* d_counter = (unsigned*)ws.get(c, 66, 64 * kRingHeights);  // one claim counter per height
  uint8_t* d_rows = (uint8_t*)ws.get(c, 60, (size_t)nwork + 16);
  uint32_t* tb = (uint32_t*)ws.get(c, 67, arena_need);
  if (!d_order || !d_tboff || !d_edge || !d_counter || !d_rows || !tb)
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (int e = h2d_async(c, d_order, order.data(), (size_t)nwork * 4, L.st)) return e;
  if (int e = h2d_async(c, d_tboff, tboff.data(), (size_t)nwork * 8, L.st)) return e;
  if (int e = h2d_async(c, d_rows, rows_of.data(), (size_t)nwork, L.st)) return e;
  int dev_sms = 0;
  MVG_CUDA_TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  span.reset();
  for (size_t wv = 0; wv + 1 < wave_begin.size(); ++wv) {
    const int64_t w0 = wave_begin[wv], w1 = wave_begin[wv + 1];
    // heights of 16 rows and more run on the side stream beside the smaller
    // ones: their few long problems end in a latency-bound tail (one warp,
    // one problem) that would otherwise hold up the next launch
    bool side_used = false;
    for (int64_t a = w0; a < w1 && !side_used; ++a) side_used = rows_of[a] >= 16;
    if (side_used) {  // the side stream starts with the wave, not after the smaller heights
      MVG_CUDA_TRY(cudaEventRecord(L.fork, L.st));
      MVG_CUDA_TRY(cudaStreamWaitEvent(L.side, L.fork, 0));
    }
    for (int64_t a = w0; a < w1;) {
      int64_t e = a;
      while (e < w1 && rows_of[e] == rows_of[a]) ++e;
      const int R = rows_of[a];
      int hq = 0;
      while (hq + 1 < kRingHeights && kRingRows[hq] != R) ++hq;
      const bool side = R >= 16;
      const cudaStream_t ks = side ? L.side : L.st;
      unsigned* ctr = d_counter + 16 * hq;
      void (*kern)(RingJob) = ring_kernel(R);
      int bps = 0;
      MVG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, kRingThreads, 0));
      if (bps < 1) bps = 1;
      const int64_t need_blocks = (e - a + kRingThreads / 32 - 1) / (kRingThreads / 32);
      const int grid = (int)std::min<int64_t>((int64_t)dev_sms * bps, need_blocks);
      RingJob J;
      J.sa = in.sa;
      J.oa = in.oa;
      J.sb = in.sb;
      J.ob = in.ob;
      J.order = d_order + a;
      J.tb_off = d_tboff + a;
      J.nwork = (int)(e - a);
      J.tb = tb;
      J.scores = in.scores;
      J.end_edge = d_edge;
      J.band_delta = d_delta;
      J.band_half = d_half;
      J.accept = d_accept;
      J.base_max = g_base_max;
      J.counter = ctr;
      J.cells = d_cells;
      MVG_CUDA_TRY(cudaMemsetAsync(ctr, 0, 4, ks));
      kern<<<grid, kRingThreads, 0, ks>>>(J);
      c->launches++;
      a = e;
    }
    if (side_used) {
      MVG_CUDA_TRY(cudaEventRecord(L.join, L.side));
      MVG_CUDA_TRY(cudaStreamWaitEvent(L.st, L.join, 0));
    }
    const int nw = (int)(w1 - w0);
    std::vector<uint32_t> slot_len(w1 - w0);
    for (int64_t q = w0; q < w1; ++q) slot_len[q - w0] = (uint32_t)(la[order[q]] + lb[order[q]]);
    bool forked = false;
    int long_path = INT_MAX;
    int trc = tb_long_fork(c, L, in, slot_len, d_order + w0, d_tboff + w0, tb, d_edge, d_delta, d_half, d_accept, 0,
                           d_rows + w0, &long_path, &forked);
    if (trc) return trc;
    k_traceback_ring<<<grid_for(nw, 128), 128, 0, L.st>>>(
        in.oa, in.ob, d_order + w0, d_rows + w0, d_tboff + w0, nw, tb, d_edge, d_delta, d_half, d_accept,
        in.path_off, in.paths, in.path_len, c->d_err, long_path);
    if ((trc = tb_long_join(L, forked))) return trc;
    k_path_compact<<<grid_for((int64_t)nw * 32, 256), 256, 0, L.st>>>(in.oa, in.ob, d_order + w0, nw, d_accept,
                                                                            in.path_off, in.paths, in.path_len);
    c->launches += 2;
    MVG_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

// Whole-matrix problems with at least this many rows run in the full DP's
// launch (strips of 32 * dp_rows rows), shorter ones in the banded strip
// launch (32 * band_rows rows).

// Every base code must be 0..3 (the kernels mask to 2 bits; this reports it).
static int check_codes(Ctx* c, const uint8_t* d_sa, uint64_t na, const uint8_t* d_sb, uint64_t nb) {
  k_check_codes<<<grid_for(na / 16 + 1, 256), 256, 0, c->stream>>>(d_sa, na, c->d_err);
  k_check_codes<<<grid_for(nb / 16 + 1, 256), 256, 0, c->stream>>>(d_sb, nb, c->d_err);
  c->launches += 2;
  MVG_CUDA_TRY(cudaGetLastError());
  return 0;
}

static int check_lengths(int64_t nprob, const uint64_t* h_oa, const uint64_t* h_ob, std::vector<int64_t>& la,
                         std::vector<int64_t>& lb) {
  if (nprob >= (1ll << 31)) return report_error(MVG_ERR_ARG, "too many problems");
  la.resize(nprob);
  lb.resize(nprob);
  for (int64_t p = 0; p < nprob; ++p) {
    la[p] = (int64_t)(h_oa[p + 1] - h_oa[p]);
    lb[p] = (int64_t)(h_ob[p + 1] - h_ob[p]);
    if (la[p] <= 0 || lb[p] <= 0) return report_error(MVG_ERR_ARG, "gap-DP problem with an empty sequence");
    if (la[p] > 1000000 || lb[p] > 1000000) return report_error(MVG_ERR_ARG, "gap-DP problem longer than 1,000,000");
  }
  return 0;
}

// Scores-only calls still run the traceback (into a scratch path buffer) so
// every call exercises the same kernels.
static int scratch_paths(Ctx* c, int64_t nprob, const std::vector<int64_t>& la, const std::vector<int64_t>& lb,
                         DpInputs& in) {
  uint64_t tot = 0;
  std::vector<uint64_t> po(nprob + 1);
  for (int64_t p = 0; p < nprob; ++p) {
    po[p] = tot;
    tot += la[p] + lb[p];
  }
  po[nprob] = tot;
  char* d_tmp_paths = (char*)c->ws.get(c, 15, tot + 16);
  uint64_t* d_tmp_poff = (uint64_t*)c->ws.get(c, 16, (nprob + 1) * 8);
  int64_t* d_tmp_plen = (int64_t*)c->ws.get(c, 17, nprob * 8);
  if (!d_tmp_paths || !d_tmp_poff || !d_tmp_plen) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (int e = h2d_async(c, d_tmp_poff, po.data(), (nprob + 1) * 8, c->stream)) return e;
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  in.paths = d_tmp_paths;
  in.path_off = d_tmp_poff;
  in.path_len = d_tmp_plen;
  return 0;
}

int gapdp_batch_dev(Ctx* c, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb, const uint64_t* d_ob,
                    int64_t nprob, int32_t* d_scores, char* d_paths, const uint64_t* d_path_off, int64_t* d_path_len,
                    const uint64_t* h_oa, const uint64_t* h_ob, int32_t* d_env) {
  if (nprob <= 0) return 0;
  std::vector<int64_t> la, lb;
  int rc = check_lengths(nprob, h_oa, h_ob, la, lb);
  if (rc) return rc;
  if ((rc = stage_reserve(c, (size_t)nprob * 40 + (1 << 20)))) return rc;
  DpInputs in{d_sa, d_oa, d_sb, d_ob, d_scores, d_paths, d_path_off, d_path_len, d_env};
  if (!d_paths && (rc = scratch_paths(c, nprob, la, lb, in))) return rc;
  std::vector<uint32_t> ids(nprob);
  std::iota(ids.begin(), ids.end(), 0u);
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  if ((rc = check_codes(c, d_sa, h_oa[nprob], d_sb, h_ob[nprob]))) return rc;
  stage_begin_call(c);
  rc = run_dp(c, in, ids, la, lb, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  stage_end(c);
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return check_device_error(c);
}

int gapdp_banded_dev(Ctx* c, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb, const uint64_t* d_ob,
                     int64_t nprob, const int32_t* h_delta, const int32_t* h_half, int32_t* d_scores, char* d_paths,
                     const uint64_t* d_path_off, int64_t* d_path_len, uint8_t* h_used_band, const uint64_t* h_oa,
                     const uint64_t* h_ob, uint64_t* banded_cells) {
  if (nprob <= 0) return 0;
  stage_begin_call(c);
  std::unique_ptr<HostSpan> plan(new HostSpan(c, "plan"));
  std::vector<int64_t> la, lb;
  int rc = check_lengths(nprob, h_oa, h_ob, la, lb);
  if (rc) return rc;
  // staging: bands, and per launch group its order, offsets, heights and long-path lists
  if ((rc = stage_reserve(c, (size_t)nprob * 96 + (1 << 20)))) return rc;
  DpInputs in{d_sa, d_oa, d_sb, d_ob, d_scores, d_paths, d_path_off, d_path_len};
  if (!d_paths && (rc = scratch_paths(c, nprob, la, lb, in))) return rc;
  std::vector<int32_t> dv(h_delta, h_delta + nprob), hv(h_half, h_half + nprob);
  uint64_t bc = 0;
  // A band covering at least band_whole (default half) of its matrix saves
  // little and may still fail its check: such problems are not banded.  They
  // run in the strip kernel's launch with a band that covers the whole matrix
  // (no exit cells, so the check always passes and the result is the full
  // DP's; short strips suit these mostly small problems better than the full
  // DP's), which spares a second pass for them (status 2).  Other bands run
  // on the ring schedule with the smallest valid group height, or in the
  // strip kernel when no height is valid (or the ring kernel is switched off).
  std::vector<uint32_t> ids, rids, wids;
  std::vector<uint8_t> rsel;
  std::vector<uint8_t> whole(nprob, 0);
  // classified in chunks on host threads, each into its own lists, then
  // joined in chunk order (the same lists as one pass in order)
  struct Part {
    std::vector<uint32_t> ids, rids, wids;
    std::vector<uint8_t> rsel;
    uint64_t bc = 0;
    bool bad = false;
  };
  std::vector<Part> parts(16);
  const int nparts = host_chunks(nprob, [&](int64_t p0, int64_t p1, int t) {
    Part& P = parts[t];
    for (int64_t p = p0; p < p1; ++p) {
      if (hv[p] < 0) {
        P.bad = true;
        return;
      }
      const uint64_t full = (uint64_t)la[p] * (uint64_t)lb[p];
      bool is_whole;
      uint64_t cells = 0;
      if (c->band_ring) {
        // columns a row keeps: both half-widths, the row's own cells and
        // the diagonal's drift over one row
        const double cols = 2.0 * hv[p] + 2.0 + std::ceil((double)lb[p] / (double)la[p]);
        is_whole = cols >= c->band_whole * (double)lb[p];
      } else {
        cells = band_cells(make_band((int)la[p], (int)lb[p], dv[p], hv[p], 32 * c->band_rows));
        is_whole = (double)cells >= c->band_whole * (double)full;
      }
      if (is_whole) {
        whole[p] = 1;
        dv[p] = 0;
        hv[p] = (int32_t)std::max(la[p], lb[p]) + 2;
        P.bc += full;
        // long ones through the full DP's taller strips, short ones beside
        // the strip kernel's bands
        (la[p] >= c->whole_full_rows ? P.wids : P.ids).push_back((uint32_t)p);
        continue;
      }
      int rr = 0;
      if (c->band_ring) {
        // the lane-reuse condition W <= 32 + 32*R*LB/LA decides most
        // heights; only heights that pass it (with a column of slack) get
        // the exact test
        const double slope = (double)lb[p] / (double)la[p];
        for (int q = 0; q < kRingHeights && !rr; ++q) {
          const int R = kRingRows[q];
          if (R > c->ring_max_rows) break;  // taller groups go to the strip kernel
          const bool many = (la[p] + R - 1) / R > 32;
          if (many && 2.0 * hv[p] + 2.0 + (R - 1) * slope > 32.0 + 32.0 * R * slope + 2.0) continue;
          if (ring_eligible(make_ring_band((int)la[p], (int)lb[p], dv[p], hv[p], R))) rr = R;
        }
      }
      if (rr) {
        P.rids.push_back((uint32_t)p);
        P.rsel.push_back((uint8_t)rr);
      } else {
        if (c->band_ring) cells = band_cells(make_band((int)la[p], (int)lb[p], dv[p], hv[p], 32 * c->band_rows));
        P.bc += cells;
        P.ids.push_back((uint32_t)p);
      }
    }
  });
  for (int t = 0; t < nparts; ++t) {
    const Part& P = parts[t];
    if (P.bad) return report_error(MVG_ERR_ARG, "negative band half-width");
    ids.insert(ids.end(), P.ids.begin(), P.ids.end());
    rids.insert(rids.end(), P.rids.begin(), P.rids.end());
    wids.insert(wids.end(), P.wids.begin(), P.wids.end());
    rsel.insert(rsel.end(), P.rsel.begin(), P.rsel.end());
    bc += P.bc;
  }
  int32_t* d_delta = (int32_t*)c->ws.get(c, 23, (size_t)nprob * 4);
  int32_t* d_half = (int32_t*)c->ws.get(c, 25, (size_t)nprob * 4);
  uint8_t* d_accept = (uint8_t*)c->ws.get(c, 26, (size_t)nprob + 16);
  unsigned long long* d_cells = (unsigned long long*)c->ws.get(c, 61, 64);
  if (!d_delta || !d_half || !d_accept || !d_cells) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if ((rc = h2d_async(c, d_delta, dv.data(), (size_t)nprob * 4, c->stream))) return rc;
  if ((rc = h2d_async(c, d_half, hv.data(), (size_t)nprob * 4, c->stream))) return rc;
  MVG_CUDA_TRY(cudaMemsetAsync(d_accept, 0, (size_t)nprob, c->stream));
  MVG_CUDA_TRY(cudaMemsetAsync(d_cells, 0, 8, c->stream));
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  if ((rc = check_codes(c, d_sa, h_oa[nprob], d_sb, h_ob[nprob]))) return rc;
  plan.reset();
  // the ring-scheduled bands on the aux stream beside the strip kernel's
  // problems on the main stream (their launches have separate tails)
  const TbLanes ring_lanes{c->aux, c->aux2, c->fork2, c->join2, 68, 69};
  const TbLanes strip_lanes{c->stream, c->aux3, c->fork3, c->join3, 57, 58};
  const TbLanes band_lanes{c->aux4, c->aux5, c->fork5, c->join5, 54, 55};
  if (!rids.empty()) {
    MVG_CUDA_TRY(cudaEventRecord(c->fork, c->stream));
    MVG_CUDA_TRY(cudaStreamWaitEvent(c->aux, c->fork, 0));
    rc = run_ring(c, ring_lanes, in, rids, rsel, la, lb, dv, hv, d_delta, d_half, d_accept, d_cells);
    if (rc) return rc;
    MVG_CUDA_TRY(cudaEventRecord(c->join, c->aux));
  }
  // the strip kernel's problems on a third lane beside the long
  // whole-matrix problems' full DP on the main stream
  if (!ids.empty()) {
    MVG_CUDA_TRY(cudaEventRecord(c->fork4, c->stream));
    MVG_CUDA_TRY(cudaStreamWaitEvent(c->aux4, c->fork4, 0));
    rc = run_dp(c, in, ids, la, lb, d_delta, d_half, &dv, &hv, d_accept, &band_lanes, kDpSlotsLane2);
    if (rc) return rc;
    MVG_CUDA_TRY(cudaEventRecord(c->join4, c->aux4));
  }
  if (!wids.empty()) {
    rc = run_dp(c, in, wids, la, lb, nullptr, nullptr, nullptr, nullptr, nullptr, &strip_lanes);
    if (rc) return rc;
  }
  if (!ids.empty()) MVG_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join4, 0));
  if (!rids.empty()) MVG_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join, 0));
  stage_mark(c, "banded_done");
  std::vector<uint8_t> acc(nprob);
  MVG_CUDA_TRY(cudaMemcpyAsync(acc.data(), d_accept, (size_t)nprob, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, d_cells, 8, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  std::unique_ptr<HostSpan> tail(new HostSpan(c, "fallback_list"));
  bc += c->h_scalars[0];
  std::vector<uint32_t> fallback;
  for (int64_t p = 0; p < nprob; ++p) {
    if (whole[p]) {
      if (!acc[p] && la[p] < c->whole_full_rows)
        return report_error(MVG_ERR_DEVICE, "whole-matrix band failed its check");
      acc[p] = 2;  // not banded: the proposed band covered most of the matrix
    } else if (!acc[p]) {
      fallback.push_back((uint32_t)p);
      bc += (uint64_t)la[p] * (uint64_t)lb[p];
    }
  }
  tail.reset();
  // rejected bands: the full DP is both the fallback and the exact result
  rc = run_dp(c, in, fallback, la, lb, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  stage_end(c);
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (h_used_band) memcpy(h_used_band, acc.data(), (size_t)nprob);
  if (banded_cells) *banded_cells = bc;
  return check_device_error(c);
}

// --------------------------------------------------------- INT32 probe

// Eight independent add/max chains per thread; 2 ops per iteration per chain.
__global__ void k_int32_probe(int iters, int32_t seed, int32_t* sink) {
  int32_t x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = seed + q + threadIdx.x;
  const int32_t c1 = seed | 1, c2 = seed ^ 0x55;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      x[q] = x[q] + c1;
      x[q] = max(x[q], c2 - q);
    }
  }
  int32_t s = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s ^= x[q];
  if (s == 0x7fffffff) *sink = s;
}

int probe_int32_peak(Ctx* c, double* ops) {
  int sms = 0;
  MVG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  int32_t* sink = (int32_t*)c->ws.get(c, 19, 64);
  if (!sink) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  cudaEvent_t e0, e1;
  MVG_CUDA_TRY(cudaEventCreate(&e0));
  MVG_CUDA_TRY(cudaEventCreate(&e1));
  k_int32_probe<<<blocks, threads, 0, c->stream>>>(iters, 3, sink);  // warm-up
  MVG_CUDA_TRY(cudaEventRecord(e0, c->stream));
  k_int32_probe<<<blocks, threads, 0, c->stream>>>(iters, 7, sink);
  MVG_CUDA_TRY(cudaEventRecord(e1, c->stream));
  c->launches += 2;
  MVG_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  MVG_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double total = (double)blocks * threads * iters * 8 * 2;
  *ops = total / (ms * 1e-3);
  return 0;
}

}  // namespace mvg
