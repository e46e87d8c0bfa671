// Batched gap-alignment DP: muscle NWSmall (MU/nwsmall.cpp:500-670) for two
// single DNA sequences, in int32, bit-exact in score and traceback.
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
// Kernel layout (k_gapdp): one warp per problem, persistent warps pull
// problems (largest first) from a counter.  The DP matrix is cut into strips
// of 32*R rows; lane t owns rows [t*R, t*R+R) of the strip and sweeps the
// columns on an anti-diagonal wavefront (lane t is t columns behind lane 0).
// Each step a lane computes an R x 1 column segment; the cells above its
// segment arrive from lane t-1 by __shfl_up_sync, the row above the strip
// comes from a per-warp row buffer written by lane 31 of the previous strip.
// Traceback bits (MU/types.h:30-43: 2 bits M source, 1 bit D<-M, 1 bit I<-M)
// are packed 8 nibbles per word and stored lane-minor, so each flush is one
// coalesced 128-byte warp store.  k_traceback then walks each problem's bits
// from (LA, LB) like BitTraceBack (MU/bittraceback.cpp:138-210).
#include <algorithm>
#include <numeric>
#include <vector>

#include "mvg_internal.h"

namespace mvg {

constexpr int kRows = 4;                 // rows per lane (R)
constexpr int kStripRows = 32 * kRows;   // rows per strip
constexpr int32_t kNeg = -(1 << 29);
constexpr int32_t kGap = -200;           // half of gap open -400
constexpr int kDpThreads = 256;

enum : uint32_t { TB_MM = 0, TB_DM = 1, TB_IM = 2, TB_MD = 4, TB_MI = 8 };

// NUC_SP + 60 (range -65..160), packed: entry (a,b) = byte b of
// c_score_rows[a], stored with a +80 bias so every byte is in 15..240.
constexpr int kScoreBias = 80;
__constant__ uint32_t c_score_rows[4];

static bool score_rows_host(uint32_t* rows) {
  const int sp[4][4] = {{91, -114, -31, -123}, {-114, 100, -125, -31}, {-31, -125, 100, -114}, {-123, -31, -114, 91}};
  for (int a = 0; a < 4; ++a) {
    uint32_t r = 0;
    for (int b = 0; b < 4; ++b) {
      const int v = sp[a][b] + 60 + kScoreBias;
      if (v < 0 || v > 255) return false;
      r |= (uint32_t)v << (8 * b);
    }
    rows[a] = r;
  }
  return true;
}

int upload_score_table() {
  uint32_t rows[4];
  if (!score_rows_host(rows)) return report_error(MVG_ERR_ARG, "score table does not fit the packed byte layout");
  MVG_CUDA_TRY(cudaMemcpyToSymbol(c_score_rows, rows, sizeof(rows)));
  return 0;
}

struct DpJob {
  const uint8_t* sa;
  const uint64_t* oa;
  const uint8_t* sb;
  const uint64_t* ob;
  const uint32_t* order;   // problem ids of this wave, largest first
  const uint64_t* tb_off;  // byte offset of each wave slot's traceback bits
  int nwork;
  uint32_t* tb;
  int4* rowbuf;
  int64_t rowbuf_stride;  // int4 entries per warp
  int32_t* scores;
  uint8_t* end_edge;  // 'M','D','I' per problem
  unsigned* counter;
  uint32_t* err;
};

__device__ __forceinline__ int32_t score_ab(uint32_t row_a, uint32_t b) {
  return (int32_t)((row_a >> (8 * b)) & 255u) - kScoreBias;
}

__global__ void __launch_bounds__(kDpThreads, 2) k_gapdp(DpJob J) {
  // Per-warp shared rings: B codes (lane t at step s reads B[s - t]) and the
  // row above the strip (lane 0 at step s reads rowbuf[s + 1]).  Both are
  // filled one 32-step chunk ahead, so no load sits on a step's critical path.
  __shared__ uint8_t sB[kDpThreads / 32][128];
  __shared__ int4 sR[kDpThreads / 32][64];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int4* rowbuf = J.rowbuf + gw * J.rowbuf_stride;
  uint8_t* ringB = sB[wib];
  int4* ringR = sR[wib];
  for (;;) {
    int w = 0;
    if (lane == 0) w = (int)atomicAdd(J.counter, 1u);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= J.nwork) break;
    const uint32_t p = J.order[w];
    const uint64_t a0 = J.oa[p], b0 = J.ob[p];
    const int LA = (int)(J.oa[p + 1] - a0), LB = (int)(J.ob[p + 1] - b0);
    const uint8_t* A = J.sa + a0;
    const uint8_t* B = J.sb + b0;
    uint32_t* tb = J.tb + J.tb_off[w] / 4;
    const int S = LB + 31;                              // steps per strip
    const int wpl = (S * kRows + 7) / 8;                // TB words per lane per strip
    const int nstrips = (LA + kStripRows - 1) / kStripRows;
    const int end_strip = (LA - 1) / kStripRows;
    const int end_lane = ((LA - 1) % kStripRows) / kRows;
    const int end_r = (LA - 1) % kRows;
    uint32_t bad = 0;

    for (int k = 0; k < nstrips; ++k) {
      const int row0 = k * kStripRows;
      uint32_t arow[kRows];
      int32_t goA[kRows];
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        const int i = row0 + lane * kRows + r + 1;
        uint32_t ac = i <= LA ? A[i - 1] : 0u;
        bad |= ac;
        arow[r] = c_score_rows[ac & 3u];
        goA[r] = (i == 1) ? 0 : kGap;
      }
      // prime the rings: B[0..63], rowbuf[1..64]
      __syncwarp();
      ringB[lane] = lane < LB ? B[lane] : 0;
      ringB[32 + lane] = 32 + lane < LB ? B[32 + lane] : 0;
      if (k > 0) {
        ringR[(1 + lane) & 63] = 1 + lane <= LB ? rowbuf[1 + lane] : make_int4(kNeg, kNeg, kNeg, 0);
        ringR[(33 + lane) & 63] = 33 + lane <= LB ? rowbuf[33 + lane] : make_int4(kNeg, kNeg, kNeg, 0);
      }
      __syncwarp();
      // left state (column j-1) per row; column 0 = (NEG, 0, NEG)
      int32_t lM[kRows], lD[kRows], lI[kRows];
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        lM[r] = kNeg;
        lD[r] = 0;
        lI[r] = kNeg;
      }
      int32_t pubM = kNeg, pubD = 0, pubI = kNeg;  // bottom row, last computed column
      int32_t upM = kNeg, upD = kNeg, upI = kNeg;  // row above, current column
      int32_t dgM, dgD, dgI;                       // row above, previous column
      uint32_t acc = 0;
      uint32_t* tbs = tb + (int64_t)k * wpl * 32;
      for (int s = 0; s < S; ++s) {
        if ((s & 31) == 0 && s > 0) {
          // refill one chunk ahead: B[s+32 .. s+63], rowbuf[s+33 .. s+64]
          __syncwarp();
          const int xb = s + 32 + lane;
          ringB[xb & 127] = xb < LB ? B[xb] : 0;
          if (k > 0) {
            const int xr = s + 33 + lane;
            ringR[xr & 63] = xr <= LB ? rowbuf[xr] : make_int4(kNeg, kNeg, kNeg, 0);
          }
          __syncwarp();
        }
        const int j = s - lane + 1;
        const int32_t rM = __shfl_up_sync(0xffffffffu, pubM, 1);
        const int32_t rD = __shfl_up_sync(0xffffffffu, pubD, 1);
        const int32_t rI = __shfl_up_sync(0xffffffffu, pubI, 1);
        const uint32_t bc = ringB[(s - lane) & 127];
        dgM = upM;
        dgD = upD;
        dgI = upI;
        if (lane == 0) {
          if (k == 0) {  // row 0: M(0,j)=NEG, D(0,j)=NEG, I(0,j)=0 for j>=1
            upM = kNeg;
            upD = kNeg;
            upI = 0;
            if (s == 0) {  // column 0 of row 0: M(0,0)=0, D(0,0)=I(0,0)=NEG
              dgM = 0;
              dgD = kNeg;
              dgI = kNeg;
            }
          } else {
            const int4 v = ringR[(s + 1) & 63];
            upM = v.x;
            upD = v.y;
            upI = v.z;
            if (s == 0) {  // column 0 of a row >= 1: (NEG, 0, NEG)
              dgM = kNeg;
              dgD = 0;
              dgI = kNeg;
            }
          }
        } else {
          upM = rM;
          upD = rD;
          upI = rI;
        }
        uint32_t nibs = 0;
        if (j >= 1 && j <= LB) {
          bad |= bc;
          const int32_t goB = j == 1 ? 0 : kGap;
          int32_t cuM = upM, cuD = upD;               // (i-1, j)
          int32_t cdM = dgM, cdD = dgD, cdI = dgI;    // (i-1, j-1)
#pragma unroll
          for (int r = 0; r < kRows; ++r) {
            // D(i,j) from D(i-1,j) (strict >) or M(i-1,j) + open
            const int32_t MD = cuM + goA[r];
            const bool dd = cuD > MD;
            const int32_t D = dd ? cuD : MD;
            // I(i,j) from M(i,j-1) + open (>=) or I(i,j-1)
            const int32_t MI = lM[r] + goB;
            const bool mi = MI >= lI[r];
            const int32_t I = mi ? MI : lI[r];
            // M(i,j) = s + max(M, D + close, I + close) at (i-1,j-1), tie M > D > I
            const int32_t DM = cdD + kGap, IM = cdI + kGap;
            const int32_t DI = max(DM, IM);
            const int32_t best = max(cdM, DI);
            const uint32_t tm = cdM >= DI ? TB_MM : (DM >= IM ? TB_DM : TB_IM);
            int32_t M = score_ab(arow[r], bc & 3u) + best;
            uint32_t tmm = tm;
            if (LA == 1 && j == 1 && k == 0 && lane == 0 && r == 0) {
              // NWSmall's last-row special case (MU/nwsmall.cpp:616-624) with
              // LA == 1: open + close of position 0, close not zeroed.
              M = score_ab(arow[0], bc & 3u) + kGap;
              tmm = TB_DM;
            }
            nibs |= (tmm | (dd ? 0u : TB_MD) | (mi ? TB_MI : 0u)) << (4 * r);
            // the row below in this lane sees this row as "up" and the old left as "diag"
            cdM = lM[r];
            cdD = lD[r];
            cdI = lI[r];
            cuM = M;
            cuD = D;
            lM[r] = M;
            lD[r] = D;
            lI[r] = I;
            if (k == end_strip && lane == end_lane && r == end_r && j == LB) {
              int32_t sc = M;
              char e = 'M';
              if (D > sc) {
                sc = D;
                e = 'D';
              }
              if (I > sc) {
                sc = I;
                e = 'I';
              }
              J.scores[p] = sc;
              J.end_edge[p] = (uint8_t)e;
            }
          }
          pubM = lM[kRows - 1];
          pubD = lD[kRows - 1];
          pubI = lI[kRows - 1];
        } else if (j == 0) {
          pubM = kNeg;
          pubD = 0;
          pubI = kNeg;
        }
        if (lane == 31 && k + 1 < nstrips && j >= 0 && j <= LB) rowbuf[j] = make_int4(pubM, pubD, pubI, 0);
        // pack R nibbles per step; kRows == 4 -> one word every 2 steps
        acc |= nibs << (16 * (s & 1));
        if ((s & 1) || s == S - 1) {
          tbs[(s >> 1) * 32 + lane] = acc;
          acc = 0;
        }
      }
      __syncwarp();
    }
    if (bad > 3u) set_error(J.err, kDevBadBase);
  }
}

// BitTraceBack from (LA, LB); writes the path reversed at the end of the
// problem's path slot and its length.
__global__ void k_traceback(const uint64_t* __restrict__ oa, const uint64_t* __restrict__ ob,
                            const uint32_t* __restrict__ order, const uint64_t* __restrict__ tb_off, int nwork,
                            const uint32_t* __restrict__ tb, const uint8_t* __restrict__ end_edge,
                            const uint64_t* __restrict__ path_off, char* __restrict__ paths, int64_t* __restrict__ path_len,
                            uint32_t* err) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += gridDim.x * blockDim.x) {
    const uint32_t p = order[w];
    const int LA = (int)(oa[p + 1] - oa[p]), LB = (int)(ob[p + 1] - ob[p]);
    const uint32_t* T = tb + tb_off[w] / 4;
    const int S = LB + 31;
    const int wpl = (S * kRows + 7) / 8;
    char* out = paths + path_off[p] + (LA + LB);  // writes go backwards from here
    int pa = LA, pb = LB;
    char cur = (char)end_edge[p];
    int64_t n = 0;
    const int64_t limit = (int64_t)LA + LB;
    for (;;) {
      if (n >= limit) {
        set_error(err, kDevCapacity);
        break;
      }
      *(--out) = cur;
      ++n;
      uint32_t bits = 0;
      if (pa >= 1 && pb >= 1) {
        const int i0 = pa - 1;
        const int k = i0 / kStripRows, rem = i0 % kStripRows;
        const int t = rem / kRows, r = rem % kRows;
        const int s = pb - 1 + t;
        const int nib = s * kRows + r;
        bits = (T[(int64_t)k * wpl * 32 + (nib >> 3) * 32 + t] >> (4 * (nib & 7))) & 15u;
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
  }
}

// Moves each path from the tail of its slot to the head (warp per problem).
__global__ void k_path_compact(const uint64_t* __restrict__ oa, const uint64_t* __restrict__ ob,
                               const uint32_t* __restrict__ order, int nwork, const uint64_t* __restrict__ path_off,
                               char* paths, const int64_t* __restrict__ path_len) {
  const int lane = threadIdx.x & 31;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwork; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t p = order[w];
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

static uint64_t tb_bytes_for(int64_t la, int64_t lb) {
  const int64_t S = lb + 31;
  const int64_t wpl = (S * kRows + 7) / 8;
  const int64_t nstrips = (la + kStripRows - 1) / kStripRows;
  return (uint64_t)(nstrips * wpl * 32 * 4);
}

int gapdp_batch_dev(Ctx* c, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb, const uint64_t* d_ob,
                    int64_t nprob, int32_t* d_scores, char* d_paths, const uint64_t* d_path_off, int64_t* d_path_len,
                    const uint64_t* h_oa, const uint64_t* h_ob) {
  if (nprob <= 0) return 0;
  if (nprob >= (1ll << 31)) return report_error(MVG_ERR_ARG, "too many problems");
  std::vector<int64_t> la(nprob), lb(nprob);
  int64_t maxlb = 0;
  for (int64_t p = 0; p < nprob; ++p) {
    la[p] = (int64_t)(h_oa[p + 1] - h_oa[p]);
    lb[p] = (int64_t)(h_ob[p + 1] - h_ob[p]);
    if (la[p] <= 0 || lb[p] <= 0) return report_error(MVG_ERR_ARG, "gap-DP problem with an empty sequence");
    if (la[p] > 1000000 || lb[p] > 1000000) return report_error(MVG_ERR_ARG, "gap-DP problem longer than 1,000,000");
    maxlb = std::max(maxlb, lb[p]);
  }
  // largest problems first (longest-processing-time order)
  std::vector<uint32_t> ord(nprob);
  std::iota(ord.begin(), ord.end(), 0u);
  std::stable_sort(ord.begin(), ord.end(),
                   [&](uint32_t x, uint32_t y) { return la[x] * lb[x] > la[y] * lb[y]; });

  int dev_sms = 0;
  MVG_CUDA_TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  int bps = 0;
  MVG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_gapdp, kDpThreads, 0));
  if (bps < 1) bps = 1;
  const int grid = dev_sms * bps;
  const int64_t nwarps = (int64_t)grid * (kDpThreads / 32);
  Workspace& ws = c->ws;
  const int64_t rb_stride = maxlb + 2;
  int4* rowbuf = (int4*)ws.get(c, 10, (size_t)nwarps * rb_stride * sizeof(int4));
  uint32_t* d_order = (uint32_t*)ws.get(c, 11, (size_t)nprob * 4);
  uint64_t* d_tboff = (uint64_t*)ws.get(c, 12, (size_t)nprob * 8);
  uint8_t* d_edge = (uint8_t*)ws.get(c, 13, (size_t)nprob + 16);
  unsigned* d_counter = (unsigned*)ws.get(c, 14, 64);
  char* d_tmp_paths = nullptr;
  uint64_t* d_tmp_poff = nullptr;
  int64_t* d_tmp_plen = nullptr;
  if (!rowbuf || !d_order || !d_tboff || !d_edge || !d_counter) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (!d_paths) {  // scores only: traceback still runs so the bits are consumed identically
    uint64_t tot = 0;
    std::vector<uint64_t> po(nprob + 1);
    for (int64_t p = 0; p < nprob; ++p) {
      po[p] = tot;
      tot += la[p] + lb[p];
    }
    po[nprob] = tot;
    d_tmp_paths = (char*)ws.get(c, 15, tot + 16);
    d_tmp_poff = (uint64_t*)ws.get(c, 16, (nprob + 1) * 8);
    d_tmp_plen = (int64_t*)ws.get(c, 17, nprob * 8);
    if (!d_tmp_paths || !d_tmp_poff || !d_tmp_plen) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    MVG_CUDA_TRY(cudaMemcpyAsync(d_tmp_poff, po.data(), (nprob + 1) * 8, cudaMemcpyHostToDevice, c->stream));
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    d_paths = d_tmp_paths;
    d_path_off = d_tmp_poff;
    d_path_len = d_tmp_plen;
  }
  // Waves that fit the traceback arena.  Problems are dealt round-robin from
  // the size-sorted list, so every wave holds the same mix of sizes (enough
  // problems to fill every warp) and stays largest-first inside.
  uint64_t arena = c->tb_arena;
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
      size_t have = c->ws.size[18] + free_b;  // the arena slot itself may be re-allocated
      uint64_t cap = (uint64_t)(have * 0.6);
      if (arena > cap) arena = cap;
    }
  }
  std::vector<uint64_t> bytes(nprob);
  uint64_t total_tb = 0, max_tb = 0;
  for (int64_t w = 0; w < nprob; ++w) {
    bytes[w] = (tb_bytes_for(la[ord[w]], lb[ord[w]]) + 255) & ~255ull;
    total_tb += bytes[w];
    max_tb = std::max(max_tb, bytes[w]);
  }
  if (max_tb > arena) return report_error(MVG_ERR_CAPACITY, "one gap-DP problem exceeds the traceback arena");
  int64_t nwaves = (int64_t)((total_tb + arena - 1) / arena);
  std::vector<uint32_t> wave_ord;
  std::vector<uint64_t> tboff;
  std::vector<int64_t> wave_begin;
  uint64_t arena_need = 0;
  for (;;) {
    wave_ord.clear();
    tboff.clear();
    wave_begin.clear();
    arena_need = 0;
    bool fits = true;
    for (int64_t v = 0; v < nwaves && fits; ++v) {
      wave_begin.push_back((int64_t)wave_ord.size());
      uint64_t acc = 0;
      for (int64_t w = v; w < nprob; w += nwaves) {
        wave_ord.push_back(ord[w]);
        tboff.push_back(acc);
        acc += bytes[w];
      }
      if (acc > arena) fits = false;
      arena_need = std::max(arena_need, acc);
    }
    if (fits) break;
    ++nwaves;
  }
  wave_begin.push_back(nprob);
  ord.swap(wave_ord);
  uint32_t* tb = (uint32_t*)ws.get(c, 18, arena_need);
  if (!tb) return report_error(MVG_ERR_NOMEM, "traceback arena allocation failed");
  MVG_CUDA_TRY(cudaMemcpyAsync(d_order, ord.data(), (size_t)nprob * 4, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_tboff, tboff.data(), (size_t)nprob * 8, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  stage_begin_call(c);
  for (size_t wv = 0; wv + 1 < wave_begin.size(); ++wv) {
    const int64_t w0 = wave_begin[wv], w1 = wave_begin[wv + 1];
    DpJob J;
    J.sa = d_sa;
    J.oa = d_oa;
    J.sb = d_sb;
    J.ob = d_ob;
    J.order = d_order + w0;
    J.tb_off = d_tboff + w0;
    J.nwork = (int)(w1 - w0);
    J.tb = tb;
    J.rowbuf = rowbuf;
    J.rowbuf_stride = rb_stride;
    J.scores = d_scores;
    J.end_edge = d_edge;
    J.counter = d_counter;
    J.err = c->d_err;
    MVG_CUDA_TRY(cudaMemsetAsync(d_counter, 0, 4, c->stream));
    stage_mark(c, "dp");
    k_gapdp<<<grid, kDpThreads, 0, c->stream>>>(J);
    stage_mark(c, "traceback");
    k_traceback<<<grid_for(J.nwork, 128), 128, 0, c->stream>>>(d_oa, d_ob, J.order, J.tb_off, J.nwork, tb, d_edge,
                                                                d_path_off, d_paths, d_path_len, c->d_err);
    stage_mark(c, "path_compact");
    k_path_compact<<<grid_for((int64_t)J.nwork * 32, 256), 256, 0, c->stream>>>(d_oa, d_ob, J.order, J.nwork,
                                                                                 d_path_off, d_paths, d_path_len);
    c->launches += 3;
    MVG_CUDA_TRY(cudaGetLastError());
  }
  stage_end(c);
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
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
