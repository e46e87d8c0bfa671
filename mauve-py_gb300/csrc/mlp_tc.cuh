// One hidden layer of the band-proposal MLP on the 5th-generation tensor
// cores (included by mlp.cu after the GELU helpers):
//
//   Z = A W^T + b,  H = GELU(Z)   A [M x K] bf16, W [256 x K] bf16, fp32 accumulate
//
// and, for the last hidden layer, the 256 -> 2 output layer folded into the
// epilogue (out = H W4^T + b4, with H rounded to bf16 as the next GEMM's
// operand would be).
//
// A CTA of 128 threads owns 128 rows and all 256 columns: the accumulator
// is 128 TMEM lanes x 256 fp32 columns (tcgen05.alloc).  K moves in chunks
// of 64 through a two-stage shared-memory ring filled by TMA: thread 0
// issues the two tile loads of a stage (A 128 x 64, W 256 x 64, 48 KB) on
// the stage's "full" mbarrier; thread 32 waits for it, issues four
// tcgen05.mma.kind::f16 (M 128, N 256, K 16) and commits them to the
// stage's "empty" mbarrier, which frees the stage for the next load.  Two
// CTAs fit on an SM (96 KB of stages each, 512 TMEM columns in all), so one
// CTA's epilogue runs under the other's main loop.
//
// Shared-memory operand layout: 8 x 8 core matrices (8 rows of 16 bytes)
// without swizzle, K-major.  The tensor maps view a K-contiguous bf16
// matrix as 4-D (8 elements, 8 rows, K/8 groups, rows/8 groups), so one box
// (8, 8, 8, R/8) lands as [row group][k group][row][8 elements]: core
// matrices adjacent in K are 128 bytes apart (leading byte offset) and
// adjacent 8-row groups 1024 bytes apart (stride byte offset).  Rows past
// the matrix and K past its end read as zeros (TMA out-of-bounds fill).
//
// Every wait is bounded (about a second of %globaltimer); a wait that runs
// out sets the error word, the CTA skips its stores, waits (bounded) for
// the loads and MMAs it issued, frees its TMEM and returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include "mvg_common.cuh"

namespace mvg {

constexpr int kTcM = 128, kTcN = 256, kTcK = 64, kTcStages = 2, kTcThreads = 128;
constexpr uint32_t kTcBytesA = kTcM * kTcK * 2;  // 16 KB
constexpr uint32_t kTcBytesB = kTcN * kTcK * 2;  // 32 KB
constexpr uint32_t kTcStageBytes = kTcBytesA + kTcBytesB;
constexpr uint32_t kTcSmem = kTcStages * kTcStageBytes + 1024;  // + alignment slack
constexpr unsigned long long kTcWaitNs = 1ull << 30;

// Instruction descriptor of kind::f16: fp32 D (bits 4-5 = 1), bf16 A and B
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);

struct TcEpilogue {
  const float* bias = nullptr;          // [256]
  float* z = nullptr;                   // [M x 256] pre-activations, or null
  __nv_bfloat16* h = nullptr;           // [M x 256] activations, or null
  const __nv_bfloat16* w_out = nullptr; // [2 x 256] output layer folded in, or null
  const float* b_out = nullptr;         // [2]
  float* out = nullptr;                 // [M x 2]
};

// Shared-memory matrix descriptor: start address, leading byte offset,
// stride byte offset (all >> 4), descriptor version 1 (bit 46), base
// offset 0, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ uint64_t tc_now() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (it == 0)
      t0 = tc_now();
    else if (tc_now() - t0 > kTcWaitNs)
      return false;
  }
}

__device__ __forceinline__ void tc_load(uint32_t dst, const CUtensorMap* map, int kgroup, int rgroup, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(kgroup), "r"(rgroup), "r"(mbar)
      : "memory");
}

__global__ void __launch_bounds__(kTcThreads) k_mlp_layer_tc(const __grid_constant__ CUtensorMap map_a,
                                                             const __grid_constant__ CUtensorMap map_w, int M, int K,
                                                             TcEpilogue ep, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  __shared__ __align__(8) uint64_t s_full[kTcStages], s_empty[kTcStages], s_done;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail, s_issued, s_consumed;
  const uint32_t base = ((uint32_t)__cvta_generic_to_shared(tc_smem) + 1023u) & ~1023u;
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTcM;
  const int nk = (K + kTcK - 1) / kTcK;
  const uint32_t full0 = (uint32_t)__cvta_generic_to_shared(&s_full[0]);
  const uint32_t empty0 = (uint32_t)__cvta_generic_to_shared(&s_empty[0]);
  const uint32_t done = (uint32_t)__cvta_generic_to_shared(&s_done);
  if (tid == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full0 + 8 * s) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(empty0 + 8 * s) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(done) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
  }
  if (wid == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(&s_tmem)),
                 "r"((uint32_t)kTcN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = s_tmem;
  volatile int* fail = &s_fail;

  if (tid == 0) {  // TMA producer
    int i = 0;
    for (; i < nk; ++i) {
      const int s = i % kTcStages;
      if (i >= kTcStages && !tc_wait(empty0 + 8 * s, (uint32_t)((i / kTcStages) - 1) & 1u)) {
        *fail = 1;
        break;
      }
      if (*fail) break;
      const uint32_t sa = base + s * kTcStageBytes, sb = sa + kTcBytesA;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full0 + 8 * s),
                   "r"(kTcStageBytes)
                   : "memory");
      tc_load(sa, &map_a, i * (kTcK / 8), m0 / 8, full0 + 8 * s);
      tc_load(sb, &map_w, i * (kTcK / 8), 0, full0 + 8 * s);
    }
    s_issued = i;
  } else if (tid == 32) {  // MMA issuer
    int i = 0;
    for (; i < nk; ++i) {
      const int s = i % kTcStages;
      if (!tc_wait(full0 + 8 * s, (uint32_t)(i / kTcStages) & 1u)) {
        *fail = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t sa = base + s * kTcStageBytes, sb = sa + kTcBytesA;
#pragma unroll
      for (int kk = 0; kk < kTcK / 16; ++kk) {
        // a K step of 16 covers k groups 2 kk and 2 kk + 1: 256 bytes further along K
        const uint64_t da = tc_desc(sa + kk * 256, 128, 1024);
        const uint64_t db = tc_desc(sb + kk * 256, 128, 1024);
        const uint32_t acc = (i > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       empty0 + 8 * s)
                   : "memory");
    }
    s_consumed = i;
    // arrives once every MMA this thread issued has completed
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(done)
                 : "memory");
  }
  __syncwarp();
  if (!tc_wait(done, 0)) *fail = 1;
  __syncthreads();
  const bool ok = (*fail == 0);
  if (!ok && tid == 0) {
    set_error(err, kDevWatchdog);
    // loads issued but never consumed still land in shared memory: wait for them
    for (int i = s_consumed; i < s_issued; ++i) tc_wait(full0 + 8 * (i % kTcStages), (uint32_t)(i / kTcStages) & 1u);
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (ok) {
    // warp w reads TMEM lanes 32 w .. 32 w + 31: lane t holds row m0 + 32 w + t
    const int row = m0 + wid * 32 + lane;
    const bool live = row < M;
    float o0 = 0.f, o1 = 0.f;
#pragma unroll 1
    for (int c0 = 0; c0 < kTcN; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (!live) continue;
      float x[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) x[j] = __uint_as_float(v[j]) + __ldg(ep.bias + c0 + j);
      if (ep.z) {
        float4* dz = reinterpret_cast<float4*>(ep.z + (int64_t)row * kTcN + c0);
#pragma unroll
        for (int q = 0; q < 8; ++q) dz[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
      }
      uint32_t hb[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const __nv_bfloat162 pr = __floats2bfloat162_rn(gelu(x[2 * j]), gelu(x[2 * j + 1]));
        hb[j] = *reinterpret_cast<const uint32_t*>(&pr);
        if (ep.w_out) {
          const float2 hf = __bfloat1622float2(pr);
          const int cc = c0 + 2 * j;
          o0 += hf.x * __bfloat162float(ep.w_out[cc]) + hf.y * __bfloat162float(ep.w_out[cc + 1]);
          o1 += hf.x * __bfloat162float(ep.w_out[kTcN + cc]) + hf.y * __bfloat162float(ep.w_out[kTcN + cc + 1]);
        }
      }
      if (ep.h) {
        uint4* dh = reinterpret_cast<uint4*>(ep.h + (int64_t)row * kTcN + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q) dh[q] = make_uint4(hb[4 * q], hb[4 * q + 1], hb[4 * q + 2], hb[4 * q + 3]);
      }
    }
    if (ep.w_out && live) {
      ep.out[(int64_t)row * 2] = o0 + ep.b_out[0];
      ep.out[(int64_t)row * 2 + 1] = o1 + ep.b_out[1];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (wid == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"((uint32_t)kTcN)
                 : "memory");
}

}  // namespace mvg
