// Band-proposal MLP for the gap DP: features, forward, backward and Adam.
//
// Input per gap (kIn = 528 after padding): the 4-mer spectra of both
// sequences (2 x 256, counts scaled to mean 1) and log(LA)/5, log(LB)/5.
// Network: 528 -> 256 -> 256 -> 256 -> 2, GELU (erf form) on the hidden
// layers, BF16 weights and activations feeding the tensor cores with FP32
// accumulation, FP32 master weights and Adam state.
// Outputs: [0] the band's diagonal offset / kDeltaScale, [1] log(1 + half).
//
// Forward hidden layers: tcgen05 tensor-core GEMMs fed by TMA with bias,
// GELU and (last layer) the 256 -> 2 output layer in the epilogue
// (mlp_tc.cuh).  Backward GEMMs, and the forward when the tcgen05 path is
// switched off or an operand does not meet its TMA rules: C[M x N] (fp32) =
// op(A)[M x K] * op(B)[K x N] with bf16 operands; a 64x64 block tile, four
// warps of 32x32 (2 x 4 mma.sync tiles), K step 32 staged in shared memory
// with both operands stored k-contiguous so every fragment is one 32-bit
// shared load.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "mvg_internal.h"

namespace mvg {

constexpr int kIn = 528, kHid = 256, kOut = 2;
constexpr float kDeltaScale = 100.0f;

// Flat parameter layout (fp32): W1 [kHid x kIn], b1, W2 [kHid x kHid], b2,
// W3 [kHid x kHid], b3, W4 [kOut x kHid], b4.
constexpr int64_t kOffW1 = 0;
constexpr int64_t kOffB1 = kOffW1 + (int64_t)kHid * kIn;
constexpr int64_t kOffW2 = kOffB1 + kHid;
constexpr int64_t kOffB2 = kOffW2 + (int64_t)kHid * kHid;
constexpr int64_t kOffW3 = kOffB2 + kHid;
constexpr int64_t kOffB3 = kOffW3 + (int64_t)kHid * kHid;
constexpr int64_t kOffW4 = kOffB3 + kHid;
constexpr int64_t kOffB4 = kOffW4 + (int64_t)kOut * kHid;
constexpr int64_t kNumParams = kOffB4 + kOut;
constexpr float kClipNorm = 1.0f;  // global gradient-norm clip of the Adam step

struct MlpState {
  float* w = nullptr;     // master weights
  float* g = nullptr;     // gradients
  float* m = nullptr;     // Adam first moment
  float* v = nullptr;     // Adam second moment
  __nv_bfloat16* wb = nullptr;  // bf16 copy of the weight matrices (same offsets)
  int64_t cap = 0;        // activation capacity (rows)
  float* z[3] = {};       // pre-activations
  __nv_bfloat16* h[3] = {};  // activations
  float* out = nullptr;   // [n x kOut]
  float* dh = nullptr;    // [n x kHid] fp32 upstream gradient
  float* dz32 = nullptr;  // [n x kHid] fp32 dZ (bias gradients)
  __nv_bfloat16* dz = nullptr;  // [n x kHid] bf16 dZ (GEMM operand)
  __nv_bfloat16* dout = nullptr;  // [n x kOut]
  float* dout32 = nullptr;
  float* loss = nullptr;
  bool ready = false;
};

// ---------------------------------------------------------------- GEMM

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// op(A)[m][k] = TA ? A[k * lda + m] : A[m * lda + k];  op(B)[k][n] = TB ? B[n * ldb + k] : B[k * ldb + n]
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ A, int lda,
                                                   const __nv_bfloat16* __restrict__ B, int ldb,
                                                   float* __restrict__ C, int ldc, int M, int N, int K) {
  constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;
  __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int wm = (wid >> 1) * 32, wn = (wid & 1) * 32;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[a][b][q] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += 128) {
      const int mm = e / BK, kk = e % BK;  // k fastest: coalesced when A is row-major
      const int gm = m0 + mm, gk = k0 + kk;
      As[mm][kk] = (gm < M && gk < K) ? (TA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk]) : zero;
    }
    for (int e = tid; e < BN * BK; e += 128) {
      int nn, kk;
      if (TB) {
        nn = e / BK;
        kk = e % BK;
      } else {
        kk = e / BN;
        nn = e % BN;
      }
      const int gn = n0 + nn, gk = k0 + kk;
      Bs[nn][kk] = (gn < N && gk < K) ? (TB ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn]) : zero;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int r = wm + a * 16 + g;
        af[a][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t]);
        af[a][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t]);
        af[a][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t + 8]);
        af[a][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int cidx = wn + b * 8 + g;
        bf[b][0] = *reinterpret_cast<const uint32_t*>(&Bs[cidx][kk + 2 * t]);
        bf[b][1] = *reinterpret_cast<const uint32_t*>(&Bs[cidx][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) mma_bf16(acc[a][b], af[a], bf[b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int r = m0 + wm + a * 16 + g, cc = n0 + wn + b * 8 + 2 * t;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int rr = r + (q >> 1) * 8, col = cc + (q & 1);
        if (rr < M && col < N) C[(int64_t)rr * ldc + col] = acc[a][b][q];
      }
    }
}

template <bool TA, bool TB>
static void gemm(cudaStream_t st, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc,
                 int M, int N, int K, uint64_t* launches) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  k_gemm_bf16<TA, TB><<<grid, 128, 0, st>>>(A, lda, B, ldb, C, ldc, M, N, K);
  ++*launches;
}

// ---------------------------------------------------------- elementwise

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

}  // namespace mvg

#include "mlp_tc.cuh"

namespace mvg {

__global__ void k_bias_gelu(float* __restrict__ z, const float* __restrict__ b, __nv_bfloat16* __restrict__ h,
                            int64_t n, int d) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * d; e += (int64_t)gridDim.x * blockDim.x) {
    const float v = z[e] + b[e % d];
    z[e] = v;
    h[e] = __float2bfloat16(gelu(v));
  }
}

__global__ void k_bias_add(float* __restrict__ z, const float* __restrict__ b, int64_t n, int d) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * d; e += (int64_t)gridDim.x * blockDim.x)
    z[e] += b[e % d];
}

// loss = mean over rows of sum_k (o - t)^2; dO = 2 (o - t) / n
__global__ void k_mse(const float* __restrict__ o, const float* __restrict__ tgt, int64_t n, float* __restrict__ d32,
                      __nv_bfloat16* __restrict__ d16, float* __restrict__ loss) {
  float s = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * kOut; e += (int64_t)gridDim.x * blockDim.x) {
    const float diff = o[e] - tgt[e];
    s += diff * diff;
    const float gd = 2.f * diff / (float)n;
    d32[e] = gd;
    d16[e] = __float2bfloat16(gd);
  }
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (float)n);
}

__global__ void k_gelu_back(const float* __restrict__ dh, const float* __restrict__ z, float* __restrict__ dz32,
                            __nv_bfloat16* __restrict__ dz, int64_t total) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const float v = dh[e] * gelu_grad(z[e]);
    dz32[e] = v;
    dz[e] = __float2bfloat16(v);
  }
}

// column sums of x [n x d] into out[d] (one block per column group)
__global__ void k_colsum(const float* __restrict__ x, int64_t n, int d, float* __restrict__ out) {
  const int col = blockIdx.x;
  float s = 0.f;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) s += x[r * d + col];
  for (int q = 16; q > 0; q >>= 1) s += __shfl_xor_sync(0xffffffffu, s, q);
  __shared__ float ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    out[col] = t;
  }
}

__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    y[e] = __float2bfloat16(x[e]);
}

// Sum of squares of the gradient into *sumsq (for norm clipping).
__global__ void k_sumsq(const float* __restrict__ g, int64_t n, float* __restrict__ sumsq) {
  float s = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    s += g[e] * g[e];
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) atomicAdd(sumsq, s);
}

// Adam on the gradient scaled to global norm <= clip; a step whose gradient
// norm is not finite leaves weights and moments untouched.
__global__ void k_adam(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, const float* __restrict__ sumsq, float clip) {
  const float ss = *sumsq;
  if (!isfinite(ss)) return;
  const float norm = sqrtf(ss);
  const float scale = norm > clip ? clip / norm : 1.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float ge = g[e] * scale;
    const float me = b1 * m[e] + (1.f - b1) * ge;
    const float ve = b2 * v[e] + (1.f - b2) * ge * ge;
    m[e] = me;
    v[e] = ve;
    const float we = w[e] - lr * (me / c1) / (sqrtf(ve / c2) + eps);
    w[e] = we;
    wb[e] = __float2bfloat16(we);
  }
}

// 4-mer spectra + log lengths, one warp per problem.
__global__ void __launch_bounds__(256) k_band_features(const uint8_t* __restrict__ sa, const uint64_t* __restrict__ oa,
                                                       const uint8_t* __restrict__ sb, const uint64_t* __restrict__ ob,
                                                       int64_t nprob, __nv_bfloat16* __restrict__ X) {
  __shared__ uint32_t hist[8][512];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < nprob;
       p += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    for (int q = lane; q < 512; q += 32) hist[wid][q] = 0;
    __syncwarp();
    const int64_t la = (int64_t)(oa[p + 1] - oa[p]), lb = (int64_t)(ob[p + 1] - ob[p]);
    for (int side = 0; side < 2; ++side) {
      const uint8_t* s = side ? sb + ob[p] : sa + oa[p];
      const int64_t L = side ? lb : la;
      for (int64_t i = lane; i + 3 < L; i += 32) {
        const uint32_t code = ((s[i] & 3u) << 6) | ((s[i + 1] & 3u) << 4) | ((s[i + 2] & 3u) << 2) | (s[i + 3] & 3u);
        atomicAdd(&hist[wid][side * 256 + code], 1u);
      }
    }
    __syncwarp();
    const float fa = la > 3 ? 256.f / (float)(la - 3) : 0.f, fb = lb > 3 ? 256.f / (float)(lb - 3) : 0.f;
    __nv_bfloat16* row = X + p * kIn;
    for (int q = lane; q < kIn; q += 32) {
      float v = 0.f;
      if (q < 256)
        v = hist[wid][q] * fa;
      else if (q < 512)
        v = hist[wid][q] * fb;
      else if (q == 512)
        v = logf((float)la) * 0.2f;
      else if (q == 513)
        v = logf((float)lb) * 0.2f;
      row[q] = __float2bfloat16(v);
    }
    __syncwarp();
  }
}

// Maps outputs to integer bands: delta = round(o0 * kDeltaScale),
// half = ceil(alpha * (exp(o1) - 1) + beta), clamped to [0, 1e6].
// Divergence gate: the share of up to 8 windows of 32 bases of A, spread
// along the diagonal j = i*LB/LA, whose best match count with B over the
// diagonal offsets -8..8 reaches `min_match` (one warp per gap; gaps
// shorter than one window score 1).  Closely related gaps keep nearly every
// window; gaps a band cannot help (divergent throughout) keep few.
constexpr int kGateWin = 8, kGateReach = 8;
__global__ void __launch_bounds__(256) k_band_gate(const uint8_t* __restrict__ sa, const uint64_t* __restrict__ oa,
                                                   const uint8_t* __restrict__ sb, const uint64_t* __restrict__ ob,
                                                   int64_t nprob, int min_match, float* __restrict__ share) {
  const int lane = threadIdx.x & 31;
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < nprob;
       p += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t la = (int64_t)(oa[p + 1] - oa[p]), lb = (int64_t)(ob[p + 1] - ob[p]);
    const uint8_t* A = sa + oa[p];
    const uint8_t* B = sb + ob[p];
    const int nwin = la < 32 ? 0 : (la / 32 < kGateWin ? (int)(la / 32) : kGateWin);
    int good = 0;
    for (int k = 0; k < nwin; ++k) {
      const int64_t i0 = nwin == 1 ? 0 : (int64_t)k * (la - 32) / (nwin - 1);
      const int64_t i = i0 + lane;
      const int64_t j = i * lb / la;
      const uint8_t a = A[i] & 3u;
      int best = 0;
#pragma unroll
      for (int o = -kGateReach; o <= kGateReach; ++o) {
        const int64_t jj = j + o;
        const bool m = jj >= 0 && jj < lb && (B[jj] & 3u) == a;
        best = max(best, __popc(__ballot_sync(0xffffffffu, m)));
      }
      good += best >= min_match;
    }
    if (lane == 0) share[p] = nwin ? (float)good / (float)nwin : 1.f;
  }
}

__global__ void k_to_band(const float* __restrict__ o, int64_t n, float alpha, float beta, int32_t* __restrict__ delta,
                          int32_t* __restrict__ half, const float* __restrict__ gate_share) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    // a non-finite output proposes the whole matrix (centred, half 1e6), and
    // so does a gap the divergence gate turns away (under half its windows
    // matched)
    const bool ok = isfinite(o[p * kOut]) && isfinite(o[p * kOut + 1]) && !(gate_share && gate_share[p] < 0.5f);
    const float d = ok ? rintf(o[p * kOut] * kDeltaScale) : 0.f;
    float h = ok ? ceilf(alpha * (expf(fminf(o[p * kOut + 1], 13.f)) - 1.f) + beta) : 1e6f;
    h = fminf(fmaxf(h, 0.f), 1e6f);
    delta[p] = (int32_t)fminf(fmaxf(d, -1e6f), 1e6f);
    half[p] = (int32_t)h;
  }
}

// ------------------------------------------------------------- driver

// Rows of an activation buffer: a multiple of 8, so the tensor maps' 8-row
// groups never reach past the allocation.
static int64_t rows8(int64_t n) { return (n + 7) & ~(int64_t)7; }

static int mlp_alloc(Ctx* c, MlpState& s, int64_t n) {
  if (!s.w) {
    if (cudaMalloc(&s.w, kNumParams * 4) != cudaSuccess || cudaMalloc(&s.g, kNumParams * 4) != cudaSuccess ||
        cudaMalloc(&s.m, kNumParams * 4) != cudaSuccess || cudaMalloc(&s.v, kNumParams * 4) != cudaSuccess ||
        cudaMalloc(&s.wb, kNumParams * 2) != cudaSuccess || cudaMalloc(&s.loss, 64) != cudaSuccess) {
      cudaGetLastError();
      return report_error(MVG_ERR_NOMEM, "MLP parameter allocation failed");
    }
    MVG_CUDA_TRY(cudaMemsetAsync(s.m, 0, kNumParams * 4, c->stream));
    MVG_CUDA_TRY(cudaMemsetAsync(s.v, 0, kNumParams * 4, c->stream));
  }
  if (n > s.cap) {
    for (int q = 0; q < 3; ++q) {
      cudaFree(s.z[q]);
      cudaFree(s.h[q]);
    }
    cudaFree(s.out);
    cudaFree(s.dh);
    cudaFree(s.dz32);
    cudaFree(s.dz);
    cudaFree(s.dout);
    cudaFree(s.dout32);
    bool ok = true;
    for (int q = 0; q < 3; ++q) {
      ok = ok && cudaMalloc(&s.z[q], n * kHid * 4) == cudaSuccess;
      ok = ok && cudaMalloc(&s.h[q], rows8(n) * kHid * 2) == cudaSuccess;
    }
    ok = ok && cudaMalloc(&s.out, n * kOut * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s.dh, n * kHid * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s.dz32, n * kHid * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s.dz, n * kHid * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&s.dout, n * kOut * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&s.dout32, n * kOut * 4) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      s.cap = 0;
      return report_error(MVG_ERR_NOMEM, "MLP activation allocation failed");
    }
    s.cap = n;
  }
  return 0;
}

static void mlp_free(MlpState& s) {
  cudaFree(s.w);
  cudaFree(s.g);
  cudaFree(s.m);
  cudaFree(s.v);
  cudaFree(s.wb);
  cudaFree(s.loss);
  for (int q = 0; q < 3; ++q) {
    cudaFree(s.z[q]);
    cudaFree(s.h[q]);
  }
  cudaFree(s.out);
  cudaFree(s.dh);
  cudaFree(s.dz32);
  cudaFree(s.dz);
  cudaFree(s.dout);
  cudaFree(s.dout32);
  s = MlpState();
}

static int eltwise_grid(int64_t n) { return grid_for((uint64_t)n, 256); }

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled encode_tiled() {
  static EncodeTiled fn = nullptr;
  static bool resolved = false;
  if (!resolved) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)f;
    resolved = true;
  }
  return fn;
}

// The 4-D view of a K-contiguous bf16 matrix described in mlp_tc.cuh: rows
// (a multiple of 8) x K (a multiple of 8), leading dimension ld elements.
// False when the driver entry point is missing or an operand breaks a TMA
// rule (16-byte aligned base, strides multiples of 16 bytes).
static bool tc_map(CUtensorMap* m, const __nv_bfloat16* p, int64_t rows, int K, int ld, int box_rows) {
  EncodeTiled enc = encode_tiled();
  if (!enc || rows <= 0 || rows % 8 || K % 8 || ld % 8 || ((uintptr_t)p & 15)) return false;
  const cuuint64_t dims[4] = {8, 8, (cuuint64_t)(K / 8), (cuuint64_t)(rows / 8)};
  const cuuint64_t strides[3] = {(cuuint64_t)ld * 2, 16, (cuuint64_t)ld * 16};
  const cuuint32_t box[4] = {8, 8, 8, (cuuint32_t)(box_rows / 8)};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)p, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Per device: the tcgen05 layer kernel's shared-memory opt-in has been set.
static bool tc_kernel_ready(int device) {
  static bool ready[64] = {};
  if (device < 0 || device >= 64) return false;
  if (!ready[device]) {
    if (cudaFuncSetAttribute(k_mlp_layer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem) !=
        cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    ready[device] = true;
  }
  return true;
}

// Forward pass into s.out.  X holds n rows of kIn features in an allocation
// of x_rows rows; train keeps the pre-activations and every activation for
// the backward pass.  The tcgen05 path runs when it is switched on and all
// six operands can be described to TMA (else the mma.sync GEMMs run).
static void mlp_forward(Ctx* c, MlpState& s, const __nv_bfloat16* X, int64_t n, int64_t x_rows, bool train) {
  cudaStream_t st = c->stream;
  const int nn = (int)n;
  if (c->mlp_tc && tc_kernel_ready(c->device)) {
    const int64_t offW[3] = {kOffW1, kOffW2, kOffW3};
    const int64_t offB[3] = {kOffB1, kOffB2, kOffB3};
    CUtensorMap ma[3], mw[3];
    bool ok = true;
    for (int q = 0; q < 3 && ok; ++q) {
      const int K = q == 0 ? kIn : kHid;
      const int64_t a_rows = q == 0 ? x_rows : rows8(n);
      ok = a_rows % 8 == 0 && tc_map(&ma[q], q == 0 ? X : s.h[q - 1], a_rows, K, K, kTcM) &&
           tc_map(&mw[q], s.wb + offW[q], kTcN, K, K, kTcN);
    }
    if (ok) {
      for (int q = 0; q < 3; ++q) {
        TcEpilogue ep;
        ep.bias = s.w + offB[q];
        ep.z = train ? s.z[q] : nullptr;
        ep.h = (train || q < 2) ? s.h[q] : nullptr;
        if (q == 2) {
          ep.w_out = s.wb + kOffW4;
          ep.b_out = s.w + kOffB4;
          ep.out = s.out;
        }
        k_mlp_layer_tc<<<(int)((n + kTcM - 1) / kTcM), kTcThreads, kTcSmem, st>>>(ma[q], mw[q], nn,
                                                                                   q == 0 ? kIn : kHid, ep, c->d_err);
      }
      c->launches += 3;
      ++c->mlp_tc_passes;
      return;
    }
  }
  gemm<false, true>(st, X, kIn, s.wb + kOffW1, kIn, s.z[0], kHid, nn, kHid, kIn, &c->launches);
  k_bias_gelu<<<eltwise_grid(n * kHid), 256, 0, st>>>(s.z[0], s.w + kOffB1, s.h[0], n, kHid);
  gemm<false, true>(st, s.h[0], kHid, s.wb + kOffW2, kHid, s.z[1], kHid, nn, kHid, kHid, &c->launches);
  k_bias_gelu<<<eltwise_grid(n * kHid), 256, 0, st>>>(s.z[1], s.w + kOffB2, s.h[1], n, kHid);
  gemm<false, true>(st, s.h[1], kHid, s.wb + kOffW3, kHid, s.z[2], kHid, nn, kHid, kHid, &c->launches);
  k_bias_gelu<<<eltwise_grid(n * kHid), 256, 0, st>>>(s.z[2], s.w + kOffB3, s.h[2], n, kHid);
  gemm<false, true>(st, s.h[2], kHid, s.wb + kOffW4, kHid, s.out, kOut, nn, kOut, kHid, &c->launches);
  k_bias_add<<<eltwise_grid(n * kOut), 256, 0, st>>>(s.out, s.w + kOffB4, n, kOut);
  c->launches += 4;
}

// Gradients of the mean-squared loss into s.g (overwritten), loss into s.loss.
static void mlp_backward(Ctx* c, MlpState& s, const __nv_bfloat16* X, const float* tgt, int64_t n) {
  cudaStream_t st = c->stream;
  const int nn = (int)n;
  cudaMemsetAsync(s.loss, 0, 4, st);
  k_mse<<<eltwise_grid(n * kOut), 256, 0, st>>>(s.out, tgt, n, s.dout32, s.dout, s.loss);
  // layer 4: dW4 = dO^T H3, db4 = sum dO, dH3 = dO W4
  gemm<true, false>(st, s.dout, kOut, s.h[2], kHid, s.g + kOffW4, kHid, kOut, kHid, nn, &c->launches);
  k_colsum<<<kOut, 256, 0, st>>>(s.dout32, n, kOut, s.g + kOffB4);
  gemm<false, false>(st, s.dout, kOut, s.wb + kOffW4, kHid, s.dh, kHid, nn, kHid, kOut, &c->launches);
  c->launches += 2;
  const int64_t offW[3] = {kOffW1, kOffW2, kOffW3};
  const int64_t offB[3] = {kOffB1, kOffB2, kOffB3};
  for (int q = 2; q >= 0; --q) {
    k_gelu_back<<<eltwise_grid(n * kHid), 256, 0, st>>>(s.dh, s.z[q], s.dz32, s.dz, n * kHid);
    k_colsum<<<kHid, 256, 0, st>>>(s.dz32, n, kHid, s.g + offB[q]);
    const __nv_bfloat16* in = q == 0 ? X : s.h[q - 1];
    const int din = q == 0 ? kIn : kHid;
    gemm<true, false>(st, s.dz, kHid, in, din, s.g + offW[q], din, kHid, din, nn, &c->launches);
    if (q > 0) gemm<false, false>(st, s.dz, kHid, s.wb + offW[q], kHid, s.dh, kHid, nn, kHid, kHid, &c->launches);
    c->launches += 2;
  }
}

}  // namespace mvg

using namespace mvg;

// One MLP per handle, kept beside it (the handle layout is internal to capi.cu).
#include <map>
#include <mutex>
static std::mutex g_mlp_mu;
static std::map<const void*, MlpState> g_mlps;

static MlpState& state_of(mvg_handle h) {
  std::lock_guard<std::mutex> lk(g_mlp_mu);
  return g_mlps[(const void*)h];
}

namespace mvg {
void mlp_release(const void* h) {
  std::lock_guard<std::mutex> lk(g_mlp_mu);
  auto it = g_mlps.find(h);
  if (it != g_mlps.end()) {
    mlp_free(it->second);
    g_mlps.erase(it);
  }
}
}  // namespace mvg

extern "C" {

int64_t mvg_mlp_num_params(void) { return kNumParams; }

int mvg_mlp_set_params(mvg_handle h, const float* params) {
  if (!h || !params) return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = reinterpret_cast<Ctx*>(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  MlpState& s = state_of(h);
  int rc = mlp_alloc(c, s, 0);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemcpyAsync(s.w, params, kNumParams * 4, cudaMemcpyHostToDevice, c->stream));
  k_to_bf16<<<grid_for(kNumParams, 256), 256, 0, c->stream>>>(s.w, s.wb, kNumParams);
  c->launches++;
  MVG_CUDA_TRY(cudaMemsetAsync(s.m, 0, kNumParams * 4, c->stream));
  MVG_CUDA_TRY(cudaMemsetAsync(s.v, 0, kNumParams * 4, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  s.ready = true;
  return 0;
}

int mvg_mlp_get_params(mvg_handle h, float* params) {
  if (!h || !params) return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = reinterpret_cast<Ctx*>(h);
  MlpState& s = state_of(h);
  if (!s.ready) return report_error(MVG_ERR_ARG, "MLP parameters not set");
  MVG_CUDA_TRY(cudaMemcpyAsync(params, s.w, kNumParams * 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int mvg_band_features_dev(mvg_handle h, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb,
                          const uint64_t* d_ob, int64_t nprob, void* d_x_bf16) {
  if (!h || nprob < 0 || (nprob && (!d_sa || !d_oa || !d_sb || !d_ob || !d_x_bf16)))
    return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (nprob == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  k_band_features<<<grid_for((uint64_t)nprob * 32, 256), 256, 0, c->stream>>>(d_sa, d_oa, d_sb, d_ob, nprob,
                                                                              (__nv_bfloat16*)d_x_bf16);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int mvg_mlp_forward_dev(mvg_handle h, const void* d_x_bf16, int64_t n, float* d_out) {
  if (!h || n < 0 || (n && (!d_x_bf16 || !d_out))) return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = reinterpret_cast<Ctx*>(h);
  MlpState& s = state_of(h);
  if (!s.ready) return report_error(MVG_ERR_ARG, "MLP parameters not set");
  if (n == 0) return 0;
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  int rc = mlp_alloc(c, s, n);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  mlp_forward(c, s, (const __nv_bfloat16*)d_x_bf16, n, n, false);
  MVG_CUDA_TRY(cudaMemcpyAsync(d_out, s.out, n * kOut * 4, cudaMemcpyDeviceToDevice, c->stream));
  MVG_CUDA_TRY(cudaGetLastError());
  return check_device_error(c);
}

int mvg_mlp_grad_dev(mvg_handle h, const void* d_x_bf16, const float* d_target, int64_t n, float* h_grads,
                     float* h_loss) {
  if (!h || n <= 0 || !d_x_bf16 || !d_target) return report_error(MVG_ERR_ARG, "null argument");
  Ctx* c = reinterpret_cast<Ctx*>(h);
  MlpState& s = state_of(h);
  if (!s.ready) return report_error(MVG_ERR_ARG, "MLP parameters not set");
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  int rc = mlp_alloc(c, s, n);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  mlp_forward(c, s, (const __nv_bfloat16*)d_x_bf16, n, n, true);
  mlp_backward(c, s, (const __nv_bfloat16*)d_x_bf16, d_target, n);
  if (h_grads) MVG_CUDA_TRY(cudaMemcpyAsync(h_grads, s.g, kNumParams * 4, cudaMemcpyDeviceToHost, c->stream));
  float loss = 0;
  MVG_CUDA_TRY(cudaMemcpyAsync(&loss, s.loss, 4, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaGetLastError());
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (h_loss) *h_loss = loss;
  return check_device_error(c);
}

int mvg_mlp_train_step_dev(mvg_handle h, const void* d_x_bf16, const float* d_target, int64_t n, float lr, int step,
                           float* h_loss) {
  if (!h || n <= 0 || !d_x_bf16 || !d_target || step < 1) return report_error(MVG_ERR_ARG, "bad argument");
  Ctx* c = reinterpret_cast<Ctx*>(h);
  MlpState& s = state_of(h);
  if (!s.ready) return report_error(MVG_ERR_ARG, "MLP parameters not set");
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  int rc = mlp_alloc(c, s, n);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  mlp_forward(c, s, (const __nv_bfloat16*)d_x_bf16, n, n, true);
  mlp_backward(c, s, (const __nv_bfloat16*)d_x_bf16, d_target, n);
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  MVG_CUDA_TRY(cudaMemsetAsync(s.loss + 1, 0, 4, c->stream));
  k_sumsq<<<grid_for(kNumParams, 256), 256, 0, c->stream>>>(s.g, kNumParams, s.loss + 1);
  k_adam<<<grid_for(kNumParams, 256), 256, 0, c->stream>>>(s.w, s.wb, s.g, s.m, s.v, kNumParams, lr, b1, b2, 1e-8f, c1,
                                                           c2, s.loss + 1, kClipNorm);
  c->launches += 2;
  if (h_loss) {
    float loss = 0;
    MVG_CUDA_TRY(cudaMemcpyAsync(&loss, s.loss, 4, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    *h_loss = loss;
  }
  MVG_CUDA_TRY(cudaGetLastError());
  return check_device_error(c);
}

int mvg_set_band_gate(mvg_handle h, int min_match) {
  if (!h || min_match < 0 || min_match > 32) return report_error(MVG_ERR_ARG, "min_match must be in 0..32");
  reinterpret_cast<Ctx*>(h)->band_gate = min_match;
  return 0;
}

int mvg_band_propose_dev(mvg_handle h, const uint8_t* d_sa, const uint64_t* d_oa, const uint8_t* d_sb,
                         const uint64_t* d_ob, int64_t nprob, float alpha, float beta, int32_t* h_delta,
                         int32_t* h_half) {
  if (!h || nprob < 0 || (nprob && (!h_delta || !h_half))) return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  MlpState& s = state_of(h);
  if (!s.ready) return report_error(MVG_ERR_ARG, "MLP parameters not set");
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  int rc = mlp_alloc(c, s, nprob);
  if (rc) return rc;
  __nv_bfloat16* X = (__nv_bfloat16*)c->ws.get(c, 27, (size_t)rows8(nprob) * kIn * 2);
  int32_t* dd = (int32_t*)c->ws.get(c, 28, (size_t)nprob * 8);
  if (!X || !dd) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  stage_mark(c, "band_features");
  k_band_features<<<grid_for((uint64_t)nprob * 32, 256), 256, 0, c->stream>>>(d_sa, d_oa, d_sb, d_ob, nprob, X);
  c->launches++;
  stage_mark(c, "mlp_forward");
  mlp_forward(c, s, X, nprob, rows8(nprob), false);
  float* gate = nullptr;
  if (c->band_gate > 0) {
    gate = (float*)c->ws.get(c, 59, (size_t)nprob * 4 + 16);
    if (!gate) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    k_band_gate<<<grid_for((uint64_t)nprob * 32, 256), 256, 0, c->stream>>>(d_sa, d_oa, d_sb, d_ob, nprob,
                                                                            c->band_gate, gate);
    c->launches++;
  }
  k_to_band<<<grid_for(nprob, 256), 256, 0, c->stream>>>(s.out, nprob, alpha, beta, dd, dd + nprob, gate);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  if ((rc = pinned_d2h(c, h_delta, dd, (size_t)nprob * 4))) return rc;
  if ((rc = pinned_d2h(c, h_half, dd + nprob, (size_t)nprob * 4))) return rc;
  return check_device_error(c);
}

int mvg_set_mlp_tcgen05(mvg_handle h, int on) {
  if (!h || (on != 0 && on != 1)) return report_error(MVG_ERR_ARG, "on must be 0 or 1");
  reinterpret_cast<Ctx*>(h)->mlp_tc = on;
  return 0;
}

int mvg_mlp_tcgen05_passes(mvg_handle h, uint64_t* passes) {
  if (!h || !passes) return report_error(MVG_ERR_ARG, "null argument");
  *passes = reinterpret_cast<Ctx*>(h)->mlp_tc_passes;
  return 0;
}

}  // extern "C"
