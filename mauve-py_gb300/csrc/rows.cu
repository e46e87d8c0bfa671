// Aligned rows from gap-DP paths: AlignTwoMSAsGivenPath (MU/aligngivenpath.cpp:256)
// for the single-sequence profiles of the pairwise path.  Each edge of a
// path is one column: 'M' takes the next character of both sequences, 'D'
// the next of A against a gap in B, 'I' a gap in A against the next of B;
// the gap character is '-' (MUSCLE's MSA gap).  The characters are copied
// as given (ASCII bases or 0..3 codes alike).
//
// One warp per problem: 32 edges per step, each lane's source positions from
// a ballot prefix of the edges before it.
#include "mvg_internal.h"

namespace mvg {

__global__ void k_path_rows(const uint8_t* __restrict__ sa, const uint64_t* __restrict__ oa,
                            const uint8_t* __restrict__ sb, const uint64_t* __restrict__ ob, int64_t nprob,
                            const char* __restrict__ paths, const uint64_t* __restrict__ path_off,
                            const int64_t* __restrict__ path_len, uint8_t* __restrict__ rows_a,
                            uint8_t* __restrict__ rows_b, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < nprob; p += nw) {
    const uint8_t* A = sa + oa[p];
    const uint8_t* B = sb + ob[p];
    const int64_t la = (int64_t)(oa[p + 1] - oa[p]), lb = (int64_t)(ob[p + 1] - ob[p]);
    const int64_t n = path_len[p];
    const char* P = paths + path_off[p];
    uint8_t* RA = rows_a + path_off[p];
    uint8_t* RB = rows_b + path_off[p];
    int64_t i = 0, j = 0;  // characters of A and B consumed before this step
    bool bad = false;
    for (int64_t t0 = 0; t0 < n; t0 += 32) {
      const int64_t t = t0 + lane;
      const char e = t < n ? P[t] : 'X';
      const bool ia = t < n && (e == 'M' || e == 'D');
      const bool ib = t < n && (e == 'M' || e == 'I');
      bad |= t < n && !ia && !ib;
      const unsigned ma = __ballot_sync(0xffffffffu, ia), mb = __ballot_sync(0xffffffffu, ib);
      const int64_t pa = i + __popc(ma & below), pb = j + __popc(mb & below);
      if (t < n) {
        bad |= (ia && pa >= la) || (ib && pb >= lb);
        RA[t] = ia ? (pa < la ? A[pa] : (uint8_t)'-') : (uint8_t)'-';
        RB[t] = ib ? (pb < lb ? B[pb] : (uint8_t)'-') : (uint8_t)'-';
      }
      i += __popc(ma);
      j += __popc(mb);
    }
    bad |= i != la || j != lb;  // the path must consume both sequences
    if (__any_sync(0xffffffffu, bad) && lane == 0) set_error(err, kDevRange);
  }
}

}  // namespace mvg

using namespace mvg;

static Ctx* rows_ctx(mvg_handle h) { return reinterpret_cast<Ctx*>(h); }

extern "C" int mvg_path_rows_dev(mvg_handle h, const uint8_t* d_seq_a, const uint64_t* d_off_a, const uint8_t* d_seq_b,
                                 const uint64_t* d_off_b, int64_t nprob, const char* d_paths,
                                 const uint64_t* d_path_off, const int64_t* d_path_len, uint8_t* d_rows_a,
                                 uint8_t* d_rows_b) {
  if (!h || nprob < 0 ||
      (nprob && (!d_seq_a || !d_off_a || !d_seq_b || !d_off_b || !d_paths || !d_path_off || !d_path_len ||
                 !d_rows_a || !d_rows_b)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  Ctx* c = rows_ctx(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  MVG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, 4, c->stream));
  const int grid = grid_for((uint64_t)nprob * 32, 256);
  k_path_rows<<<grid, 256, 0, c->stream>>>(d_seq_a, d_off_a, d_seq_b, d_off_b, nprob, d_paths, d_path_off,
                                           d_path_len, d_rows_a, d_rows_b, c->d_err);
  c->launches++;
  MVG_CUDA_TRY(cudaGetLastError());
  const int rc = check_device_error(c);
  if (rc == MVG_ERR_RANGE) return report_error(MVG_ERR_ARG, "a path does not consume exactly its two sequences");
  return rc;
}

extern "C" int mvg_path_rows(mvg_handle h, const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b,
                             const uint64_t* off_b, int64_t nprob, const char* paths, const uint64_t* path_off,
                             const int64_t* path_len, uint8_t* rows_a, uint8_t* rows_b) {
  if (!h || nprob < 0 ||
      (nprob && (!seq_a || !off_a || !seq_b || !off_b || !paths || !path_off || !path_len || !rows_a || !rows_b)))
    return report_error(MVG_ERR_ARG, "null argument");
  if (nprob == 0) return 0;
  Ctx* c = rows_ctx(h);
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  const uint64_t na = off_a[nprob], nb = off_b[nprob], np = path_off[nprob];
  Workspace& ws = c->ws;
  uint8_t* dsa = (uint8_t*)ws.get(c, 46, na + 16);
  uint8_t* dsb = (uint8_t*)ws.get(c, 47, nb + 16);
  uint64_t* doa = (uint64_t*)ws.get(c, 5, (nprob + 1) * 8);
  uint64_t* dob = (uint64_t*)ws.get(c, 6, (nprob + 1) * 8);
  char* dpa = (char*)ws.get(c, 9, np + 16);
  uint64_t* dpo = (uint64_t*)ws.get(c, 8, (nprob + 1) * 8);
  int64_t* dpl = (int64_t*)ws.get(c, 22, nprob * 8);
  uint8_t* dra = (uint8_t*)ws.get(c, 68, np + 16);
  uint8_t* drb = (uint8_t*)ws.get(c, 69, np + 16);
  if (!dsa || !dsb || !doa || !dob || !dpa || !dpo || !dpl || !dra || !drb)
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  MVG_CUDA_TRY(cudaMemcpyAsync(dsa, seq_a, na, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dsb, seq_b, nb, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(doa, off_a, (nprob + 1) * 8, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dob, off_b, (nprob + 1) * 8, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dpa, paths, np, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dpo, path_off, (nprob + 1) * 8, cudaMemcpyHostToDevice, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(dpl, path_len, nprob * 8, cudaMemcpyHostToDevice, c->stream));
  int rc = mvg_path_rows_dev(h, dsa, doa, dsb, dob, nprob, dpa, dpo, dpl, dra, drb);
  if (rc) return rc;
  MVG_CUDA_TRY(cudaMemcpyAsync(rows_a, dra, np, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaMemcpyAsync(rows_b, drb, np, cudaMemcpyDeviceToHost, c->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}
