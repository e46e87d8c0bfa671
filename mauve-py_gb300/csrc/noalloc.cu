// Sorted-mer-list build that allocates nothing (mvg_sml_build_noalloc).
//
// Some callers cannot call cudaMalloc when they need a sorted mer list.
// Examples: a host process whose other runtime reserved the whole device for
// its own caching pool up front, or a latency-bound loop that cannot accept
// cudaMalloc's implicit device-wide synchronisation.  This entry point runs the same
// kernels as mvg_sml_build_dev, but its scratch lives in one file-scope
// device array of kNoAllocScratchBytes, which every GPU that loads this
// library holds until the process exits.  The caller still passes the input
// and output buffers.
//
// In host code the array's name is only a host-side stand-in, not a device
// address, so its device address is looked up once per device (and context),
// with that device current, through cudaGetSymbolAddress.  The first call on a
// device does this set-up (and uploads the 2-bit translation table), so that
// first call should come before any stream capture.  A call with n = 0 does
// the set-up alone.  Under CUDA's default lazy module loading the array's
// device memory is committed by that first look-up, not when the library is
// loaded: a caller that is about to hand the rest of the device to another
// allocator makes its first call (n = 0 is enough) before doing so.  The
// look-up is keyed on the current context's ID, so after cudaDeviceReset the
// next call repeats the set-up in the new context instead of using a stale
// address.  All calls share the one array and it keeps the previous call's
// contents: everything read is written first, except the error word, which
// every call clears.  Calls whose GPU work overlaps (two streams, or host
// threads) race on the array.
#include <cuda.h>

#include <mutex>

#include "mvg_internal.h"
#include "prim.cuh"

namespace mvg {

constexpr uint64_t kNoAllocMaxBases = 1ull << 18;  // 262,144 bases per call

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch layout: error word, packed bases, two key buffers (8-byte keys at
// most), two position buffers, radix-sort counters.
constexpr size_t kNaErr = 256;
constexpr size_t kNaPacked = ((kNoAllocMaxBases / 16 + 3) * 4 + 255) / 256 * 256;
constexpr size_t kNaKeys = kNoAllocMaxBases * 8;
constexpr size_t kNaVals = kNoAllocMaxBases * 4;
constexpr size_t kNaRadix =
    ((2 * 256 * ((kNoAllocMaxBases + kSortTile - 1) / kSortTile) + (256 * ((kNoAllocMaxBases + kSortTile - 1) / kSortTile) + kScanTile - 1) / kScanTile + 1 + 2) * 4 + 255) / 256 * 256;
constexpr size_t kNoAllocScratchBytes = kNaErr + kNaPacked + 2 * kNaKeys + 2 * kNaVals + kNaRadix;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_na_mu;
static uint8_t* g_na_addr[kMaxDevices] = {};
static unsigned long long g_na_ctx[kMaxDevices] = {};

// ID of the calling thread's current CUDA context (0 if none), read through
// the driver entry points the runtime exposes, so the library does not link
// the driver library itself.
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
    resolved = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Once per device and context, with that device current: translation table
// and the scratch array's device address.
static int noalloc_setup(int dev, uint8_t** out) {
  if (dev < 0 || dev >= kMaxDevices) return report_error(MVG_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_na_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_na_addr[dev] || ctx == 0 || ctx != g_na_ctx[dev]) {
    int rc = upload_base_table();
    if (rc) return rc;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return report_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_na_addr[dev] = (uint8_t*)p;
    g_na_ctx[dev] = current_context_id();  // the look-up made the primary context current
  }
  *out = g_na_addr[dev];
  return 0;
}

}  // namespace mvg

using namespace mvg;

extern "C" int mvg_sml_build_noalloc(const uint8_t* d_seq, uint64_t n, uint64_t seed, uint32_t* d_pos_out,
                                     uint64_t* d_mer_out, uint64_t cap, uint64_t* count, void* stream) {
  if (!count || (!d_seq && n)) return report_error(MVG_ERR_ARG, "null argument");
  const SeedDesc s = make_seed_desc(seed);
  if (s.L == 0 || s.L > 31) return report_error(MVG_ERR_ARG, "invalid seed pattern");
  if (n > kNoAllocMaxBases)
    return report_error(MVG_ERR_CAPACITY, "sequence longer than the no-allocation limit of 262,144 bases");
  const uint64_t cnt = n >= (uint64_t)s.L ? n - s.L + 1 : 0;
  *count = cnt;
  if (cnt > cap) return report_error(MVG_ERR_CAPACITY, "SML output buffer too small");
  int dev = 0;
  MVG_CUDA_TRY(cudaGetDevice(&dev));
  uint8_t* base = nullptr;
  int rc = noalloc_setup(dev, &base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t* d_err = (uint32_t*)base;
  uint32_t* packed = (uint32_t*)(base + kNaErr);
  uint8_t* k0 = base + kNaErr + kNaPacked;
  uint8_t* k1 = k0 + kNaKeys;
  uint32_t* v0 = (uint32_t*)(k1 + kNaKeys);
  uint32_t* v1 = (uint32_t*)((uint8_t*)v0 + kNaVals);
  uint32_t* scr = (uint32_t*)((uint8_t*)v1 + kNaVals);
  MVG_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st));
  uint64_t launches = 0;
  rc = sml_build_into(d_seq, n, cnt, s, packed, k0, k1, v0, v1, scr, d_pos_out, d_mer_out, st, d_err, &launches);
  if (rc) return rc;
  uint32_t herr = 0;
  MVG_CUDA_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  MVG_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr == kDevGapChar) return report_error(MVG_ERR_GAP_CHAR, "gap character '-' in genome sequence");
  if (herr) return report_error(MVG_ERR_DEVICE, "device kernel reported an error");
  return 0;
}
