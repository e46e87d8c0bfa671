// The sorted-mer-list cache file (.sslist) that progressiveMauve writes next
// to each input FASTA: FileSML::Create (LM/FileSML.cpp:401-459) writes the
// SMLHeader struct (LM/SortedMerList.h:48-63) as raw bytes, then the 2-bit
// packed sequence (translate32's words, binary_seq_len of them), then one
// uint32 position per SML entry in sorted order; FileSML::LoadFile2
// (LM/FileSML.cpp:120-195) reads it back and rejects a file that is short,
// of another format version, or truncated.
//
// The header is written member by member at the offsets of the C struct on
// the platforms the reference builds for (little-endian, natural alignment:
// 2352 bytes, pinned against the compiled struct by the tests).  Members the
// reference leaves uninitialised (word_size, little_endian, padding, the
// description after its first byte, the two pad words after the sequence)
// are written as the natural value or zero.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "mvg_internal.h"

namespace mvg {

namespace sslist {
constexpr size_t kHeaderBytes = 2352;
constexpr size_t kVersion = 0, kAlphaBits = 4, kSeed = 8, kSeedLength = 16, kSeedWeight = 20, kLength = 24,
                 kUniqueMers = 32, kWordSize = 36, kLittleEndian = 40, kId = 42, kCircular = 44, kTable = 45,
                 kDescription = 300;
constexpr uint32_t kFormatVersion = 5;  // DNAFileSML::FormatVersion (LM/DNAFileSML.h:59-62)
constexpr uint32_t kNoUniqueCount = 0xffffffffu;
}  // namespace sslist

template <typename T>
static void put(uint8_t* h, size_t off, T v) {
  memcpy(h + off, &v, sizeof(T));
}
template <typename T>
static T get(const uint8_t* h, size_t off) {
  T v;
  memcpy(&v, h + off, sizeof(T));
  return v;
}

// The translation table SortedMerList::BasicDNATable installs
// (LM/SortedMerList.cpp:29-47); 255 entries (UINT8_MAX) are stored.
static void basic_dna_table(uint8_t* t) {
  memset(t, 0, 256);
  for (const char* p = "cCbByY"; *p; ++p) t[(uint8_t)*p] = 1;
  for (const char* p = "gGsSkK"; *p; ++p) t[(uint8_t)*p] = 2;
  t[(uint8_t)'t'] = 3;
  t[(uint8_t)'T'] = 3;
}

static uint64_t sslist_words(uint64_t length) { return (length * 2 + 31) / 32 + 2; }

}  // namespace mvg

using namespace mvg;

extern "C" {

int mvg_sslist_write(mvg_handle handle, const uint8_t* seq, uint64_t n, uint64_t seed, const char* path) {
  if (!handle || !path || (!seq && n)) return report_error(MVG_ERR_ARG, "null argument");
  Ctx* h = reinterpret_cast<Ctx*>(handle);
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  const SeedDesc s = make_seed_desc(seed);
  if (s.L == 0 || s.L > 31) return report_error(MVG_ERR_ARG, "invalid seed pattern");
  if (n >= 0xffffffffull) return report_error(MVG_ERR_ARG, "sequence longer than 2^32-1");
  const uint64_t cnt = n >= (uint64_t)s.L ? n - s.L + 1 : 0;
  const uint64_t nwords = sslist_words(n);
  std::vector<uint32_t> pos(cnt), words(nwords, 0);
  uint8_t* d_seq = (uint8_t*)h->ws.get(h, 46, n + 16);
  uint32_t* d_pos = (uint32_t*)h->ws.get(h, 47, cnt * 4 + 16);
  if (!d_seq || !d_pos) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (n) MVG_CUDA_TRY(cudaMemcpyAsync(d_seq, seq, n, cudaMemcpyHostToDevice, h->stream));
  uint64_t got = 0;
  int rc = mvg_sml_build_dev(handle, d_seq, n, seed, d_pos, nullptr, cnt, &got);
  if (rc) return rc;
  // the packed words the build left in its workspace (packed_words(n) of
  // them: the sequence words and the two pad words)
  const uint32_t* d_words = (const uint32_t*)h->ws.ptr[20];
  if (cnt) MVG_CUDA_TRY(cudaMemcpyAsync(pos.data(), d_pos, cnt * 4, cudaMemcpyDeviceToHost, h->stream));
  if (n) MVG_CUDA_TRY(cudaMemcpyAsync(words.data(), d_words, (nwords - 2) * 4, cudaMemcpyDeviceToHost, h->stream));
  MVG_CUDA_TRY(cudaStreamSynchronize(h->stream));

  uint8_t hdr[sslist::kHeaderBytes];
  memset(hdr, 0, sizeof(hdr));
  put<uint32_t>(hdr, sslist::kVersion, sslist::kFormatVersion);
  put<uint32_t>(hdr, sslist::kAlphaBits, 2u);
  put<uint64_t>(hdr, sslist::kSeed, seed);
  put<uint32_t>(hdr, sslist::kSeedLength, (uint32_t)s.L);
  put<uint32_t>(hdr, sslist::kSeedWeight, (uint32_t)s.w);
  put<uint64_t>(hdr, sslist::kLength, n);
  put<uint32_t>(hdr, sslist::kUniqueMers, sslist::kNoUniqueCount);
  put<uint32_t>(hdr, sslist::kWordSize, 32u);
  put<uint8_t>(hdr, sslist::kLittleEndian, 1u);
  put<int16_t>(hdr, sslist::kId, (int16_t)0);
  put<uint8_t>(hdr, sslist::kCircular, 0u);
  uint8_t table[256];
  basic_dna_table(table);
  memcpy(hdr + sslist::kTable, table, 255);

  FILE* f = fopen(path, "wb");
  if (!f) return report_error(MVG_ERR_ARG, "cannot open the .sslist file for writing");
  bool ok = fwrite(hdr, 1, sizeof(hdr), f) == sizeof(hdr);
  ok = ok && fwrite(words.data(), 4, nwords, f) == nwords;
  ok = ok && (cnt == 0 || fwrite(pos.data(), 4, cnt, f) == cnt);
  ok = (fclose(f) == 0) && ok;
  if (!ok) return report_error(MVG_ERR_ARG, "error writing the .sslist file");
  return 0;
}

int mvg_sslist_read(const char* path, mvg_sslist_info* info, uint32_t* words, uint64_t cap_words, uint32_t* pos,
                    uint64_t cap_pos) {
  if (!path || !info) return report_error(MVG_ERR_ARG, "null argument");
  memset(info, 0, sizeof(*info));
  FILE* f = fopen(path, "rb");
  if (!f) {
    info->status = 1;
    return report_error(MVG_ERR_ARG, "cannot open the .sslist file");
  }
  uint8_t hdr[sslist::kHeaderBytes];
  const bool have_header = fread(hdr, 1, sizeof(hdr), f) == sizeof(hdr);
  auto fail = [&](int status, const char* msg) {
    fclose(f);
    info->status = status;
    return report_error(MVG_ERR_ARG, msg);
  };
  if (!have_header) return fail(2, "short .sslist header");
  if (get<uint32_t>(hdr, sslist::kVersion) != sslist::kFormatVersion) return fail(3, "unsupported .sslist version");
  info->seed = get<uint64_t>(hdr, sslist::kSeed);
  info->seed_length = get<uint32_t>(hdr, sslist::kSeedLength);
  info->seed_weight = get<uint32_t>(hdr, sslist::kSeedWeight);
  info->length = get<uint64_t>(hdr, sslist::kLength);
  info->circular = get<uint8_t>(hdr, sslist::kCircular) ? 1 : 0;
  const uint32_t abits = get<uint32_t>(hdr, sslist::kAlphaBits);
  uint64_t seq_len = info->length + (info->circular ? info->seed_length - 1 : 0);
  const uint64_t nwords = (seq_len * abits) / 32 + (((seq_len * abits) % 32) ? 1 : 0) + 2;
  info->words = nwords;
  // entries: everything after the sequence, one uint32 each
  if (fseek(f, 0, SEEK_END) != 0) return fail(5, "cannot size the .sslist file");
  const long end = ftell(f);
  const uint64_t seq_end = sizeof(hdr) + nwords * 4;
  if (end < 0 || (uint64_t)end < seq_end) return fail(4, "truncated .sslist sequence");
  info->entries = ((uint64_t)end - seq_end) / 4;
  if (words) {
    if (cap_words < nwords) return fail(0, ".sslist word buffer too small");
    if (fseek(f, (long)sizeof(hdr), SEEK_SET) != 0 || fread(words, 4, nwords, f) != nwords)
      return fail(4, "error reading the .sslist sequence");
  }
  if (pos) {
    if (cap_pos < info->entries) return fail(0, ".sslist position buffer too small");
    if (fseek(f, (long)seq_end, SEEK_SET) != 0 ||
        (info->entries && fread(pos, 4, info->entries, f) != info->entries))
      return fail(5, "error reading the .sslist positions");
  }
  fclose(f);
  return 0;
}

}  // extern "C"
