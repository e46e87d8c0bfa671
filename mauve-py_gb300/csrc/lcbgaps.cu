// The search outside the LCBs for two genomes: SearchLCBGaps
// (LM/Aligner.cpp:784-928) as ProgressiveAligner::alignPP issues it after a
// recursion round (LM/ProgressiveAligner.cpp:2474-2488).
//
// Every region of a genome that lies outside the LCBs (the flanks
// recurseOnPairs collects, :784-834) is cut out and the cuts are
// concatenated, one sequence per genome.  The two concatenations are
// searched on the GPU by the pairwise matcher with the rank-0 seed of
// getDefaultSeedWeight of their mean length (MaskedMemHash without a mask
// hashes exactly the pairs PairwiseMatchFinder does for two genomes).  The
// matches then go back to genome coordinates on the host, in the reference's
// order of operations: MultiplicityFilter(2), transposeMatches for each
// genome (:973-1045; a match that runs over the seam between two regions is
// split there), EliminateOverlaps (:62-176), MultiplicityFilter(2) and
// LengthFilter(MIN_ANCHOR_LENGTH = 9).
//
// The host steps sort with std::sort under comparators that order exactly
// as the reference's (MatchLeftEndComparator, :937-966; SingleStartComparator,
// LM/AbstractMatch.h:324-351).  std::sort is not stable, so ties keep the
// order the same algorithm gives the same input, which is why the match
// list goes through the same sequence of sorts, crops and compactions as
// the reference's MatchList.  A match is a libMems two-sequence Match
// (LM/HybridAbstractMatch.h:151-290): a signed 1-based start per genome
// (negative = reverse strand, 0 = not in that genome) and one length;
// CropStart moves the forward starts, CropEnd the reverse ones
// (LM/UngappedLocalAlignment.h:138-152).
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "mauve_gb300.h"
#include "mvg_internal.h"

namespace mvg {
namespace {

constexpr int64_t kMinAnchorLength = 9;  // MIN_ANCHOR_LENGTH (LM/Aligner.h:266)
constexpr unsigned kMinSeedWeight = 5;   // MIN_DNA_SEED_WEIGHT (LM/SeedMasks.h:375)
constexpr uint32_t kNoSeq = 0xffffffffu;

struct Am {
  int64_t s[2];
  int64_t len;
  bool live;
  uint32_t first() const { return s[0] ? 0u : (s[1] ? 1u : kNoSeq); }
  unsigned mult() const { return (s[0] != 0) + (s[1] != 0); }
  // CropStart / CropEnd; false where the reference throws (crop past the end)
  bool crop_start(int64_t k) {
    if (k < 0 || k > len) return false;
    len -= k;
    for (int q = 0; q < 2; ++q)
      if (s[q] > 0) s[q] += k;
    return true;
  }
  bool crop_end(int64_t k) {
    if (k < 0 || k > len) return false;
    len -= k;
    for (int q = 0; q < 2; ++q)
      if (s[q] < 0) s[q] -= k;
    return true;
  }
};

int64_t absv(int64_t v) { return v < 0 ? -v : v; }

// MatchLeftEndComparator(seq): the first defined sequence (no lower than
// seq) first, then the left ends from seq on, skipping undefined or equal
// ones.
struct LeftEndOrder {
  uint32_t q;
  bool operator()(const Am& a, const Am& b) const {
    const int32_t start_diff = (int32_t)(std::max(a.first(), q) - std::max(b.first(), q));
    if (start_diff == 0) {
      for (uint32_t k = q; k < 2; ++k) {
        const int64_t as = absv(a.s[k]), bs = absv(b.s[k]);
        if (as == 0 || bs == 0 || as == bs) continue;
        return as < bs;
      }
    }
    return start_diff < 0;
  }
};

// SingleStartComparator(seq): undefined before defined, then by left end.
struct SingleStartOrder {
  int q;
  bool operator()(const Am& a, const Am& b) const {
    const int64_t as = absv(a.s[q]), bs = absv(b.s[q]);
    if (as == 0 || bs == 0) return bs != 0;
    return as < bs;
  }
};

// transposeMatches: concatenation coordinates of sequence q back to the
// genome, splitting at region seams.  regions: (left end, right end + 1)
// pairs, 1-based, in concatenation order.
int transpose(std::vector<Am>& ml, uint32_t q, const int64_t* reg, uint64_t nreg) {
  if (nreg < 2) return 0;
  std::sort(ml.begin(), ml.end(), LeftEndOrder{q});
  uint64_t ri = 0;
  int64_t rsum = reg[1] - reg[0], rstart = 0;
  std::vector<Am> pieces;
  for (size_t i = 0; i < ml.size(); ++i) {
    int64_t ts = ml[i].s[q];
    int64_t orig = ts;
    if (ts == 0) continue;
    while (rsum < absv(ts) && ri + 2 < nreg) {
      ri += 2;
      rstart = rsum;
      rsum += reg[ri + 1] - reg[ri];
    }
    if (ts < 0)
      ts = -reg[ri] - (-ts - rstart) + 1;
    else
      ts = reg[ri] + (ts - rstart) - 1;
    const int64_t te = orig > 0 ? orig + ml[i].len - 1 : orig - ml[i].len + 1;
    ml[i].s[q] = ts;
    int64_t esum = rsum;
    uint64_t eri = ri;
    // the piece still to split: ml[i] first, then the last piece made
    Am* cur = &ml[i];
    while (esum < absv(te) && eri + 2 < nreg) {
      eri += 2;
      Am left = *cur;
      const int64_t cut = absv(orig) + left.len - esum - 1;
      bool ok;
      if (left.s[q] < 0) {
        ok = cur->crop_start(cut) && left.crop_end(cur->len);
      } else {
        ok = cur->crop_end(cut) && left.crop_start(cur->len);
      }
      if (!ok) return report_error(MVG_ERR_ARG, "match crosses a region seam past its end");
      orig += orig > 0 ? cur->len : -cur->len;
      if (ts < 0)
        ts = -reg[eri] - (-orig - esum) + 1;
      else if (ts > 0)
        ts = reg[eri] + (orig - esum) - 1;
      left.s[q] = ts;
      pieces.push_back(left);
      cur = &pieces.back();
      esum += reg[eri + 1] - reg[eri];
    }
  }
  ml.insert(ml.end(), pieces.begin(), pieces.end());
  return 0;
}

// EliminateOverlaps for two-genome matches: per genome, sort by left end and
// crop (or drop) the smaller of each overlapping pair.  The overlapping part
// the reference copies out keeps only the other genome, so with two genomes
// it is always discarded (multiplicity 1).
int eliminate_overlaps(std::vector<Am>& ml) {
  if (ml.size() < 2) return 0;
  for (int q = 0; q < 2; ++q) {
    std::sort(ml.begin(), ml.end(), SingleStartOrder{q});
    const int64_t n = (int64_t)ml.size();
    int64_t i = 0, deleted = 0;
    for (; i != n; ++i)
      if (ml[i].s[q] != 0) break;
    for (; i < n; ++i) {
      if (!ml[i].live) continue;
      for (int64_t j = i + 1; j < n; ++j) {
        if (!ml[j].live) continue;
        bool deleted_i = false;
        const int64_t si = ml[i].s[q], li = ml[i].len, sj = ml[j].s[q];
        int64_t diff = absv(sj) - absv(si) - li;
        if (diff >= 0) break;  // no more overlaps
        diff = -diff;
        bool ok = true;
        if (ml[j].mult() > ml[i].mult() || (ml[j].mult() == ml[i].mult() && ml[j].len > ml[i].len)) {
          if (diff >= li) {
            ml[i].live = false;
            --i;
            deleted_i = true;
            ++deleted;
          } else {
            ok = si > 0 ? ml[i].crop_end(diff) : ml[i].crop_start(diff);
          }
        } else {
          if (diff >= ml[j].len) {
            ml[j].live = false;
            ++deleted;
          } else {
            ok = sj > 0 ? ml[j].crop_start(diff) : ml[j].crop_end(diff);
          }
        }
        if (!ok) return report_error(MVG_ERR_ARG, "overlap crop past the match");
        if (deleted_i) break;
      }
    }
    if (deleted > 0) ml.erase(std::remove_if(ml.begin(), ml.end(), [](const Am& m) { return !m.live; }), ml.end());
  }
  return 0;
}

void keep_if(std::vector<Am>& ml, bool (*pred)(const Am&)) {
  ml.erase(std::remove_if(ml.begin(), ml.end(), [pred](const Am& m) { return !pred(m); }), ml.end());
}

void load(std::vector<Am>& ml, const int64_t* m, uint64_t n) {
  ml.resize(n);
  for (uint64_t i = 0; i < n; ++i) ml[i] = Am{{m[3 * i], m[3 * i + 1]}, m[3 * i + 2], true};
}

int store(const std::vector<Am>& ml, int64_t* out, uint64_t cap, uint64_t* count) {
  *count = ml.size();
  if (ml.size() > cap) return report_error(MVG_ERR_CAPACITY, "match output buffer too small");
  for (size_t i = 0; i < ml.size(); ++i) {
    out[3 * i] = ml[i].s[0];
    out[3 * i + 1] = ml[i].s[1];
    out[3 * i + 2] = ml[i].len;
  }
  return 0;
}

int check_matches(const int64_t* m, uint64_t n) {
  if (n && !m) return report_error(MVG_ERR_ARG, "null argument");
  for (uint64_t i = 0; i < n; ++i)
    if (m[3 * i + 2] < 0) return report_error(MVG_ERR_ARG, "negative match length");
  return 0;
}

// Regions: an even number of 1-based boundaries, each pair (l, r) with
// 1 <= l <= r <= n + 1 (the bases l .. r-1 of a genome of n bases).
int check_regions(const int64_t* reg, uint64_t nreg, uint64_t n, uint64_t* total) {
  if (nreg % 2 || (nreg && !reg)) return report_error(MVG_ERR_ARG, "regions must be (left, right) pairs");
  *total = 0;
  for (uint64_t k = 0; k < nreg; k += 2) {
    if (reg[k] < 1 || reg[k + 1] < reg[k] || (uint64_t)reg[k + 1] > n + 1)
      return report_error(MVG_ERR_RANGE, "region outside its genome");
    *total += (uint64_t)(reg[k + 1] - reg[k]);
  }
  return 0;
}

int finish(std::vector<Am>& ml, const int64_t* ra, uint64_t nra, const int64_t* rb, uint64_t nrb) {
  keep_if(ml, [](const Am& m) { return m.mult() == 2; });
  if (int rc = transpose(ml, 0, ra, nra)) return rc;
  if (int rc = transpose(ml, 1, rb, nrb)) return rc;
  if (int rc = eliminate_overlaps(ml)) return rc;
  keep_if(ml, [](const Am& m) { return m.mult() == 2; });
  keep_if(ml, [](const Am& m) { return m.len >= kMinAnchorLength; });
  return 0;
}

// One block per region: bytes reg[2k]-1 .. reg[2k+1]-2 of src to dst_off[k].
__global__ void k_gather_regions(const uint8_t* __restrict__ src, const int64_t* __restrict__ reg,
                                 const uint64_t* __restrict__ dst_off, uint32_t nreg2, uint8_t* __restrict__ dst) {
  for (uint32_t k = blockIdx.x; k < nreg2; k += gridDim.x) {
    const uint64_t from = (uint64_t)reg[2 * k] - 1, len = (uint64_t)(reg[2 * k + 1] - reg[2 * k]);
    const uint64_t to = dst_off[k];
    for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) dst[to + i] = src[from + i];
  }
}

// The search over two device concatenations, then the host steps.
int search_concat(Ctx* c, const uint8_t* d_ca, uint64_t la, const uint8_t* d_cb, uint64_t lb, const int64_t* ra,
                  uint64_t nra, const int64_t* rb, uint64_t nrb, int64_t* out, uint64_t cap, uint64_t* count,
                  uint32_t* weight) {
  const unsigned w = mvg_default_seed_weight((la + lb) / 2);
  if (weight) *weight = w;
  *count = 0;
  if (w < kMinSeedWeight) return 0;  // the reference returns without searching
  const uint64_t seed = mvg_get_seed((int)w, 0);
  const int L = mvg_seed_length(seed);
  const uint64_t bound = std::min(la >= (uint64_t)L ? la - L + 1 : 0, lb >= (uint64_t)L ? lb - L + 1 : 0);
  uint64_t mcap = std::max<uint64_t>(4096, bound / 16);
  std::vector<int64_t> raw;
  uint64_t nm = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    int64_t* d_out = (int64_t*)c->ws.get(c, 83, mcap * 24);
    if (!d_out) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
    int rc = pairwise_matches_dev(c, d_ca, la, d_cb, lb, seed, d_out, mcap, &nm);
    if (rc == MVG_ERR_CAPACITY && attempt == 0) {
      mcap = nm;
      continue;
    }
    if (rc) return rc;
    raw.resize(nm * 3);
    if (nm) MVG_CUDA_TRY(cudaMemcpyAsync(raw.data(), d_out, nm * 24, cudaMemcpyDeviceToHost, c->stream));
    MVG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    break;
  }
  std::vector<Am> ml;
  load(ml, raw.data(), nm);
  if (int rc = finish(ml, ra, nra, rb, nrb)) return rc;
  return store(ml, out, cap, count);
}

}  // namespace
}  // namespace mvg

using namespace mvg;

static Ctx* lg_ctx(mvg_handle h) { return reinterpret_cast<Ctx*>(h); }

extern "C" int mvg_transpose_matches(const int64_t* matches, uint64_t n, unsigned seq, const int64_t* regions,
                                     uint64_t nregions, int64_t* out, uint64_t cap, uint64_t* count) {
  if (!count || seq > 1 || (cap && !out) || nregions % 2 || (nregions && !regions))
    return report_error(MVG_ERR_ARG, "bad argument");
  for (uint64_t k = 0; k < nregions; k += 2)
    if (regions[k + 1] < regions[k]) return report_error(MVG_ERR_ARG, "region ends before it starts");
  if (int rc = check_matches(matches, n)) return rc;
  std::vector<Am> ml;
  load(ml, matches, n);
  if (int rc = transpose(ml, seq, regions, nregions)) return rc;
  return store(ml, out, cap, count);
}

extern "C" int mvg_eliminate_overlaps(const int64_t* matches, uint64_t n, int64_t* out, uint64_t cap,
                                      uint64_t* count) {
  if (!count || (cap && !out)) return report_error(MVG_ERR_ARG, "bad argument");
  if (int rc = check_matches(matches, n)) return rc;
  std::vector<Am> ml;
  load(ml, matches, n);
  if (int rc = eliminate_overlaps(ml)) return rc;
  return store(ml, out, cap, count);
}

extern "C" int mvg_lcb_gap_finish(const int64_t* matches, uint64_t n, const int64_t* regions_a, uint64_t nra,
                                  const int64_t* regions_b, uint64_t nrb, int64_t* out, uint64_t cap,
                                  uint64_t* count) {
  if (!count || (cap && !out) || nra % 2 || nrb % 2 || (nra && !regions_a) || (nrb && !regions_b))
    return report_error(MVG_ERR_ARG, "bad argument");
  for (int g = 0; g < 2; ++g)
    for (uint64_t k = 0; k < (g ? nrb : nra); k += 2)
      if ((g ? regions_b : regions_a)[k + 1] < (g ? regions_b : regions_a)[k])
        return report_error(MVG_ERR_ARG, "region ends before it starts");
  if (int rc = check_matches(matches, n)) return rc;
  std::vector<Am> ml;
  load(ml, matches, n);
  if (int rc = finish(ml, regions_a, nra, regions_b, nrb)) return rc;
  return store(ml, out, cap, count);
}

extern "C" int mvg_search_lcb_gaps(mvg_handle hd, const uint8_t* seq_a, uint64_t na, const uint8_t* seq_b,
                                   uint64_t nb, const int64_t* regions_a, uint64_t nra, const int64_t* regions_b,
                                   uint64_t nrb, int64_t* out, uint64_t cap, uint64_t* count, uint32_t* weight) {
  Ctx* h = lg_ctx(hd);
  if (!h || !count || (na && !seq_a) || (nb && !seq_b) || (cap && !out)) return report_error(MVG_ERR_ARG, "null argument");
  uint64_t la = 0, lb = 0;
  if (int rc = check_regions(regions_a, nra, na, &la)) return rc;
  if (int rc = check_regions(regions_b, nrb, nb, &lb)) return rc;
  if (la >= 0x7fffffffull || lb >= 0x7fffffffull) return report_error(MVG_ERR_ARG, "regions longer than 2^31-1");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  // the concatenations are cut on the host and only they are copied
  std::vector<uint8_t> ca(la), cb(lb);
  for (int g = 0; g < 2; ++g) {
    const uint8_t* src = g ? seq_b : seq_a;
    const int64_t* reg = g ? regions_b : regions_a;
    std::vector<uint8_t>& dst = g ? cb : ca;
    uint64_t at = 0;
    for (uint64_t k = 0; k < (g ? nrb : nra); k += 2) {
      const uint64_t len = (uint64_t)(reg[k + 1] - reg[k]);
      if (len) memcpy(dst.data() + at, src + reg[k] - 1, len);
      at += len;
    }
  }
  uint8_t* d_ca = (uint8_t*)h->ws.get(h, 80, la + 16);
  uint8_t* d_cb = (uint8_t*)h->ws.get(h, 81, lb + 16);
  if (!d_ca || !d_cb) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (la) MVG_CUDA_TRY(cudaMemcpyAsync(d_ca, ca.data(), la, cudaMemcpyHostToDevice, h->stream));
  if (lb) MVG_CUDA_TRY(cudaMemcpyAsync(d_cb, cb.data(), lb, cudaMemcpyHostToDevice, h->stream));
  return search_concat(h, d_ca, la, d_cb, lb, regions_a, nra, regions_b, nrb, out, cap, count, weight);
}

extern "C" int mvg_search_lcb_gaps_dev(mvg_handle hd, const uint8_t* d_seq_a, uint64_t na, const uint8_t* d_seq_b,
                                       uint64_t nb, const int64_t* regions_a, uint64_t nra, const int64_t* regions_b,
                                       uint64_t nrb, int64_t* out, uint64_t cap, uint64_t* count, uint32_t* weight) {
  Ctx* h = lg_ctx(hd);
  if (!h || !count || (na && !d_seq_a) || (nb && !d_seq_b) || (cap && !out))
    return report_error(MVG_ERR_ARG, "null argument");
  uint64_t la = 0, lb = 0;
  if (int rc = check_regions(regions_a, nra, na, &la)) return rc;
  if (int rc = check_regions(regions_b, nrb, nb, &lb)) return rc;
  if (la >= 0x7fffffffull || lb >= 0x7fffffffull) return report_error(MVG_ERR_ARG, "regions longer than 2^31-1");
  MVG_CUDA_TRY(cudaSetDevice(h->device));
  // region table (boundaries, then destination offsets) in one upload
  const uint64_t nr = (nra + nrb) / 2;
  std::vector<int64_t> tab(2 * nr + nr);
  uint64_t at = 0, k2 = 0;
  for (int g = 0; g < 2; ++g) {
    const int64_t* reg = g ? regions_b : regions_a;
    at = 0;
    for (uint64_t k = 0; k < (g ? nrb : nra); k += 2, ++k2) {
      tab[2 * k2] = reg[k];
      tab[2 * k2 + 1] = reg[k + 1];
      tab[2 * nr + k2] = (int64_t)at;
      at += (uint64_t)(reg[k + 1] - reg[k]);
    }
  }
  uint8_t* d_ca = (uint8_t*)h->ws.get(h, 80, la + 16);
  uint8_t* d_cb = (uint8_t*)h->ws.get(h, 81, lb + 16);
  int64_t* d_tab = (int64_t*)h->ws.get(h, 82, tab.size() * 8 + 16);
  if (!d_ca || !d_cb || !d_tab) return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  if (nr) {
    MVG_CUDA_TRY(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, h->stream));
    const uint32_t nreg_a = (uint32_t)(nra / 2), nreg_b = (uint32_t)(nrb / 2);
    const uint64_t* d_off = (const uint64_t*)(d_tab + 2 * nr);
    if (nreg_a) {
      k_gather_regions<<<std::min<uint32_t>(nreg_a, 4096), 256, 0, h->stream>>>(d_seq_a, d_tab, d_off, nreg_a, d_ca);
      h->launches++;
    }
    if (nreg_b) {
      k_gather_regions<<<std::min<uint32_t>(nreg_b, 4096), 256, 0, h->stream>>>(d_seq_b, d_tab + 2 * nreg_a,
                                                                                d_off + nreg_a, nreg_b, d_cb);
      h->launches++;
    }
    MVG_CUDA_TRY(cudaGetLastError());
  }
  return search_concat(h, d_ca, la, d_cb, lb, regions_a, nra, regions_b, nrb, out, cap, count, weight);
}
