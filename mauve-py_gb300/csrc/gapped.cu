// Both gapped-alignment passes of a two-genome progressiveMauve run over
// many LCBs in one call: doGappedAlignment (LM/ProgressiveAligner.cpp:
// 1242-1290) with refineAlignment (:1119-1230), first with profile_aln =
// true (step 8 of alignProfileToProfile, :2560-2565), then with profile_aln
// = false (the final iterative refinement, :3750-3755).
//
// Pass 1: every window of every LCB (lcb_windows) that is not a gap window
// and holds bases of both genomes is cut at MUSCLE's anchor columns
// (anchor_columns) as ProfileAlignFast(anchored) does
// (LM/MuscleInterface.cpp:1053-1109, MU/anchoredpp.cpp:429-552); each range
// of at least one column with bases of both genomes is one gap-DP problem, a
// range with bases of one genome becomes those bases against gaps.  Pass 2:
// RefineFast's column windows (500 or 200 columns of windows of density
// class 1 or 2; MU/refinew.cpp:75-184) with bases of both genomes are one
// problem each, everything else keeps its columns.  Each pass plans on the
// host, runs every problem of every LCB in one batched gap-DP call, rebuilds
// the rows of every problem on the GPU (k_path_rows) and splices them into
// the LCBs' rows on the host.
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "lcb_host.h"
#include "mauve_gb300.h"
#include "mvg_internal.h"

namespace mvg {
namespace {

bool is_gap_char(uint8_t c) { return c == '-' || c == '.'; }

// 0..3 for A/C/G/T in either case, 255 otherwise.
uint8_t base_code(uint8_t c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 255;
  }
}

// A piece of an LCB's new rows: either a gap-DP problem's rows or literal
// columns.
struct Piece {
  int64_t prob;            // problem index (within its LCB's plan until merged), or -1
  std::vector<uint8_t> a;  // literal rows (prob < 0)
  std::vector<uint8_t> b;
};

// The plan of one LCB: its pieces in column order and its problems' bases.
struct Plan {
  std::vector<Piece> pieces;
  std::vector<uint8_t> chars_a, chars_b, codes_a, codes_b;
  std::vector<uint64_t> off_a{0}, off_b{0};
  int rc = 0;

  int add_problem(const uint8_t* ra, const uint8_t* rb, uint64_t lo, uint64_t hi) {
    for (uint64_t c = lo; c < hi; ++c) {
      for (int q = 0; q < 2; ++q) {
        const uint8_t ch = (q ? rb : ra)[c];
        if (is_gap_char(ch)) continue;
        const uint8_t code = base_code(ch);
        if (code > 3) return MVG_ERR_BAD_BASE;
        (q ? chars_b : chars_a).push_back(ch);
        (q ? codes_b : codes_a).push_back(code);
      }
    }
    pieces.push_back(Piece{(int64_t)off_a.size() - 1, {}, {}});
    off_a.push_back(chars_a.size());
    off_b.push_back(chars_b.size());
    return 0;
  }
  void add_literal(const uint8_t* ra, const uint8_t* rb, uint64_t lo, uint64_t hi) {
    if (hi > lo) pieces.push_back(Piece{-1, std::vector<uint8_t>(ra + lo, ra + hi), std::vector<uint8_t>(rb + lo, rb + hi)});
  }
  int64_t nprob() const { return (int64_t)off_a.size() - 1; }
};

uint64_t bases_in(const uint8_t* r, uint64_t lo, uint64_t hi) {
  uint64_t n = 0;
  for (uint64_t c = lo; c < hi; ++c) n += !is_gap_char(r[c]);
  return n;
}

// Pass 1 plan for one LCB.
int plan_anchored(Plan& p, const uint8_t* ra, const uint8_t* rb, uint64_t n, double maxw) {
  std::vector<unsigned> cols;
  for (const LcbWindow& w : lcb_windows(ra, rb, n, maxw)) {
    if (w.gap || !bases_in(ra, w.lo, w.hi) || !bases_in(rb, w.lo, w.hi)) {
      p.add_literal(ra, rb, w.lo, w.hi);
      continue;
    }
    anchor_columns(ra + w.lo, rb + w.lo, (unsigned)(w.hi - w.lo), cols);
    uint64_t lo = w.lo;
    for (size_t k = 0; k <= cols.size(); ++k) {
      const uint64_t hi = k < cols.size() ? w.lo + cols[k] : w.hi;
      if (hi > lo) {
        const uint64_t na = bases_in(ra, lo, hi), nb = bases_in(rb, lo, hi);
        if (na && nb) {
          if (int rc = p.add_problem(ra, rb, lo, hi)) return rc;
        } else {  // the other genome's bases against gaps
          Piece piece{-1, {}, {}};
          for (uint64_t c = lo; c < hi; ++c) {
            const uint8_t ch = (na ? ra : rb)[c];
            if (is_gap_char(ch)) continue;
            piece.a.push_back(na ? ch : (uint8_t)'-');
            piece.b.push_back(na ? (uint8_t)'-' : ch);
          }
          if (!piece.a.empty()) p.pieces.push_back(std::move(piece));
        }
      }
      lo = hi > lo ? hi : lo;
    }
  }
  return 0;
}

// Pass 2 plan for one LCB.
int plan_refine(Plan& p, const uint8_t* ra, const uint8_t* rb, uint64_t n, double maxw) {
  uint64_t at = 0;
  for (const LcbWindow& w : lcb_windows(ra, rb, n, maxw)) {
    const uint64_t width = refine_width(w.density);
    if (w.gap || width == 0) continue;
    for (uint64_t lo = w.lo; lo < w.hi; lo += width) {
      const uint64_t hi = lo + width < w.hi ? lo + width : w.hi;
      p.add_literal(ra, rb, at, lo);
      if (bases_in(ra, lo, hi) && bases_in(rb, lo, hi)) {
        if (int rc = p.add_problem(ra, rb, lo, hi)) return rc;
      } else {
        p.add_literal(ra, rb, lo, hi);
      }
      at = hi;
    }
  }
  p.add_literal(ra, rb, at, n);
  return 0;
}

// Runs fn(k) for k in [0, n) on up to 16 host threads claiming one index at
// a time (LCBs differ in size).
template <class F>
void for_each_lcb(size_t n, F&& fn) {
  const size_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t nt = std::min(hw, n);
  std::atomic<size_t> next{0};
  auto worker = [&]() {
    for (size_t k; (k = next.fetch_add(1)) < n;) fn(k);
  };
  if (nt <= 1) {
    worker();
    return;
  }
  std::vector<std::thread> pool;
  for (size_t t = 0; t < nt; ++t) pool.emplace_back(worker);
  for (std::thread& th : pool) th.join();
}

// The problems of every LCB's plan, concatenated in LCB order.
struct Batch {
  std::vector<uint8_t> chars_a, chars_b, codes_a, codes_b;
  std::vector<uint64_t> off_a{0}, off_b{0};
  std::vector<int64_t> base;  // first problem of each LCB
  int64_t nprob() const { return (int64_t)off_a.size() - 1; }
};

void merge(const std::vector<Plan>& plans, Batch& b) {
  b.base.assign(plans.size() + 1, 0);
  for (size_t k = 0; k < plans.size(); ++k) {
    const Plan& p = plans[k];
    b.base[k + 1] = b.base[k] + p.nprob();
    const uint64_t oa = b.chars_a.size(), ob = b.chars_b.size();
    b.chars_a.insert(b.chars_a.end(), p.chars_a.begin(), p.chars_a.end());
    b.chars_b.insert(b.chars_b.end(), p.chars_b.begin(), p.chars_b.end());
    b.codes_a.insert(b.codes_a.end(), p.codes_a.begin(), p.codes_a.end());
    b.codes_b.insert(b.codes_b.end(), p.codes_b.begin(), p.codes_b.end());
    for (int64_t q = 1; q <= p.nprob(); ++q) {
      b.off_a.push_back(oa + p.off_a[q]);
      b.off_b.push_back(ob + p.off_b[q]);
    }
  }
}

// Runs every problem of a plan on the GPU; rows_a/rows_b get each problem's
// rows at row_off[k].
int solve(Ctx* c, const Batch& p, std::vector<uint8_t>& rows_a, std::vector<uint8_t>& rows_b,
          std::vector<uint64_t>& row_off) {
  const int64_t np = p.nprob();
  row_off.assign(np + 1, 0);
  for (int64_t k = 0; k < np; ++k)
    row_off[k + 1] = row_off[k] + (p.off_a[k + 1] - p.off_a[k]) + (p.off_b[k + 1] - p.off_b[k]);
  if (np == 0) return 0;
  const uint64_t na = p.chars_a.size(), nb = p.chars_b.size(), nr = row_off[np];
  Workspace& ws = c->ws;
  uint8_t* d_codes_a = (uint8_t*)ws.get(c, 84, na + 16);
  uint8_t* d_codes_b = (uint8_t*)ws.get(c, 85, nb + 16);
  uint8_t* d_chars_a = (uint8_t*)ws.get(c, 86, na + 16);
  uint8_t* d_chars_b = (uint8_t*)ws.get(c, 87, nb + 16);
  uint64_t* d_off = (uint64_t*)ws.get(c, 88, 3 * (np + 1) * 8);
  int32_t* d_scores = (int32_t*)ws.get(c, 89, np * 4 + 16);
  char* d_paths = (char*)ws.get(c, 90, nr + 16);
  int64_t* d_plen = (int64_t*)ws.get(c, 91, np * 8 + 16);
  uint8_t* d_rows = (uint8_t*)ws.get(c, 92, 2 * nr + 32);
  if (!d_codes_a || !d_codes_b || !d_chars_a || !d_chars_b || !d_off || !d_scores || !d_paths || !d_plen || !d_rows)
    return report_error(MVG_ERR_NOMEM, "workspace allocation failed");
  uint64_t* d_oa = d_off;
  uint64_t* d_ob = d_off + (np + 1);
  uint64_t* d_po = d_off + 2 * (np + 1);
  cudaStream_t s = c->stream;
  MVG_CUDA_TRY(cudaMemcpyAsync(d_codes_a, p.codes_a.data(), na, cudaMemcpyHostToDevice, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_codes_b, p.codes_b.data(), nb, cudaMemcpyHostToDevice, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_chars_a, p.chars_a.data(), na, cudaMemcpyHostToDevice, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_chars_b, p.chars_b.data(), nb, cudaMemcpyHostToDevice, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_oa, p.off_a.data(), (np + 1) * 8, cudaMemcpyHostToDevice, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_ob, p.off_b.data(), (np + 1) * 8, cudaMemcpyHostToDevice, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(d_po, row_off.data(), (np + 1) * 8, cudaMemcpyHostToDevice, s));
  if (int rc = gapdp_batch_dev(c, d_codes_a, d_oa, d_codes_b, d_ob, np, d_scores, d_paths, d_po, d_plen,
                               p.off_a.data(), p.off_b.data()))
    return rc;
  if (int rc = mvg_path_rows_dev(reinterpret_cast<mvg_handle>(c), d_chars_a, d_oa, d_chars_b, d_ob, np, d_paths,
                                 d_po, d_plen, d_rows, d_rows + nr + 16))
    return rc;
  std::vector<int64_t> plen(np);
  rows_a.resize(nr);
  rows_b.resize(nr);
  MVG_CUDA_TRY(cudaMemcpyAsync(plen.data(), d_plen, np * 8, cudaMemcpyDeviceToHost, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(rows_a.data(), d_rows, nr, cudaMemcpyDeviceToHost, s));
  MVG_CUDA_TRY(cudaMemcpyAsync(rows_b.data(), d_rows + nr + 16, nr, cudaMemcpyDeviceToHost, s));
  MVG_CUDA_TRY(cudaStreamSynchronize(s));
  // a path is one column per edge: its rows are path_len long
  for (int64_t k = 0; k < np; ++k) row_off[k + 1] = row_off[k] + (uint64_t)plen[k];
  // compact: the problems were written at their maximal offsets
  std::vector<uint64_t> at(np + 1, 0);
  for (int64_t k = 0; k < np; ++k)
    at[k + 1] = at[k] + (p.off_a[k + 1] - p.off_a[k]) + (p.off_b[k + 1] - p.off_b[k]);
  for (int64_t k = 0; k < np; ++k) {
    if (row_off[k] == at[k]) continue;
    std::memmove(rows_a.data() + row_off[k], rows_a.data() + at[k], (size_t)plen[k]);
    std::memmove(rows_b.data() + row_off[k], rows_b.data() + at[k], (size_t)plen[k]);
  }
  return 0;
}

// One pass over all LCBs: plan (host threads, one LCB at a time), solve,
// splice.  rows/col_off in, out.
int run_pass(Ctx* c, bool anchored, double maxw, std::vector<uint8_t>& ra, std::vector<uint8_t>& rb,
             std::vector<uint64_t>& col_off) {
  const size_t nlcb = col_off.size() - 1;
  std::vector<Plan> plans(nlcb);
  for_each_lcb(nlcb, [&](size_t k) {
    const uint64_t lo = col_off[k], n = col_off[k + 1] - lo;
    plans[k].rc = anchored ? plan_anchored(plans[k], ra.data() + lo, rb.data() + lo, n, maxw)
                           : plan_refine(plans[k], ra.data() + lo, rb.data() + lo, n, maxw);
  });
  for (const Plan& p : plans)
    if (p.rc) return report_error(p.rc, "the gap DP takes A, C, G and T only");
  Batch batch;
  merge(plans, batch);
  std::vector<uint8_t> pa, pb;
  std::vector<uint64_t> poff;
  if (int rc = solve(c, batch, pa, pb, poff)) return rc;
  // each LCB's new length, then the splice into place (host threads)
  std::vector<uint64_t> noff(nlcb + 1, 0);
  for (size_t k = 0; k < nlcb; ++k) {
    uint64_t len = 0;
    for (const Piece& piece : plans[k].pieces)
      len += piece.prob < 0 ? piece.a.size()
                            : poff[batch.base[k] + piece.prob + 1] - poff[batch.base[k] + piece.prob];
    noff[k + 1] = noff[k] + len;
  }
  std::vector<uint8_t> na(noff[nlcb]), nb(noff[nlcb]);
  for_each_lcb(nlcb, [&](size_t k) {
    uint64_t at = noff[k];
    for (const Piece& piece : plans[k].pieces) {
      if (piece.prob < 0) {
        std::memcpy(na.data() + at, piece.a.data(), piece.a.size());
        std::memcpy(nb.data() + at, piece.b.data(), piece.b.size());
        at += piece.a.size();
      } else {
        const int64_t g = batch.base[k] + piece.prob;
        const uint64_t o = poff[g], len = poff[g + 1] - o;
        std::memcpy(na.data() + at, pa.data() + o, len);
        std::memcpy(nb.data() + at, pb.data() + o, len);
        at += len;
      }
    }
  });
  ra.swap(na);
  rb.swap(nb);
  col_off.swap(noff);
  return 0;
}

}  // namespace
}  // namespace mvg

using namespace mvg;

extern "C" int mvg_gapped_alignment(mvg_handle hd, const uint8_t* rows_a, const uint8_t* rows_b,
                                    const uint64_t* col_off, int64_t nlcb, double max_window_size, int passes,
                                    uint8_t* out_a, uint8_t* out_b, uint64_t* out_off, uint64_t cap) {
  Ctx* c = reinterpret_cast<Ctx*>(hd);
  if (!c || nlcb < 0 || !col_off || !out_off || (passes & ~3) || !(max_window_size > 200.0))
    return report_error(MVG_ERR_ARG, "bad argument");
  const uint64_t ncols = col_off[nlcb];
  if ((ncols && (!rows_a || !rows_b)) || (cap && (!out_a || !out_b))) return report_error(MVG_ERR_ARG, "null argument");
  for (int64_t k = 0; k < nlcb; ++k)
    if (col_off[k + 1] < col_off[k]) return report_error(MVG_ERR_ARG, "column offsets must not decrease");
  MVG_CUDA_TRY(cudaSetDevice(c->device));
  std::vector<uint8_t> ra(rows_a, rows_a + ncols), rb(rows_b, rows_b + ncols);
  std::vector<uint64_t> off(col_off, col_off + nlcb + 1);
  const uint64_t base = off[0];
  for (uint64_t& o : off) o -= base;
  if (passes & 1)
    if (int rc = run_pass(c, true, max_window_size, ra, rb, off)) return rc;
  if (passes & 2)
    if (int rc = run_pass(c, false, max_window_size, ra, rb, off)) return rc;
  for (int64_t k = 0; k <= nlcb; ++k) out_off[k] = off[k];
  if (ra.size() > cap) return report_error(MVG_ERR_CAPACITY, "row buffer too small");
  if (!ra.empty()) {
    std::memcpy(out_a, ra.data(), ra.size());
    std::memcpy(out_b, rb.data(), rb.size());
  }
  return 0;
}
