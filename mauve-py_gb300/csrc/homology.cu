// Homologous segments of two-genome alignments: the detection step of the
// backbone computation, findHssHomologyHMM (LM/Islands.h:122-196), as
// detectAndApplyBackbone runs it over every LCB (LM/Backbone.cpp:1081-1088)
// with the parameters applyBackbone sets up
// (MA/progressiveMauve.cpp:226-238, LM/HomologyHMM/parameters.h).  Host
// code, LCBs on host threads.
//
// Each column of the pair becomes an emission symbol (match classes '1'-'6',
// a gap '7', the inner columns of runs of three or more gaps '8'; columns
// gapped in both are dropped), the two-state HMM (homologous / unrelated,
// LM/HomologyHMM/homology.cc:307-552) runs forward and backward over the
// symbols, and a column is homologous where its posterior is at least 0.9
// (LM/HomologyHMM/homologymain.cc:24-63).  The passes run in HMMoC's
// extended-exponent arithmetic (LM/HomologyHMM/algebras.h): a float mantissa
// and an integer exponent of 2^104, renormalised one step per product, with
// sums aligned through a two-entry table of powers of 2^-104.  Every
// operation is restated in the reference's order and precision, so the
// decisions are the reference's bit for bit: the chain is inherently
// sequential (each step rounds the previous one's mantissa), which is why it
// runs on the host, one LCB per thread.
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <string>
#include <thread>
#include <vector>

#include "mauve_gb300.h"
#include "mvg_internal.h"

namespace mvg {
namespace {

// HMMoC's BFloat (LM/HomologyHMM/algebras.h): value f * 2^(104 e).
struct BF {
  float f;
  int e;
};

constexpr float kRange = 20282409603651670423947251286016.0f;  // 2^104
constexpr int kInfExp = 1000000000;
constexpr int kConv = 100;
constexpr int kDConv = 50;

struct BfTables {
  float range_inv, range_sqrt, range_inv_sqrt, logc;
  float conv[kConv];      // 2^(-104 k) in float: 1, 2^-104, then 0
  double dconv[kDConv];   // 2^(104 (k - 25)) as the reference computes it
  BfTables() {
    range_inv = (float)(1.0 / (double)kRange);
    range_sqrt = 1.0e+18f;
    range_inv_sqrt = 1.0e-18f;
    logc = std::log(kRange);
    float x = 1.0f;
    for (int i = 0; i < kConv; ++i) {
      conv[i] = x;
      x *= range_inv;
    }
    for (int i = 0; i < kDConv; ++i) dconv[i] = (double)std::exp((float)(i - kDConv / 2) * logc);
  }
};

const BfTables& T() {
  static const BfTables t;
  return t;
}

constexpr BF kZero{0.0f, -kInfExp};

// BFloatNormalise: one step down or up.
inline void fnorm(BF& a) {
  const BfTables& t = T();
  if (a.f > t.range_sqrt) {
    a.f *= t.range_inv;
    a.e++;
  } else if (a.f < t.range_inv_sqrt) {
    if (a.f == 0.0f) {
      a.e = -kInfExp;
    } else {
      a.f *= kRange;
      a.e--;
    }
  }
}

// bfloat_pr_double_product: the mantissa times a double, renormalised in
// double precision, then narrowed.
inline BF mul_d(const BF& a, double b) {
  const BfTables& t = T();
  double m = (double)a.f * b;
  int e = a.e;
  if (m <= 0.0) {
    m = 0.0;
    e = -kInfExp;
  } else {
    while (m > (double)t.range_sqrt) {
      m *= (double)t.range_inv;
      ++e;
    }
    while (m < (double)t.range_inv_sqrt) {
      m *= (double)kRange;
      --e;
    }
  }
  return BF{(float)m, e};
}

// bfloat_pr_sum_accum
inline void add_to(BF& a, const BF& b) {
  const BfTables& t = T();
  if (a.e >= b.e) {
    if (a.e < b.e + kConv) a.f += b.f * t.conv[a.e - b.e];
  } else if (a.e > b.e - kConv) {
    a.f = b.f + a.f * t.conv[b.e - a.e];
    a.e = b.e;
  } else {
    a = b;
  }
}

inline BF mul(const BF& a, const BF& b) {
  BF s{a.f * b.f, a.e + b.e};
  fnorm(s);
  return s;
}

inline BF div(const BF& a, const BF& b) {
  BF s{a.f / b.f, a.e - b.e};
  fnorm(s);
  return s;
}

// BFloat::Value
inline double value(const BF& x) {
  const BfTables& t = T();
  if (abs(x.e) < kDConv / 2) return (double)x.f * t.dconv[x.e + kDConv / 2];
  if (x.e < kDConv / 2) return 0.0;
  return (double)x.f * std::exp((double)x.e * (double)t.logc);
}

// The HMM's eight transition probabilities (homology.cc:323-338).
struct Trans {
  double t[8];
  explicit Trans(const mvg_hmm_params& p) {
    t[0] = p.start_homologous;
    t[1] = 1.0 - p.start_homologous;
    t[2] = 1.0 - p.go_unrelated - p.go_stop_from_homologous;
    t[3] = p.go_unrelated;
    t[4] = 1.0 - p.go_homologous - p.go_stop_from_unrelated;
    t[5] = p.go_homologous;
    t[6] = p.go_stop_from_homologous;
    t[7] = p.go_stop_from_unrelated;
  }
};

// Posterior decoding of one symbol string: pred[i] = posterior of the
// homologous state at symbol i >= 0.9.  State 0 = homologous, 1 = unrelated.
void decode(const std::string& sym, const mvg_hmm_params& p, std::vector<uint8_t>& pred) {
  const int L = (int)sym.size();
  pred.assign(L, 0);
  if (L == 0) return;
  const Trans tr(p);
  const double* T_ = tr.t;
  auto eu = [&](char s) { return p.emit_unrelated[s - '1']; };
  auto eh = [&](char s) { return p.emit_homologous[s - '1']; };
  // forward (homology.cc:307-398): F[pos], pos = 1..L
  std::vector<BF> F(2 * (size_t)(L + 1));
  const BF one{1.0f, 0};
  for (int pos = 1; pos <= L; ++pos) {
    const char s = sym[pos - 1];
    const double e0 = eu(s), e1 = eh(s);
    BF* to = &F[2 * (size_t)pos];
    if (pos == 1) {
      to[1] = mul_d(one, T_[1] * e0);
      to[0] = mul_d(one, T_[0] * e1);
    } else {
      const BF* fr = &F[2 * (size_t)(pos - 1)];
      to[0] = kZero;
      to[1] = kZero;
      add_to(to[1], mul_d(fr[1], T_[4] * e0));
      add_to(to[1], mul_d(fr[0], T_[3] * e0));
      add_to(to[0], mul_d(fr[1], T_[5] * e1));
      add_to(to[0], mul_d(fr[0], T_[2] * e1));
    }
  }
  BF total = mul_d(F[2 * (size_t)L + 1], T_[7] * 1.0);
  add_to(total, mul_d(F[2 * (size_t)L], T_[6] * 1.0));
  // backward (homology.cc:400-552), with the posterior of each symbol
  const BF end{1.0f, 0};
  BF nxt[2] = {kZero, kZero};
  for (int pos = L; pos >= 1; --pos) {
    const char s = pos <= L - 1 ? sym[pos] : '1';
    const double e0 = eu(s), e1 = eh(s);
    BF to[2] = {kZero, kZero};
    if (pos + 1 <= L) {
      to[0] = mul_d(nxt[0], T_[2] * e1);
      add_to(to[0], mul_d(nxt[1], T_[3] * e0));
      to[1] = mul_d(nxt[1], T_[4] * e0);
      add_to(to[1], mul_d(nxt[0], T_[5] * e1));
    }
    if (pos >= L) {
      add_to(to[0], mul_d(end, T_[6] * 1.0));
      add_to(to[1], mul_d(end, T_[7] * 1.0));
    }
    const double post = value(div(mul(F[2 * (size_t)pos], to[0]), total));
    pred[pos - 1] = post >= 0.9;
    nxt[0] = to[0];
    nxt[1] = to[1];
  }
}

// Emission code of a character (LM/Islands.h:92-121): a c g t - in either
// case, anything else counts as 'a'.
inline int col_code(uint8_t c) {
  switch (c) {
    case 'c': case 'C': return 1;
    case 'g': case 'G': return 2;
    case 't': case 'T': return 3;
    case '-': return 4;
    default: return 0;
  }
}

constexpr char kColMap[5][5] = {
    {'1', '3', '4', '5', '7'}, {'3', '2', '6', '4', '7'}, {'4', '6', '2', '3', '7'},
    {'5', '4', '3', '1', '7'}, {'7', '7', '7', '7', '\0'}};

// findHssHomologyHMM for one LCB: homologous column ranges (inclusive).
void segments(const uint8_t* ra, const uint8_t* rb, uint64_t n, const mvg_hmm_params& p, bool left_h, bool right_h,
              std::vector<int64_t>& out) {
  std::string sym;
  std::vector<uint64_t> col_ref;
  sym.reserve(n);
  col_ref.reserve(n);
  for (uint64_t c = 0; c < n; ++c) {
    const char s = kColMap[col_code(ra[c])][col_code(rb[c])];
    if (s == '\0') continue;
    sym.push_back(s);
    col_ref.push_back(c);
  }
  // runs of gap columns: the inner ones (and gapped ends) become '8'
  for (size_t i = 2; i < sym.size(); ++i)
    if (sym[i] == '7' && sym[i - 1] == '7' && (sym[i - 2] == '7' || sym[i - 2] == '8')) sym[i - 1] = '8';
  const size_t L = sym.size();
  if (L > 1 && sym[0] == '7' && (sym[1] == '7' || sym[1] == '8')) sym[0] = '8';
  if (L > 1 && sym[L - 1] == '7' && (sym[L - 2] == '7' || sym[L - 2] == '8')) sym[L - 1] = '8';
  const bool rev = right_h && !left_h;
  if (rev) std::reverse(sym.begin(), sym.end());
  std::vector<uint8_t> pred;
  decode(sym, p, pred);
  if (rev) std::reverse(pred.begin(), pred.end());
  size_t prev_h = 0, i = 1;
  for (; i < pred.size(); ++i) {
    if (pred[i] && !pred[i - 1]) prev_h = i;
    if (!pred[i] && pred[i - 1]) {
      out.push_back((int64_t)col_ref[prev_h]);
      out.push_back((int64_t)col_ref[i - 1]);
      prev_h = i;
    }
  }
  if (!pred.empty() && pred[i - 1]) {
    out.push_back((int64_t)col_ref[prev_h]);
    out.push_back((int64_t)col_ref[i - 1]);
  }
}

}  // namespace
}  // namespace mvg

using namespace mvg;

extern "C" int mvg_hmm_backbone_params(double gc_content, double go_homologous, double go_unrelated,
                                       double pct_identity, mvg_hmm_params* out) {
  if (!out || !(pct_identity > 0) || pct_identity > 1) return report_error(MVG_ERR_ARG, "bad argument");
  mvg_hmm_params p;
  // getAdaptedHoxdMatrixParameters (LM/HomologyHMM/parameters.h)
  const double at = 1 - gc_content;
  const double gO_u = 0.0483, gE_u = 0.2535, gO_h = 0.004461, gE_h = 0.050733;
  double* u = p.emit_unrelated;
  double* h = p.emit_homologous;
  u[0] = (at / 2) * (at / 2) + (at / 2) * (at / 2);
  u[1] = (gc_content / 2) * (gc_content / 2) + (gc_content / 2) * (gc_content / 2);
  u[2] = (at / 2) * (gc_content / 2) + (gc_content / 2) * (at / 2);
  u[3] = u[2];
  u[4] = u[0];
  u[5] = u[1];
  double norm = (1 - (gO_u + gE_u)) / (u[0] + u[1] + u[2] + u[3] + u[4] + u[5]);
  for (int k = 0; k < 6; ++k) u[k] = u[k] * norm;
  u[6] = gO_u;
  u[7] = 1 - (u[0] + u[1] + u[2] + u[3] + u[4] + u[5] + u[6]);
  const double H_AA = 0.1723 * 2, H_CC = 0.1462 * 2, H_AC = 0.0180 * 4, H_AG = 0.0426 * 4, H_AT = 0.0186 * 2,
               H_CG = 0.0142 * 2;
  h[0] = (at / 0.525) * H_AA;
  h[1] = (gc_content / 0.475) * H_CC;
  h[2] = H_AC;
  h[3] = H_AG;
  h[4] = (at / 0.525) * H_AT;
  h[5] = (gc_content / 0.475) * H_CG;
  norm = (1 - (gO_h + gE_h)) / (h[0] + h[1] + h[2] + h[3] + h[4] + h[5]);
  for (int k = 0; k < 6; ++k) h[k] = h[k] * norm;
  h[6] = gO_h;
  h[7] = 1 - (h[0] + h[1] + h[2] + h[3] + h[4] + h[5] + h[6]);
  p.start_homologous = 0.5;
  p.go_homologous = 0.00001;
  p.go_unrelated = 0.0000001;
  p.go_stop_from_homologous = 0.0000001;
  p.go_stop_from_unrelated = 0.0000001;
  // applyBackbone's overrides (MA/progressiveMauve.cpp:236-237)
  p.go_homologous = go_homologous;
  p.go_unrelated = go_unrelated;
  // adaptToPercentIdentity (LM/HomologyHMM/parameters.h)
  const double gapnorm = pct_identity * (1.0 - h[6] - h[7]);
  const double prev_id = h[0] + h[1];
  const double diff = prev_id - gapnorm;
  const double rest = h[2] + h[3] + h[4] + h[5];
  h[2] += diff * h[2] / rest;
  h[3] += diff * h[3] / rest;
  h[4] += diff * h[4] / rest;
  h[5] += diff * h[5] / rest;
  h[0] -= diff * h[0] / prev_id;
  h[1] -= diff * h[1] / prev_id;
  *out = p;
  return 0;
}

extern "C" int mvg_homologous_segments(const uint8_t* rows_a, const uint8_t* rows_b, const uint64_t* col_off,
                                       int64_t nlcb, const mvg_hmm_params* params, int left_homologous,
                                       int right_homologous, int64_t* segs, uint64_t cap, uint64_t* nsegs,
                                       uint64_t* seg_off) {
  if (nlcb < 0 || !col_off || !params || !nsegs || !seg_off || (cap && !segs))
    return report_error(MVG_ERR_ARG, "bad argument");
  if (col_off[nlcb] > col_off[0] && (!rows_a || !rows_b)) return report_error(MVG_ERR_ARG, "null argument");
  for (int64_t k = 0; k < nlcb; ++k)
    if (col_off[k + 1] < col_off[k]) return report_error(MVG_ERR_ARG, "column offsets must not decrease");
  std::vector<std::vector<int64_t>> per(nlcb);
  const size_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t nt = std::min<size_t>(hw, (size_t)nlcb);
  std::atomic<int64_t> next{0};
  auto worker = [&]() {
    for (int64_t k; (k = next.fetch_add(1)) < nlcb;)
      segments(rows_a + col_off[k], rows_b + col_off[k], col_off[k + 1] - col_off[k], *params, left_homologous != 0,
               right_homologous != 0, per[k]);
  };
  if (nt <= 1) {
    worker();
  } else {
    std::vector<std::thread> pool;
    for (size_t t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (std::thread& th : pool) th.join();
  }
  uint64_t n = 0;
  seg_off[0] = 0;
  for (int64_t k = 0; k < nlcb; ++k) {
    const uint64_t m = per[k].size() / 2;
    for (uint64_t i = 0; i < m && n + i < cap; ++i) {
      segs[2 * (n + i)] = per[k][2 * i];
      segs[2 * (n + i) + 1] = per[k][2 * i + 1];
    }
    n += m;
    seg_off[k + 1] = n;
  }
  *nsegs = n;
  if (n > cap) return report_error(MVG_ERR_CAPACITY, "segment buffer too small");
  return 0;
}
