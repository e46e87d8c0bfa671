// LCBs of a two-genome match list with greedy breakpoint elimination, as
// alignProfileToProfile computes them when the genomes are taken as
// collinear (LM/ProgressiveAligner.cpp:2281-2303): IdentifyBreakpoints and
// ComputeLCBs_v2 (LM/GreedyBreakpointElimination.h:162-242), each LCB's
// weight by SimpleGetLCBCoverage (LM/ProgressiveAligner.h:409-430), the
// breakpoint penalty 100 + the weights' sum, computeLCBAdjacencies_v3 (:252-314)
// with FindBoundaries (LM/Interval.h:704-780), greedyBreakpointElimination_v4
// (:650-755) with the SimpleBreakpointScorer in collinear mode and
// RemoveLCBandCoalesce / undoLcbRemoval (LM/GreedyBreakpointElimination.cpp:
// 147-325, 884-948), and filterMatches_v2 (:328-399).  Host code.
//
// Every sort is std::sort (or the heap operations) under comparators that
// order as the reference's, on sequences that went through the same steps,
// so ties, the move heap's order (built over the whole vector, whose second
// half holds value-initialised moves, as the reference builds it) and hence
// the LCBs are the reference's.  A match is a two-genome ungapped libMems
// Match: signed 1-based starts (negative = reverse), defined in both genomes.
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <stack>
#include <utility>
#include <vector>

#include "mauve_gb300.h"
#include "mvg_internal.h"

namespace mvg {
namespace {

constexpr uint32_t kNone = 0xffffffffu;  // (uint)-1: no adjacent LCB, LCB_UNASSIGNED
constexpr int kSeqs = 2;

struct Mt {
  int64_t s[2];
  int64_t len;
};

enum { kUndef = 0, kFwd = 1, kRev = 2 };
inline int orient(const Mt& m, int q) { return m.s[q] == 0 ? kUndef : (m.s[q] > 0 ? kFwd : kRev); }
inline uint64_t left_end(const Mt& m, int q) { return (uint64_t)(m.s[q] < 0 ? -m.s[q] : m.s[q]); }

struct Lcb {
  int64_t left_end[kSeqs];
  int64_t right_end[kSeqs];
  uint32_t left_adj[kSeqs];
  uint32_t right_adj[kSeqs];
  int lcb_id;
  double weight;
  bool to_be_deleted;
};

using MatchList = std::vector<uint32_t>;  // match ids

// SSC(seq): undefined before defined, then by left end.
struct SscOrder {
  const std::vector<Mt>* m;
  int q;
  bool operator()(uint32_t a, uint32_t b) const {
    const uint64_t as = left_end((*m)[a], q), bs = left_end((*m)[b], q);
    if (as == 0 || bs == 0) return bs != 0;
    return as < bs;
  }
};

void identify_breakpoints(const std::vector<Mt>& M, MatchList& ml, std::vector<uint64_t>& bps) {
  if (ml.empty()) return;
  bps.assign(1, ml.size() - 1);
  std::sort(ml.begin(), ml.end(), SscOrder{&M, 0});
  std::vector<std::pair<uint32_t, uint64_t>> label(ml.size());
  for (size_t i = 0; i < ml.size(); ++i) label[i] = std::make_pair(ml[i], (uint64_t)i);
  for (int q = 1; q < kSeqs; ++q) {
    const SscOrder ssc{&M, q};
    std::sort(label.begin(), label.end(),
              [&](const std::pair<uint32_t, uint64_t>& x, const std::pair<uint32_t, uint64_t>& y) {
                return ssc(x.first, y.first);
              });
    size_t prev = 0;
    bool prev_orient = orient(M[label[prev].first], q) == orient(M[label[prev].first], 0);
    if (!prev_orient) bps.push_back(label[prev].second);
    for (size_t it = 1; it < label.size(); ++it) {
      const bool cur_orient = orient(M[label[it].first], q) == orient(M[label[it].first], 0);
      if (prev_orient == cur_orient && ((prev_orient && label[prev].second + 1 == label[it].second) ||
                                        (!prev_orient && label[prev].second - 1 == label[it].second))) {
        prev_orient = cur_orient;
        ++prev;
        continue;
      }
      if (prev_orient) bps.push_back(label[prev].second);
      if (!cur_orient) bps.push_back(label[it].second);
      prev_orient = cur_orient;
      ++prev;
    }
    if (prev_orient) bps.push_back(label[prev].second);
  }
  std::sort(bps.begin(), bps.end());
  bps.erase(std::unique(bps.begin(), bps.end()), bps.end());
}

void compute_lcbs(const MatchList& ml, const std::vector<uint64_t>& bps, std::vector<MatchList>& lcbs) {
  if (bps.empty()) return;
  lcbs.clear();
  uint32_t prev = 0;
  for (uint64_t b : bps) {
    lcbs.emplace_back(ml.begin() + prev, ml.begin() + b + 1);
    prev = (uint32_t)(b + 1);
  }
}

// SimpleGetLCBCoverage for two-genome ungapped matches.
uint64_t coverage(const std::vector<Mt>& M, const MatchList& lcb) {
  uint64_t cov = 0;
  for (uint32_t id : lcb) {
    const Mt& m = M[id];
    double maxlen = 0, minlen = 0;
    for (int q = 0; q < kSeqs; ++q) {
      if (left_end(m, q) == 0) continue;
      maxlen += (double)m.len;
      if ((double)m.len > minlen) minlen = (double)m.len;
    }
    double score = std::exp(((double)m.len - minlen) / (maxlen - minlen));
    score *= maxlen;
    cov += (uint64_t)score;
  }
  return cov;
}

// FindBoundaries for one LCB's matches.
void find_boundaries(const std::vector<Mt>& M, const MatchList& ms, uint64_t le[kSeqs], uint64_t ln[kSeqs],
                     bool fw[kSeqs]) {
  for (int q = 0; q < kSeqs; ++q) {
    le[q] = 0;
    ln[q] = 0;
    fw[q] = false;
  }
  const size_t n = ms.size();
  for (size_t i = 0; i != n; ++i) {
    bool zero = false;
    for (int q = 0; q < kSeqs; ++q) {
      if (le[q] == 0 && orient(M[ms[i]], q) == kFwd) {
        le[q] = left_end(M[ms[i]], q);
        fw[q] = true;
      } else if (le[q] == 0) {
        zero = true;
      }
    }
    if (!zero) break;
  }
  for (size_t i = n; i > 0; --i) {
    bool zero = false;
    for (int q = 0; q < kSeqs; ++q) {
      const Mt& m = M[ms[i - 1]];
      if (ln[q] == 0 && orient(m, q) == kFwd) ln[q] = left_end(m, q) + (uint64_t)m.len - le[q];
      if (le[q] != 0 && ln[q] == 0) zero = true;
    }
    if (!zero) break;
  }
  for (size_t i = n; i > 0; --i) {
    bool zero = false;
    for (int q = 0; q < kSeqs; ++q) {
      const Mt& m = M[ms[i - 1]];
      if (le[q] == 0 && orient(m, q) == kRev) le[q] = left_end(m, q);
      if (le[q] == 0) zero = true;
    }
    if (!zero) break;
  }
  for (size_t i = 0; i != n; ++i) {
    bool zero = false;
    for (int q = 0; q < kSeqs; ++q) {
      const Mt& m = M[ms[i]];
      if (ln[q] == 0 && orient(m, q) == kRev) ln[q] = (uint64_t)m.len + (left_end(m, q) - le[q]);
      if (ln[q] == 0) zero = true;
    }
    if (!zero) break;
  }
}

void compute_adjacencies(const std::vector<Mt>& M, const std::vector<MatchList>& lcbs,
                         const std::vector<double>& weights, std::vector<Lcb>& adj) {
  adj.clear();
  if (lcbs.empty()) return;
  for (size_t k = 0; k < lcbs.size(); ++k) {
    uint64_t le[kSeqs], ln[kSeqs];
    bool fw[kSeqs];
    find_boundaries(M, lcbs[k], le, ln, fw);
    Lcb l;
    for (int q = 0; q < kSeqs; ++q) {
      l.left_adj[q] = kNone;
      l.right_adj[q] = kNone;
      l.left_end[q] = 0;
      l.right_end[q] = 0;
      if (le[q] == 0) continue;
      l.left_end[q] = (int64_t)le[q];
      l.right_end[q] = (int64_t)(le[q] + ln[q]);
      if (!fw[q]) {
        l.left_end[q] = -l.left_end[q];
        l.right_end[q] = -l.right_end[q];
      }
    }
    l.lcb_id = (int)adj.size();
    l.weight = weights[k];
    l.to_be_deleted = false;
    adj.push_back(l);
  }
  for (int q = 0; q < kSeqs; ++q) {
    std::sort(adj.begin(), adj.end(), [q](const Lcb& a, const Lcb& b) {  // LCBLeftComparator
      int64_t as = a.left_end[q], bs = b.left_end[q];
      if (as == 0 || bs == 0) return bs != 0;
      if (as < 0) as = -as;
      if (bs < 0) bs = -bs;
      return as - bs < 0;
    });
    size_t k = 1;
    for (; k + 1 < lcbs.size(); ++k) {
      adj[k].left_adj[q] = (uint32_t)adj[k - 1].lcb_id;
      adj[k].right_adj[q] = (uint32_t)adj[k + 1].lcb_id;
    }
    if (k == lcbs.size()) --k;
    adj[0].left_adj[q] = kNone;
    adj[k].right_adj[q] = kNone;
    if (k > 0) {
      adj[0].right_adj[q] = (uint32_t)adj[1].lcb_id;
      adj[k].left_adj[q] = (uint32_t)adj[k - 1].lcb_id;
    }
  }
  std::sort(adj.begin(), adj.end(), [](const Lcb& a, const Lcb& b) { return a.lcb_id < b.lcb_id; });
}

inline bool is_self(const std::vector<Lcb>& adj, uint32_t i) { return (uint32_t)adj[i].lcb_id == i; }

uint32_t remove_and_coalesce(size_t lcbI, std::vector<Lcb>& adj, std::vector<double>& scores,
                             std::vector<std::pair<uint32_t, uint32_t>>& remaps, std::vector<uint32_t>& impact) {
  uint32_t removed = 0;
  impact.assign(kSeqs * (2 + kSeqs * 4), kNone);
  size_t ii = 0;
  remaps.clear();
  adj[lcbI].lcb_id = -2;
  for (int q = 0; q < kSeqs; ++q) {
    const uint32_t l = adj[lcbI].left_adj[q], r = adj[lcbI].right_adj[q];
    if (l != kNone) adj[l].right_adj[q] = r;
    if (r != kNone && r != adj.size()) adj[r].left_adj[q] = l;
  }
  for (int q = 0; q < kSeqs; ++q) {
    const uint32_t l = adj[lcbI].left_adj[q], r = adj[lcbI].right_adj[q];
    impact[ii++] = l;
    impact[ii++] = r;
    for (int j = 0; j < kSeqs; ++j) {
      if (l != kNone) {
        impact[ii++] = adj[l].left_adj[j];
        impact[ii++] = adj[l].right_adj[j];
      }
      if (r != kNone) {
        impact[ii++] = adj[r].left_adj[j];
        impact[ii++] = adj[r].right_adj[j];
      }
    }
  }
  remaps.push_back(std::make_pair((uint32_t)lcbI, kNone));
  removed++;
  for (int q = 0; q < kSeqs; ++q) {
    uint32_t l = adj[lcbI].left_adj[q], r = adj[lcbI].right_adj[q];
    while (l != kNone && !is_self(adj, l)) l = adj[l].left_adj[q];
    while (r != kNone && !is_self(adj, r)) r = adj[r].right_adj[q];
    if (l == kNone || r == kNone) continue;
    if (!is_self(adj, l) || !is_self(adj, r)) {
      if (q > 0) continue;
    }
    const bool orientation = adj[l].left_end[q] > 0;
    int j;
    for (j = 0; j < kSeqs; ++j) {
      const bool jo = adj[l].left_end[j] > 0;
      if (jo == orientation && adj[l].right_adj[j] != r) break;
      if (jo != orientation && adj[l].left_adj[j] != r) break;
      if ((adj[r].left_end[j] > 0) != jo) break;
    }
    if (j != kSeqs || adj[l].to_be_deleted || adj[r].to_be_deleted) continue;
    remaps.push_back(std::make_pair((uint32_t)adj[r].lcb_id, l));
    adj[r].lcb_id = (int)l;
    scores[l] += scores[r];
    adj[l].weight += adj[r].weight;
    for (j = 0; j < kSeqs; ++j) {
      const bool jo = adj[l].left_end[j] > 0;
      const uint32_t rr = adj[r].right_adj[j], rl = adj[r].left_adj[j];
      if (jo == orientation) {
        adj[l].right_end[j] = adj[r].right_end[j];
        adj[l].right_adj[j] = rr;
        if (rr != kNone) adj[rr].left_adj[j] = l;
      } else {
        adj[l].left_end[j] = adj[r].left_end[j];
        adj[l].left_adj[j] = rl;
        if (rl != kNone) adj[rl].right_adj[j] = l;
      }
    }
    removed++;
  }
  std::sort(impact.begin(), impact.end());
  auto end = std::unique(impact.begin(), impact.end());
  auto pre = std::lower_bound(impact.begin(), end, kNone);
  impact.erase(pre, impact.end());
  return removed;
}

void undo_removal(std::vector<Lcb>& adj, const std::vector<std::pair<uint32_t, uint32_t>>& remaps) {
  for (size_t k = remaps.size(); k > 0; --k) {
    if (remaps[k - 1].second == kNone) {
      const uint32_t i = remaps[k - 1].first;
      for (int q = 0; q < kSeqs; ++q) {
        const uint32_t l = adj[i].left_adj[q], r = adj[i].right_adj[q];
        if (l != kNone) adj[l].right_adj[q] = i;
        if (r != kNone && r != adj.size()) adj[r].left_adj[q] = i;
      }
      adj[i].lcb_id = (int)i;
      adj[i].to_be_deleted = false;
    } else {
      const uint32_t i = remaps[k - 1].first, j = remaps[k - 1].second;
      adj[i].lcb_id = (int)i;
      adj[j].weight -= adj[i].weight;
      for (int q = 0; q < kSeqs; ++q) {
        const uint32_t l = adj[i].left_adj[q], r = adj[i].right_adj[q];
        if (l == j) {
          adj[j].right_adj[q] = i;
          if (r != kNone && r != adj.size()) adj[r].left_adj[q] = i;
        } else if (r == j) {
          adj[j].left_adj[q] = i;
          if (l != kNone && l != adj.size()) adj[l].right_adj[q] = i;
        }
      }
    }
  }
}

// SimpleBreakpointScorer (collinear): its own copy of the adjacencies.
struct Scorer {
  std::vector<Lcb> adjs;
  double bp_penalty;
  std::vector<double> scores;
  double total_weight = 0;
  size_t bp_count;
  bool collinear;
  Scorer(const std::vector<Lcb>& a, double penalty, bool col)
      : adjs(a), bp_penalty(penalty), scores(a.size(), 0), bp_count(a.size()), collinear(col) {
    for (const Lcb& l : adjs) total_weight += l.weight;
  }
  double score() const { return total_weight - (double)bp_count * bp_penalty; }
  // scratch of move(), kept between calls so that scoring allocates nothing
  std::vector<std::pair<uint32_t, uint32_t>> mv_remaps;
  std::vector<uint32_t> mv_impact;
  double move(size_t i) {
    const double cur = score();
    const uint32_t bp_removed = remove_and_coalesce(i, adjs, scores, mv_remaps, mv_impact);
    undo_removal(adjs, mv_remaps);
    const double bp_score = (double)(bp_count - bp_removed) * bp_penalty;
    const double move_score = total_weight - adjs[i].weight - bp_score;
    const double diff = move_score - cur;
    if (collinear && bp_count - bp_removed > 0 && diff < 0) return 1 / (-diff);
    return move_score - cur;
  }
  bool valid(size_t i, double s) {
    if ((uint32_t)adjs[i].lcb_id != i) return false;
    return move(i) == s;
  }
  void remove(uint32_t i, std::vector<std::pair<double, size_t>>& new_moves) {
    std::vector<std::pair<uint32_t, uint32_t>> remaps;
    std::vector<uint32_t> impact;
    const uint32_t bp_removed = remove_and_coalesce(i, adjs, scores, remaps, impact);
    total_weight -= adjs[i].weight;
    bp_count -= bp_removed;
    for (uint32_t x : impact) {
      if ((uint32_t)adjs[x].lcb_id != x) continue;
      new_moves.push_back(std::make_pair(move(x), (size_t)x));
    }
  }
};

struct MoveOrder {
  bool operator()(const std::pair<double, size_t>& a, const std::pair<double, size_t>& b) const {
    return a.first < b.first;
  }
};

void greedy_elimination(std::vector<Lcb>& adj, std::vector<double>& scores, Scorer& sc) {
  double total = 0;
  for (double w : scores) total += w;
  double current = total;
  if (adj.empty()) return;
  const size_t nmoves = adj.size();
  std::vector<std::pair<double, size_t>> heap(nmoves * 2);
  size_t heap_end = nmoves;
  for (size_t i = 0; i < nmoves; ++i) {
    heap[i].first = sc.move(i);
    heap[i].second = i;
  }
  const MoveOrder order;
  std::make_heap(heap.begin(), heap.end(), order);
  while (heap_end > 0) {
    std::pop_heap(heap.begin(), heap.begin() + heap_end, order);
    heap_end--;
    const std::pair<double, size_t> best = heap[heap_end];
    if (best.first < 0 || current == scores[best.second]) break;
    std::vector<std::pair<double, size_t>> new_moves;
    if (!sc.valid(best.second, best.first)) continue;
    sc.remove((uint32_t)best.second, new_moves);
    for (size_t k = 0; k < new_moves.size(); ++k) {
      if (heap_end < heap.size()) {
        heap_end++;
        heap[heap_end - 1] = new_moves[k];
        std::push_heap(heap.begin(), heap.begin() + heap_end, order);
      } else {
        const size_t prev_size = heap.size();
        heap.insert(heap.end(), new_moves.begin() + k, new_moves.end());
        for (size_t d = 0; d < new_moves.size() - k; ++d)
          std::push_heap(heap.begin(), heap.begin() + prev_size + d + 1, order);
        heap_end = heap.size();
        break;
      }
    }
    current -= scores[best.second];
    std::vector<std::pair<uint32_t, uint32_t>> remaps;
    std::vector<uint32_t> impact;
    remove_and_coalesce(best.second, adj, scores, remaps, impact);
  }
}

// MatchStartComparator(0) for two-genome matches (its sequence-precedence
// test compares a match with itself, so it is always a tie).
struct StartOrder {
  const std::vector<Mt>* m;
  bool operator()(uint32_t x, uint32_t y) const {
    const Mt& a = (*m)[x];
    const Mt& b = (*m)[y];
    for (int q = 0; q < kSeqs; ++q) {
      const uint64_t as = orient(a, q) == kFwd ? left_end(a, q) : (left_end(a, q) ? left_end(a, q) + a.len - 1 : 0);
      const uint64_t bs = orient(b, q) == kFwd ? left_end(b, q) : (left_end(b, q) ? left_end(b, q) + b.len - 1 : 0);
      if (as == 0 || bs == 0 || as == bs) continue;
      return as < bs;
    }
    return false;
  }
};

void filter_matches(const std::vector<Mt>& M, std::vector<Lcb>& adj, std::vector<MatchList>& lcbs,
                    std::vector<double>& weights, MatchList& deleted) {
  if (lcbs.empty()) return;
  std::vector<MatchList> filtered(lcbs.size());
  for (uint32_t i = 0; i < adj.size(); ++i) {
    if ((uint32_t)adj[i].lcb_id == i) {
      filtered[i].insert(filtered[i].end(), lcbs[i].begin(), lcbs[i].end());
      continue;
    }
    if (adj[i].lcb_id == -1) continue;
    if (adj[i].lcb_id == -2) {
      deleted.insert(deleted.end(), lcbs[i].begin(), lcbs[i].end());
      continue;
    }
    std::stack<uint32_t> visited;
    visited.push(i);
    uint32_t cur = (uint32_t)adj[i].lcb_id;
    while ((uint32_t)adj[cur].lcb_id != cur) {
      visited.push(cur);
      cur = (uint32_t)adj[cur].lcb_id;
      if (cur == kNone || cur == (uint32_t)-2) break;
    }
    while (!visited.empty()) {
      adj[visited.top()].lcb_id = (int)cur;
      visited.pop();
    }
    if (cur != kNone && cur != (uint32_t)-2)
      filtered[cur].insert(filtered[cur].end(), lcbs[i].begin(), lcbs[i].end());
    else
      deleted.insert(deleted.end(), lcbs[i].begin(), lcbs[i].end());
  }
  lcbs.clear();
  std::vector<double> nw;
  for (size_t i = 0; i < filtered.size(); ++i) {
    if (filtered[i].empty()) continue;
    lcbs.push_back(filtered[i]);
    nw.push_back(weights[i]);
  }
  for (MatchList& l : lcbs) std::sort(l.begin(), l.end(), StartOrder{&M});
  weights = nw;
  compute_adjacencies(M, lcbs, weights, adj);
}

}  // namespace
}  // namespace mvg

using namespace mvg;

extern "C" int mvg_collinear_lcbs(const int64_t* matches, uint64_t n, int64_t* out, uint64_t* lcb_off,
                                  uint64_t lcb_cap, uint64_t* nlcb, int64_t* deleted, uint64_t* ndeleted) {
  if (!nlcb || !ndeleted || (n && (!matches || !out || !deleted)) || (lcb_cap && !lcb_off))
    return report_error(MVG_ERR_ARG, "bad argument");
  if (n >= 0xffffffffull) return report_error(MVG_ERR_ARG, "too many matches");
  std::vector<Mt> M(n);
  for (uint64_t i = 0; i < n; ++i) {
    M[i] = Mt{{matches[3 * i], matches[3 * i + 1]}, matches[3 * i + 2]};
    if (M[i].s[0] == 0 || M[i].s[1] == 0 || M[i].len <= 0)
      return report_error(MVG_ERR_ARG, "matches must be defined in both genomes with a positive length");
  }
  MatchList ml(n);
  for (uint64_t i = 0; i < n; ++i) ml[i] = (uint32_t)i;
  std::vector<uint64_t> bps;
  identify_breakpoints(M, ml, bps);
  std::vector<MatchList> lcbs;
  compute_lcbs(ml, bps, lcbs);
  std::vector<double> scores(lcbs.size());
  double penalty = 100;  // "anything > 0 would work" (LM/ProgressiveAligner.cpp:2288)
  for (size_t k = 0; k < lcbs.size(); ++k) {
    scores[k] = (double)coverage(M, lcbs[k]);
    penalty += scores[k];
  }
  std::vector<Lcb> adj;
  compute_adjacencies(M, lcbs, scores, adj);
  Scorer sc(adj, penalty, true);
  greedy_elimination(adj, scores, sc);
  MatchList del;
  filter_matches(M, adj, lcbs, scores, del);
  // out: every LCB's matches in order, then lcb_off
  uint64_t at = 0;
  *nlcb = lcbs.size();
  if (lcbs.size() + 1 > lcb_cap) return report_error(MVG_ERR_CAPACITY, "LCB offset buffer too small");
  lcb_off[0] = 0;
  for (size_t k = 0; k < lcbs.size(); ++k) {
    for (uint32_t id : lcbs[k]) {
      out[3 * at] = M[id].s[0];
      out[3 * at + 1] = M[id].s[1];
      out[3 * at + 2] = M[id].len;
      ++at;
    }
    lcb_off[k + 1] = at;
  }
  *ndeleted = del.size();
  for (size_t i = 0; i < del.size(); ++i) {
    deleted[3 * i] = M[del[i]].s[0];
    deleted[3 * i + 1] = M[del[i]].s[1];
    deleted[3 * i + 2] = M[del[i]].len;
  }
  return 0;
}
