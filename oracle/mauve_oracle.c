/* CPU oracle for the pairwise anchoring and gap-alignment path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference algorithm,
 * used as the checker for the CUDA path (tests/, __graft_entry__.smoke(),
 * bench.py's CPU baseline).  The product library never links it.
 * Citations are file:line within the mauve-py source tree:
 *   LM/ = mauve/src/libMems/libMems/, MU/ = mauve/src/muscle/libMUSCLE/.
 */
#define _GNU_SOURCE
#include "mauve_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ seeds */

/* Resolved seed pattern for (weight, rank), weights 3..31, ranks 0..5.
 * Same values as getSeed() (LM/SeedMasks.h:298-321) over the pattern tables
 * of LM/SeedMasks.h:44-260, with its solid-seed fallbacks already applied
 * (a zero table entry or rank > 5 yields a solid seed). */
static const uint64_t kSeedTable[29][6] = {
    {0xb, 0x7, 0x7, 0x7, 0x7, 0x7},
    {0x3b, 0xf, 0xf, 0xf, 0xf, 0xf},
    {0x6b, 0x139, 0x193, 0x6b, 0x1f, 0x1f},
    {0x58d, 0x653, 0x1ab, 0xdb, 0x3f, 0x3f},
    {0x1953, 0x588d, 0x688b, 0x17d, 0x164d, 0x7f},
    {0x3927, 0x1ca7, 0x6553, 0xb6d, 0xff, 0xff},
    {0x7497, 0x1c927, 0x72a7, 0x6fb, 0x16ed, 0x1ff},
    {0x1d297, 0x3a497, 0xe997, 0x6d5b, 0x3ff, 0x3ff},
    {0x7954f, 0x75257, 0x1c9527, 0x5bed, 0x5b26d, 0x7ff},
    {0x7954f, 0x3d32f, 0x768b7, 0x5b56d, 0xfff, 0xfff},
    {0x792a4f, 0x1d64d7, 0x1d3597, 0x1b7db, 0x75ad7, 0x1fff},
    {0x1e6acf, 0xf59af, 0x3d4caf, 0x35ad6b, 0x3fff, 0x3fff},
    {0x7ac9af, 0x7b2a6f, 0x79aacf, 0x16df6d, 0x6b5d6b, 0x7fff},
    {0xf599af, 0xee5a77, 0x7cd59f, 0xeb5ad7, 0xffff, 0xffff},
    {0x6dbedb, 0x1ffff, 0x1ffff, 0x1ffff, 0x1ffff, 0x1ffff},
    {0x3e6b59f, 0x3eb335f, 0x7b3566f, 0x3ffff, 0x3ffff, 0x3ffff},
    {0x7b974ef, 0x7d6735f, 0x1edd74f, 0x7ffff, 0x7ffff, 0x7ffff},
    {0x1f59b35f, 0x3edcedf, 0xfae675f, 0xfffff, 0xfffff, 0xfffff},
    {0x7ddaddf, 0xaeb3f, 0x7eb76bf, 0x1fffff, 0x1fffff, 0x1fffff},
    {0x3fffff, 0x3fffff, 0x3fffff, 0x3fffff, 0x3fffff, 0x3fffff},
    {0x7fffff, 0x7fffff, 0x7fffff, 0x7fffff, 0x7fffff, 0x7fffff},
    {0xffffff, 0xffffff, 0xffffff, 0xffffff, 0xffffff, 0xffffff},
    {0x1ffffff, 0x1ffffff, 0x1ffffff, 0x1ffffff, 0x1ffffff, 0x1ffffff},
    {0x3ffffff, 0x3ffffff, 0x3ffffff, 0x3ffffff, 0x3ffffff, 0x3ffffff},
    {0x7ffffff, 0x7ffffff, 0x7ffffff, 0x7ffffff, 0x7ffffff, 0x7ffffff},
    {0xfffffff, 0xfffffff, 0xfffffff, 0xfffffff, 0xfffffff, 0xfffffff},
    {0x1fffffff, 0x1fffffff, 0x1fffffff, 0x1fffffff, 0x1fffffff, 0x1fffffff},
    {0x3fffffff, 0x3fffffff, 0x3fffffff, 0x3fffffff, 0x3fffffff, 0x3fffffff},
    {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff},
};

/* LM/SeedMasks.h:273-321 */
uint64_t mo_get_seed(int weight, int rank) {
  if (weight > 31) return 0xffffffffull;
  if (rank == INT_MAX || rank > 5 || rank < 0) return (1ull << weight) - 1;
  if (weight < 3) return 0;
  return kSeedTable[weight - 3][rank];
}

/* LM/SeedMasks.h:334-351 */
int mo_seed_length(uint64_t seed) {
  if (!seed) return 0;
  return 64 - __builtin_clzll(seed) - __builtin_ctzll(seed);
}

/* LM/SeedMasks.h:358-371 */
int mo_seed_weight(uint64_t seed) { return __builtin_popcountll(seed); }

/* LM/SeedMasks.h:389-401 */
unsigned mo_default_seed_weight(uint64_t avg_len) {
  unsigned w = (unsigned)ceil((log((double)avg_len) / log(2.0)) / 1.5);
  if (!(w & 1)) ++w;
  w = w < 5 ? 0 : w;
  if (avg_len == 0) w = 0;
  return w > 31 ? 31 : w;
}

/* ---------------------------------------------------------------- packing */

/* LM/SortedMerList.cpp:29-47 (CreateBasicDNATable) */
static uint32_t base_code(uint8_t c) {
  switch (c) {
    case 'c': case 'C': case 'b': case 'B': case 'y': case 'Y': return 1;
    case 'g': case 'G': case 's': case 'S': case 'k': case 'K': return 2;
    case 't': case 'T': return 3;
    default: return 0;
  }
}

/* LM/SortedMerList.cpp:306-319 (SetSequence) and 425-459 (translate32) */
int64_t mo_pack(const uint8_t* seq, uint64_t n, uint32_t* out) {
  uint64_t words = (n * 2) / 32 + (((n * 2) % 32) ? 1 : 0) + 2;
  memset(out, 0, words * sizeof(uint32_t));
  for (uint64_t i = 0; i < n; ++i) {
    if (seq[i] == '-') return -1;
    out[i >> 4] |= base_code(seq[i]) << (30 - 2 * (i & 15));
  }
  return (int64_t)words;
}

/* --------------------------------------------------------------- seed mers */

typedef struct {
  uint64_t seed, mer_mask, seed_mask;
  int L, w;
} seedinfo;

static seedinfo make_seedinfo(uint64_t seed) {
  seedinfo s;
  s.seed = seed;
  s.L = mo_seed_length(seed);
  s.w = mo_seed_weight(seed);
  s.mer_mask = s.L ? (~0ull << (64 - 2 * s.L)) : 0; /* LM/SortedMerList.cpp:271-282 */
  s.seed_mask = s.w ? (~0ull << (64 - 2 * s.w)) : 0;
  return s;
}

/* 32-base window at pos, masked to the seed length (LM/SortedMerList.cpp:321-343) */
static uint64_t get_mer(const uint32_t* g, uint64_t pos, uint64_t mer_mask) {
  uint64_t w = pos >> 4, bit = (pos & 15) * 2;
  uint64_t m = ((uint64_t)g[w] << 32) | g[w + 1];
  if (bit) m = (m << bit) | (g[w + 2] >> (32 - bit));
  return m & mer_mask;
}

/* Pattern-selected bases, MSB-first, left-aligned (LM/SortedMerList.cpp:726-762) */
static uint64_t seed_mer(const uint32_t* g, uint64_t pos, const seedinfo* s) {
  uint64_t m = get_mer(g, pos, s->mer_mask), out = 0;
  for (int k = 0; k < s->L; ++k) {
    if (s->seed & (1ull << (s->L - 1 - k))) out = (out << 2) | ((m >> (62 - 2 * k)) & 3);
  }
  return out << (64 - 2 * s->w);
}

/* Reverse complement, left-aligned, low bit set as strand marker
 * (LM/SortedMerList.cpp:597-615) */
static uint64_t revcomp_mer(uint64_t mer, int w) {
  uint64_t b = ~mer, c = 0;
  for (int i = 0; i < 32; ++i) {
    c |= b & 3;
    b >>= 2;
    c <<= 2;
  }
  c <<= 64 - 2 * (w + 1);
  return c | 1;
}

/* LM/SortedMerList.cpp:764-769 (GetDnaSeedMer) */
static uint64_t canon_mer(const uint32_t* g, uint64_t pos, const seedinfo* s) {
  uint64_t f = seed_mer(g, pos, s), r = revcomp_mer(f, s->w);
  return f < r ? f : r;
}

static uint32_t* pack_alloc(const uint8_t* seq, uint64_t n) {
  uint32_t* g = (uint32_t*)malloc(((n / 16) + 3) * sizeof(uint32_t));
  if (!g) return NULL;
  if (mo_pack(seq, n, g) < 0) {
    free(g);
    return NULL;
  }
  return g;
}

/* LM/SortedMerList.cpp:771-784 (FillDnaSeedSML); for a solid seed the
 * reference fills with FillDnaSML (617-724), which yields the same canonical
 * mers, and every later Read() recomputes GetDnaSeedMer (LM/MemorySML.cpp:62-84). */
int64_t mo_seed_mers(const uint8_t* seq, uint64_t n, uint64_t seed, uint64_t* mer_out) {
  seedinfo s = make_seedinfo(seed);
  if (s.L == 0 || n < (uint64_t)s.L) return 0;
  uint32_t* g = pack_alloc(seq, n);
  if (!g) return -2;
  uint64_t cnt = n - s.L + 1;
  for (uint64_t p = 0; p < cnt; ++p) mer_out[p] = canon_mer(g, p, &s);
  free(g);
  return (int64_t)cnt;
}

typedef struct {
  uint64_t key;
  uint32_t pos;
} kp_t;

static int kp_cmp(const void* x, const void* y) {
  const kp_t* a = (const kp_t*)x;
  const kp_t* b = (const kp_t*)y;
  if (a->key != b->key) return a->key < b->key ? -1 : 1;
  return a->pos < b->pos ? -1 : (a->pos > b->pos);
}

/* LM/MemorySML.cpp:45-60: fill then sort by mer.  The reference's std::sort
 * leaves equal mers in unspecified order; this restatement breaks ties by
 * position so its output is deterministic. */
int64_t mo_sml_build(const uint8_t* seq, uint64_t n, uint64_t seed, uint32_t* pos_out, uint64_t* mer_out) {
  seedinfo s = make_seedinfo(seed);
  if (s.L == 0 || n < (uint64_t)s.L) return 0;
  uint32_t* g = pack_alloc(seq, n);
  if (!g) return -2;
  uint64_t cnt = n - s.L + 1;
  kp_t* v = (kp_t*)malloc(cnt * sizeof(kp_t));
  for (uint64_t p = 0; p < cnt; ++p) {
    v[p].key = canon_mer(g, p, &s);
    v[p].pos = (uint32_t)p;
  }
  qsort(v, cnt, sizeof(kp_t), kp_cmp);
  for (uint64_t i = 0; i < cnt; ++i) {
    pos_out[i] = v[i].pos;
    if (mer_out) mer_out[i] = v[i].key;
  }
  free(v);
  free(g);
  return (int64_t)cnt;
}

/* ------------------------------------------------------------ match finding */

#define TABLE_SIZE 40000       /* LM/MemHash.h:30 DEFAULT_MEM_TABLE_SIZE */
#define MER_REPEAT_LIMIT 1000  /* LM/MatchFinder.cpp:166 */

typedef struct {
  int64_t s0, s1; /* 1-based starts, negative = reverse strand */
  int64_t len;
  int64_t off; /* generalised offset, fixed at hash time */
} mhe_t;

typedef struct {
  const uint32_t* g[2];
  uint64_t n[2];
  seedinfo s;
} mctx;

/* LM/MatchHashEntry.cpp:164-200 (Contains) for two sequences */
static int mhe_contains(const mhe_t* c, const mhe_t* m) {
  if (c->off != m->off) return 0;
  int64_t diff = m->s0 - c->s0;
  if (c->s0 == 0) return 0;
  if (diff < 0 || (uint64_t)c->len < (uint64_t)(m->len + diff)) return 0;
  int64_t diff_rc = m->len - c->len + diff;
  int64_t diff_i = m->s1 - c->s1;
  if (m->s1 == 0 && c->s1 == 0) return 1;
  if (m->s1 < 0 && diff_rc == diff_i) return 1;
  if (diff != diff_i) return 0;
  return 1;
}

/* LM/MatchHashEntry.cpp:48-67 (strict_start_lessthan_ptr) */
static int mhe_strict_lt(const mhe_t* a, const mhe_t* b, int L) {
  int64_t as[2] = {a->s0, a->s1}, bs[2] = {b->s0, b->s1};
  for (int k = 0; k < 2; ++k) {
    int64_t x = as[k], y = bs[k];
    if (x < 0) x = -x + a->len - L;
    if (y < 0) y = -y + b->len - L;
    if (x != y) return x < y;
  }
  return 0;
}

/* LM/MatchHashEntry.h:121-143 (MheCompare); every pairwise entry hits both
 * genomes with genome 0 forward, so FirstStart is 0 for all of them. */
static int mhe_less(const mhe_t* a, const mhe_t* b, int L) {
  if (mhe_contains(a, b) || mhe_contains(b, a)) return 0;
  return mhe_strict_lt(a, b, L);
}

typedef struct {
  mhe_t* v;
  int64_t n, cap;
} bucket_t;

/* The textbook lower_bound bisection (std::lower_bound): the comparator is
 * not a strict weak order, so the probe sequence itself decides which entry
 * is tested for containment and has to be followed exactly. */
static int64_t lower_bound_mhe(const bucket_t* b, const mhe_t* x, int L) {
  int64_t first = 0, len = b->n;
  while (len > 0) {
    int64_t half = len >> 1, mid = first + half;
    if (mhe_less(&b->v[mid], x, L)) {
      first = mid + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  return first;
}

/* LM/MatchFinder.h:218-374 (ExtendMatch) for two sequences, both used. */
static void extend_match(const mctx* c, mhe_t* m) {
  const int L = c->s.L;
  int64_t st[2] = {m->s0, m->s1};
  int64_t len = m->len;
  int jump = L;
  int extend_again = 0;
  for (int dir = 0; dir < 4; ++dir) {
    int64_t maxlen = dir < 2 ? (int64_t)UINT32_MAX : (int64_t)L;
    for (int k = 0; k < 2; ++k) {
      if (st[k] < 0) {
        int64_t rc_len = (int64_t)c->n[k] - len + st[k] + 1;
        if (rc_len < maxlen) maxlen = rc_len;
      } else if (st[k] - 1 < maxlen) {
        maxlen = st[k] - 1;
      }
    }
    int i = 2, j = 0;
    uint32_t extend_limit = 0, extend_attempts = 0;
    while (maxlen - jump >= 0) {
      len += jump;
      maxlen -= jump;
      for (j = 0; j < 2; ++j) {
        if (st[j] > 0) {
          st[j] -= jump;
          if (st[j] <= 0) st[j] += (int64_t)c->n[j];
        }
      }
      uint64_t mer[2];
      int par[2];
      for (int k = 0; k < 2; ++k) {
        int64_t get = st[k];
        if (get < 0) get = -get + len - L;
        uint64_t cm = canon_mer(c->g[k], (uint64_t)(get - 1), &c->s);
        par[k] = st[k] < 0 ? (int)(cm & 1) : !(cm & 1);
        mer[k] = cm & c->s.seed_mask;
      }
      i = 1;
      if (mer[0] != mer[1] || par[0] != par[1]) {
        if (dir < 2) maxlen = 0;
      } else {
        i = 2;
      }
      extend_attempts += jump;
      if (i == 2) extend_limit = extend_attempts;
      if (dir > 1 && extend_attempts == (uint32_t)L) break;
    }
    if (i < 2) {
      len -= jump;
      for (; j > 0; j--)
        if (st[j - 1] >= 0) st[j - 1] += jump;
    }
    if (dir > 1 && extend_attempts > 0) {
      if (extend_limit > 0) extend_again = 1;
      int unmatched = (int)(extend_attempts - extend_limit);
      if (i < 2) unmatched -= jump;
      len -= unmatched;
      for (j = 0; j < 2; ++j) {
        if (st[j] > 0) {
          st[j] += unmatched;
          if (st[j] > (int64_t)c->n[j]) st[j] -= (int64_t)c->n[j];
        }
      }
    }
    st[0] = -st[0]; /* Invert (LM/HybridAbstractMatch.h:206-213) */
    st[1] = -st[1];
    if (dir >= 1) jump = 1;
    if (dir == 3 && extend_again) {
      dir = -1;
      jump = L;
      extend_again = 0;
    }
  }
  m->s0 = st[0];
  m->s1 = st[1];
  m->len = len;
}

/* LM/MemHash.cpp:167-251: HashMatch -> SetDirection -> CalculateOffset ->
 * AddHashEntry (containment test, ExtendMatch, sorted insert). */
static int add_seed_pair(const mctx* c, bucket_t* table, uint32_t pa, uint32_t pb, uint64_t ca, uint64_t cb) {
  const int L = c->s.L;
  mhe_t m;
  m.s0 = (int64_t)pa + 1;
  m.s1 = (int64_t)pb + 1;
  m.len = L;
  int ref_forward = !(ca & 1); /* LM/MemHash.cpp:189-207 */
  if (ref_forward == (int)(cb & 1)) m.s1 = -m.s1;
  m.off = m.s1 - m.s0; /* LM/MatchHashEntry.cpp:141-162 */
  if (m.s1 < 0) m.off -= m.len;
  int64_t bi = ((m.off % TABLE_SIZE) + TABLE_SIZE) % TABLE_SIZE;
  bucket_t* b = &table[bi];
  int64_t at = lower_bound_mhe(b, &m, L);
  if (at != b->n && !mhe_less(&b->v[at], &m, L) && !mhe_less(&m, &b->v[at], L)) return 0;
  extend_match(c, &m);
  at = lower_bound_mhe(b, &m, L);
  if (b->n == b->cap) {
    b->cap = b->cap ? b->cap * 2 : 4;
    b->v = (mhe_t*)realloc(b->v, b->cap * sizeof(mhe_t));
  }
  memmove(&b->v[at + 1], &b->v[at], (b->n - at) * sizeof(mhe_t));
  b->v[at] = m;
  b->n++;
  return 1;
}

/* Both genomes' canonical mers sorted by seed key. */
typedef struct {
  kp_t* v[2];
  uint64_t cnt[2];
  uint32_t* g[2];
} sorted_pair;

static int build_sorted(const uint8_t* a, uint64_t na, const uint8_t* b, uint64_t nb, const seedinfo* s,
                        sorted_pair* sp) {
  const uint8_t* seqs[2] = {a, b};
  uint64_t ns[2] = {na, nb};
  memset(sp, 0, sizeof(*sp));
  for (int k = 0; k < 2; ++k) {
    sp->g[k] = pack_alloc(seqs[k], ns[k]);
    if (!sp->g[k]) return -2;
    uint64_t cnt = ns[k] >= (uint64_t)s->L ? ns[k] - s->L + 1 : 0;
    sp->cnt[k] = cnt;
    sp->v[k] = (kp_t*)malloc((cnt ? cnt : 1) * sizeof(kp_t));
    for (uint64_t p = 0; p < cnt; ++p) {
      sp->v[k][p].key = canon_mer(sp->g[k], p, s);
      sp->v[k][p].pos = (uint32_t)p;
    }
    qsort(sp->v[k], cnt, sizeof(kp_t), kp_cmp);
  }
  return 0;
}

static void free_sorted(sorted_pair* sp) {
  for (int k = 0; k < 2; ++k) {
    free(sp->v[k]);
    free(sp->g[k]);
  }
}

/* Seeds unique in both genomes, in ascending key order: the pairs that
 * SearchRange (LM/MatchFinder.cpp:172-340) hands to
 * PairwiseMatchFinder::EnumerateMatches (LM/PairwiseMatchFinder.cpp:37-71).
 * Keys are compared under the seed mask, which drops the strand bit.  A key
 * seen more than MER_REPEAT_LIMIT times is skipped by the reference; such a
 * key never has count 1 in both genomes, so it never yields a pair here. */
typedef void (*pair_cb)(void* ctx, uint32_t pa, uint32_t pb, uint64_t ca, uint64_t cb);

static void join_unique(const sorted_pair* sp, const seedinfo* s, pair_cb cb, void* ctx) {
  uint64_t i = 0, j = 0;
  const uint64_t msk = s->seed_mask;
  while (i < sp->cnt[0] && j < sp->cnt[1]) {
    uint64_t ka = sp->v[0][i].key & msk, kb = sp->v[1][j].key & msk;
    if (ka < kb) {
      while (i < sp->cnt[0] && (sp->v[0][i].key & msk) == ka) ++i;
    } else if (kb < ka) {
      while (j < sp->cnt[1] && (sp->v[1][j].key & msk) == kb) ++j;
    } else {
      uint64_t i0 = i, j0 = j;
      while (i < sp->cnt[0] && (sp->v[0][i].key & msk) == ka) ++i;
      while (j < sp->cnt[1] && (sp->v[1][j].key & msk) == kb) ++j;
      if (i - i0 == 1 && j - j0 == 1) cb(ctx, sp->v[0][i0].pos, sp->v[1][j0].pos, sp->v[0][i0].key, sp->v[1][j0].key);
    }
  }
}

typedef struct {
  uint32_t *pa, *pb;
  uint64_t n, cap;
} pair_sink;

static void sink_pair(void* ctx, uint32_t pa, uint32_t pb, uint64_t ca, uint64_t cb) {
  (void)ca;
  (void)cb;
  pair_sink* s = (pair_sink*)ctx;
  if (s->n < s->cap) {
    s->pa[s->n] = pa;
    s->pb[s->n] = pb;
  }
  s->n++;
}

int64_t mo_unique_pairs(const uint8_t* a, uint64_t na, const uint8_t* b, uint64_t nb, uint64_t seed, uint32_t* pa,
                        uint32_t* pb, uint64_t cap) {
  seedinfo s = make_seedinfo(seed);
  if (s.L == 0) return -2;
  sorted_pair sp;
  if (build_sorted(a, na, b, nb, &s, &sp)) {
    free_sorted(&sp);
    return -2;
  }
  pair_sink sink = {pa, pb, 0, cap};
  join_unique(&sp, &s, sink_pair, &sink);
  free_sorted(&sp);
  return sink.n > cap ? -1 : (int64_t)sink.n;
}

typedef struct {
  mctx c;
  bucket_t* table;
} hash_ctx;

static void hash_pair(void* ctx, uint32_t pa, uint32_t pb, uint64_t ca, uint64_t cb) {
  hash_ctx* h = (hash_ctx*)ctx;
  add_seed_pair(&h->c, h->table, pa, pb, ca, cb);
}

int64_t mo_pairwise_matches(const uint8_t* a, uint64_t na, const uint8_t* b, uint64_t nb, uint64_t seed, int64_t* out,
                            uint64_t cap) {
  seedinfo s = make_seedinfo(seed);
  if (s.L == 0) return -2;
  sorted_pair sp;
  if (build_sorted(a, na, b, nb, &s, &sp)) {
    free_sorted(&sp);
    return -2;
  }
  hash_ctx h;
  h.c.g[0] = sp.g[0];
  h.c.g[1] = sp.g[1];
  h.c.n[0] = na;
  h.c.n[1] = nb;
  h.c.s = s;
  h.table = (bucket_t*)calloc(TABLE_SIZE, sizeof(bucket_t));
  join_unique(&sp, &s, hash_pair, &h);
  /* LM/MemHash.h:182-203 (GetMatchList): bucket order, then vector order */
  uint64_t n = 0;
  for (int64_t t = 0; t < TABLE_SIZE; ++t) {
    for (int64_t k = 0; k < h.table[t].n; ++k) {
      if (n < cap) {
        out[3 * n + 0] = h.table[t].v[k].s0;
        out[3 * n + 1] = h.table[t].v[k].s1;
        out[3 * n + 2] = h.table[t].v[k].len;
      }
      ++n;
    }
    free(h.table[t].v);
  }
  free(h.table);
  free_sorted(&sp);
  return n > cap ? -1 : (int64_t)n;
}

/* ------------------------------------------------------------------ gap DP */

/* MU/nucmx.cpp:8-25: NUC_SP with the center (2 x 30) pre-added. */
static const int32_t kNucSP[4][4] = {
    {91 + 60, -114 + 60, -31 + 60, -123 + 60},
    {-114 + 60, 100 + 60, -125 + 60, -31 + 60},
    {-31 + 60, -125 + 60, 100 + 60, -114 + 60},
    {-123 + 60, -31 + 60, -114 + 60, 91 + 60},
};
#define GAP_HALF (-200) /* g_scoreGapOpen/2 with gap open -400 (MU/params.cpp:296-304, MU/profilefrommsa.cpp:291-292) */
#define NEG_INF INT32_MIN /* stands for MINUS_INFINITY (MU/intmath.h:46); absorbing under addition */

/* Absorbing addition: MINUS_INFINITY + finite stays MINUS_INFINITY in the
 * reference's float arithmetic. */
static inline int32_t sadd(int32_t a, int32_t b) { return a == NEG_INF ? NEG_INF : a + b; }

/* Traceback bit layout (MU/types.h:30-43). */
enum { TB_MM = 0, TB_DM = 1, TB_IM = 2, TB_XM = 3, TB_MD = 4, TB_MI = 8 };

/* Per-position gap penalties after SetTermGaps with TERMGAPS_Half
 * (MU/termgaps.cpp:6-38): the first position's open and (if L > 1) the last
 * position's close are free. */
static inline int32_t gap_open(int i, int L) {
  (void)L;
  return i == 0 ? 0 : GAP_HALF;
}
static inline int32_t gap_close(int i, int L) { return (i == L - 1 && L > 1) ? 0 : GAP_HALF; }

/* MU/nwsmall.cpp:500-670 (NWSmall) with extend e = 0, then
 * MU/bittraceback.cpp:138-210 (BitTraceBack).  tb may be NULL for score only. */
static int32_t nw_core(const uint8_t* A, int LA, const uint8_t* B, int LB, uint8_t* tb, char* path, int64_t* plen) {
  const int W = LB + 1;
  int32_t* Mprev = (int32_t*)malloc(sizeof(int32_t) * W);
  int32_t* Mcurr = (int32_t*)malloc(sizeof(int32_t) * W);
  int32_t* Mnext = (int32_t*)malloc(sizeof(int32_t) * W);
  int32_t* D = (int32_t*)malloc(sizeof(int32_t) * W);
#define TB(i, j) tb[(size_t)(i) * W + (j)]
#define S(i, j) kNucSP[A[i]][B[j]]
  if (tb) memset(tb, 0, (size_t)(LA + 1) * W);
  int32_t I;
  for (int j = 0; j <= LB; ++j) D[j] = NEG_INF;
  Mprev[0] = 0;
  for (int j = 1; j <= LB; ++j) Mprev[j] = NEG_INF;
  Mcurr[0] = NEG_INF;
  Mcurr[1] = S(0, 0);
  if (tb) TB(1, 1) = (TB(1, 1) & ~TB_XM) | TB_MM;
  for (int j = 2; j <= LB; ++j) {
    Mcurr[j] = S(0, j - 1) + gap_open(0, LB) + gap_close(j - 2, LB);
    if (tb) TB(1, j) = (TB(1, j) & ~TB_XM) | TB_IM;
  }
  for (int i = 1; i < LA; ++i) {
    I = NEG_INF;
    D[0] = gap_open(0, LA);
    Mcurr[0] = NEG_INF;
    if (i == 1) {
      Mcurr[1] = S(0, 0);
      if (tb) TB(i, 1) = (TB(i, 1) & ~TB_XM) | TB_MM;
    } else {
      Mcurr[1] = S(i - 1, 0) + gap_open(0, LA) + gap_close(i - 2, LA);
      if (tb) TB(i, 1) = (TB(i, 1) & ~TB_XM) | TB_DM;
    }
    for (int j = 1; j < LB; ++j) Mnext[j + 1] = S(i, j);
    const int32_t goA = gap_open(i - 1, LA), gcA = gap_close(i - 1, LA);
    for (int j = 1; j <= LB; ++j) {
      /* RECURSE_D (MU/nwsmall.cpp:68-86): ties go to the M branch */
      int32_t DD = D[j], MD = sadd(Mprev[j], goA);
      if (DD > MD) {
        D[j] = DD;
      } else {
        D[j] = MD;
        if (tb) TB(i, j) = (TB(i, j) & ~TB_MD) | TB_MD;
      }
      /* RECURSE_I (MU/nwsmall.cpp:91-107): ties go to the M branch */
      int32_t MI = sadd(Mcurr[j - 1], gap_open(j - 1, LB));
      if (MI >= I) {
        I = MI;
        if (tb) TB(i, j) = (TB(i, j) & ~TB_MI) | TB_MI;
      }
      if (j == LB) break;
      /* RECURSE_M (MU/nwsmall.cpp:112-142): prefer M, then D, then I */
      int32_t DM = sadd(D[j], gcA), IM = sadd(I, gap_close(j - 1, LB)), MM = Mcurr[j];
      uint8_t bit;
      int32_t best;
      if (MM >= DM && MM >= IM) {
        best = MM;
        bit = TB_MM;
      } else if (DM >= MM && DM >= IM) {
        best = DM;
        bit = TB_DM;
      } else {
        best = IM;
        bit = TB_IM;
      }
      Mnext[j + 1] = sadd(best, Mnext[j + 1]);
      if (tb) TB(i + 1, j + 1) = (TB(i + 1, j + 1) & ~TB_XM) | bit;
    }
    int32_t* t = Mprev;
    Mprev = Mcurr;
    Mcurr = Mnext;
    Mnext = t;
  }
  /* last row (MU/nwsmall.cpp:616-639) */
  Mcurr[0] = NEG_INF;
  if (LA > 1)
    Mcurr[1] = S(LA - 1, 0) + gap_open(0, LA) + gap_close(LA - 2, LA);
  else
    Mcurr[1] = S(LA - 1, 0) + gap_open(0, LA) + gap_close(0, LA);
  if (tb) TB(LA, 1) = (TB(LA, 1) & ~TB_XM) | TB_DM;
  const int32_t goA = gap_open(LA - 1, LA);
  for (int j = 1; j <= LB; ++j) {
    int32_t DD = D[j], MD = sadd(Mprev[j], goA);
    if (DD > MD) {
      D[j] = DD;
    } else {
      D[j] = MD;
      if (tb) TB(LA, j) = (TB(LA, j) & ~TB_MD) | TB_MD;
    }
  }
  I = NEG_INF;
  for (int j = 1; j <= LB; ++j) {
    int32_t MI = sadd(Mcurr[j - 1], gap_open(j - 1, LB));
    if (MI >= I) {
      I = MI;
      if (tb) TB(LA, j) = (TB(LA, j) & ~TB_MI) | TB_MI;
    }
  }
  int32_t MAB = Mcurr[LB], DAB = D[LB], IAB = I;
  int32_t score = MAB;
  char edge = 'M';
  if (DAB > score) {
    score = DAB;
    edge = 'D';
  }
  if (IAB > score) {
    score = IAB;
    edge = 'I';
  }
  if (tb && path) {
    /* BitTraceBack: walk back from (LA, LB), then reverse */
    int pa = LA, pb = LB;
    int64_t n = 0;
    char cur = edge;
    for (;;) {
      path[n++] = cur;
      uint8_t bits = TB(pa, pb);
      char next;
      if (cur == 'M') {
        int x = bits & TB_XM;
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
        n = -1;
        break;
      }
      cur = next;
    }
    if (n > 0)
      for (int64_t k = 0; k < n / 2; ++k) {
        char t = path[k];
        path[k] = path[n - 1 - k];
        path[n - 1 - k] = t;
      }
    *plen = n;
  }
#undef TB
#undef S
  free(Mprev);
  free(Mcurr);
  free(Mnext);
  free(D);
  return score;
}

static int valid_codes(const uint8_t* s, int n) {
  for (int i = 0; i < n; ++i)
    if (s[i] > 3) return 0;
  return 1;
}

int64_t mo_nw_align(const uint8_t* a, int la, const uint8_t* b, int lb, char* path, int32_t* score) {
  if (la <= 0 || lb <= 0 || !valid_codes(a, la) || !valid_codes(b, lb)) return -1;
  uint8_t* tb = (uint8_t*)malloc((size_t)(la + 1) * (lb + 1));
  if (!tb) return -1;
  int64_t n = 0;
  int32_t s = nw_core(a, la, b, lb, tb, path, &n);
  free(tb);
  if (score) *score = s;
  return n;
}

int32_t mo_nw_score(const uint8_t* a, int la, const uint8_t* b, int lb) {
  if (la <= 0 || lb <= 0) return NEG_INF;
  return nw_core(a, la, b, lb, NULL, NULL, NULL);
}

typedef struct {
  const uint8_t *sa, *sb;
  const uint64_t *oa, *ob, *po;
  char* paths;
  int64_t* plen;
  int32_t* scores;
  int64_t nprob;
  int64_t next;
  pthread_mutex_t mu;
} batch_ctx;

static void* batch_worker(void* p) {
  batch_ctx* c = (batch_ctx*)p;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int64_t k = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (k >= c->nprob) break;
    int la = (int)(c->oa[k + 1] - c->oa[k]), lb = (int)(c->ob[k + 1] - c->ob[k]);
    int32_t s = 0;
    int64_t n = mo_nw_align(c->sa + c->oa[k], la, c->sb + c->ob[k], lb, c->paths ? c->paths + c->po[k] : NULL, &s);
    if (!c->paths) n = 0;
    if (c->plen) c->plen[k] = n;
    if (c->scores) c->scores[k] = s;
  }
  return NULL;
}

int64_t mo_nw_batch(const uint8_t* seq_a, const uint64_t* off_a, const uint8_t* seq_b, const uint64_t* off_b,
                    int64_t nprob, char* paths, const uint64_t* path_off, int64_t* path_len, int32_t* scores,
                    int nthreads) {
  batch_ctx c;
  c.sa = seq_a;
  c.sb = seq_b;
  c.oa = off_a;
  c.ob = off_b;
  c.po = path_off;
  c.paths = paths;
  c.plen = path_len;
  c.scores = scores;
  c.nprob = nprob;
  c.next = 0;
  pthread_mutex_init(&c.mu, NULL);
  if (nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (nthreads < 1) nthreads = 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, batch_worker, &c);
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&c.mu);
  return nprob;
}
