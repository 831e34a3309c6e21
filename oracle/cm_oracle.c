/*
 * cm_oracle.c -- CPU ORACLE for the coarsening hot path.  TEST INFRASTRUCTURE
 * ONLY: it is the checker for the CUDA library, imported by the tests, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and never by the
 * product path.
 *
 * Plain single-threaded C restatements of the cuMetis coarsening steps
 * (paths inside the cuMetis project; "cu:" = cuMetis.cu):
 *   or_match_greedy    the deterministic heavy-edge matching the GPU library
 *                      computes (eligibility rules of cu:1563-1595, singleton
 *                      rule of cu:1600-1630), stated as a sequential greedy
 *                      pass over eligible edges in a fixed total order
 *   or_match_rounds    the same matching by synchronous mutual-proposal
 *                      rounds (an independent restatement used to cross-check
 *                      the greedy form and to count rounds)
 *   or_check_matching  legality of any matching (involution, edge exists,
 *                      weight cap and light-vertex rule) and maximality
 *   or_build_cmap      cu:1621-1694 (findc1..findc4) + cu:1755-1789
 *                      (inclusive scan) + cu:1304 (host exclusive scan)
 *   or_contract        cu:1006-1068 (gather) + bb_segsort (cu:1332) +
 *                      cu:1072-1271 (head flags, scan, merge) -> sorted rows
 *   or_ref_cpu_match / or_ref_cpu_contract
 *                      the reference's own CPU coarsening, cu:830-918
 *                      (random-order HEM) and cu:737-825 (hash-table
 *                      contraction), restated; used as the timed CPU baseline
 *   or_gen_rmat        the R-MAT workload generator of the library, restated
 *                      (the CPU arm's input, without the product library)
 *
 * Parity pin: tests/golden holds outputs of the reference's CPU coarsening
 * (cuMetis_cpu_match / cuMetis_cpu_create_cgraph, built from the reference
 * sources by oracle/build.py); the oracle's cmap and contraction must
 * reproduce them exactly (rows compared after sorting by coarse id).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_HEM 0
#define OR_HEM_HASH 1

/* 32-bit priority of an undirected edge (lo < hi) for the hashed tie-break.
 * Must equal cm_edge_hash() in the CUDA library. */
uint32_t or_edge_hash(uint32_t lo, uint32_t hi) {
  uint64_t x = ((uint64_t)lo << 32) | hi;
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (uint32_t)(x >> 32);
}

/* Eligibility of the pair (v,k) as in cuda_shem2 (cu:1570, cu:1583): the
 * proposer must be light (3*vwgt < maxvwgt) and the pair within the cap.  In
 * an undirected formulation a pair is eligible if either end may propose. */
static int eligible(const int32_t *vwgt, int32_t maxvwgt, int32_t v, int32_t k) {
  if (v == k) return 0;
  if ((int64_t)vwgt[v] + vwgt[k] > maxvwgt) return 0;
  return 3 * (int64_t)vwgt[v] < maxvwgt || 3 * (int64_t)vwgt[k] < maxvwgt;
}

typedef struct { int32_t w; uint32_t h; int32_t lo, hi; } or_edge;

static int edge_cmp(const void *pa, const void *pb) {
  const or_edge *a = (const or_edge *)pa, *b = (const or_edge *)pb;
  if (a->w != b->w) return a->w > b->w ? -1 : 1;       /* heavier first      */
  if (a->h != b->h) return a->h < b->h ? -1 : 1;       /* hashed tie (mode 1) */
  if (a->lo != b->lo) return a->lo < b->lo ? -1 : 1;   /* lower id first     */
  if (a->hi != b->hi) return a->hi < b->hi ? -1 : 1;
  return 0;
}

/* Deterministic heavy-edge matching: greedy over eligible edges sorted by
 * (weight desc, [hash asc,] lo asc, hi asc).  With mode OR_HEM the order
 * among equal weights is "lower vertex id first" from either endpoint's view.
 * Unmatched vertices end as singletons, match[v] = v (cu:1621-1630).
 * Returns the number of matched pairs. */
int64_t or_match_greedy(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *adjwgt,
                        const int32_t *vwgt, int32_t maxvwgt, int32_t mode, int32_t *match) {
  int64_t ne = 0, pairs = 0;
  for (int32_t v = 0; v < n; ++v)
    for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j)
      if (adjncy[j] > v && eligible(vwgt, maxvwgt, v, adjncy[j])) ++ne;
  or_edge *e = (or_edge *)malloc(sizeof(or_edge) * (size_t)(ne ? ne : 1));
  if (!e) return -1;
  ne = 0;
  for (int32_t v = 0; v < n; ++v)
    for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) {
      int32_t k = adjncy[j];
      if (k > v && eligible(vwgt, maxvwgt, v, k)) {
        e[ne].w = adjwgt[j];
        e[ne].h = mode == OR_HEM_HASH ? or_edge_hash((uint32_t)v, (uint32_t)k) : 0;
        e[ne].lo = v; e[ne].hi = k;
        ++ne;
      }
    }
  qsort(e, (size_t)ne, sizeof(or_edge), edge_cmp);
  for (int32_t v = 0; v < n; ++v) match[v] = -1;
  for (int64_t i = 0; i < ne; ++i)
    if (match[e[i].lo] == -1 && match[e[i].hi] == -1) {
      match[e[i].lo] = e[i].hi;
      match[e[i].hi] = e[i].lo;
      ++pairs;
    }
  for (int32_t v = 0; v < n; ++v)
    if (match[v] == -1) match[v] = v;
  free(e);
  return pairs;
}

/* True if edge (v,a) precedes edge (v,b) in the matching order. */
static int better(int32_t mode, int32_t v, int32_t wa, int32_t a, int32_t wb, int32_t b) {
  if (wa != wb) return wa > wb;
  if (mode == OR_HEM_HASH) {
    uint32_t ha = or_edge_hash((uint32_t)(v < a ? v : a), (uint32_t)(v < a ? a : v));
    uint32_t hb = or_edge_hash((uint32_t)(v < b ? v : b), (uint32_t)(v < b ? b : v));
    if (ha != hb) return ha < hb;
    int32_t la = v < a ? v : a, lb = v < b ? v : b;
    if (la != lb) return la < lb;
  }
  return a < b;
}

/* The same matching by synchronous rounds: every unmatched vertex points at
 * its best eligible unmatched neighbour; mutual pointers become pairs.
 * Returns the number of rounds until no vertex can point anywhere. */
int32_t or_match_rounds(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *adjwgt,
                        const int32_t *vwgt, int32_t maxvwgt, int32_t mode, int32_t max_rounds,
                        int32_t *match) {
  int32_t *ptr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  int32_t rounds = 0;
  for (int32_t v = 0; v < n; ++v) match[v] = -1;
  for (;;) {
    int any = 0;
    for (int32_t v = 0; v < n; ++v) {
      ptr[v] = -1;
      if (match[v] != -1) continue;
      int32_t best = -1, bw = 0;
      for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) {
        int32_t k = adjncy[j];
        if (match[k] != -1 || !eligible(vwgt, maxvwgt, v, k)) continue;
        if (best < 0 || better(mode, v, adjwgt[j], k, bw, best)) { best = k; bw = adjwgt[j]; }
      }
      ptr[v] = best;
      any |= best >= 0;
    }
    if (!any || rounds >= max_rounds) break;
    ++rounds;
    for (int32_t v = 0; v < n; ++v)
      if (ptr[v] >= 0 && ptr[ptr[v]] == v) match[v] = ptr[v];
  }
  for (int32_t v = 0; v < n; ++v)
    if (match[v] == -1) match[v] = v;
  free(ptr);
  return rounds;
}

/* Legality of a matching (match[v] = partner or v).  With require_light the
 * pair rule is the GPU path's (one end light, cu:1570); without it only the
 * weight cap (the reference's CPU matching, cu:862).  Returns 0 if legal,
 * otherwise the first offending vertex's class:
 *   1 not an involution / out of range, 2 partner not adjacent,
 *   3 weight cap or light rule violated.
 * *maximal_out = 1 if no eligible edge joins two singletons. */
int32_t or_check_matching(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *vwgt,
                          int32_t maxvwgt, int32_t require_light, const int32_t *match, int32_t *bad_vertex,
                          int32_t *maximal_out) {
  int32_t maximal = 1;
  for (int32_t v = 0; v < n; ++v) {
    int32_t u = match[v];
    if (u < 0 || u >= n || match[u] != v) { if (bad_vertex) *bad_vertex = v; return 1; }
    if (u != v) {
      int found = 0;
      for (int32_t j = xadj[v]; j < xadj[v + 1] && !found; ++j) found = adjncy[j] == u;
      if (!found) { if (bad_vertex) *bad_vertex = v; return 2; }
      const int ok = require_light ? eligible(vwgt, maxvwgt, v, u) : (int64_t)vwgt[v] + vwgt[u] <= maxvwgt;
      if (!ok) { if (bad_vertex) *bad_vertex = v; return 3; }
    } else {
      for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) {
        int32_t k = adjncy[j];
        if (match[k] == k && eligible(vwgt, maxvwgt, v, k)) maximal = 0;
      }
    }
  }
  if (maximal_out) *maximal_out = maximal;
  return 0;
}

/* Coarse-vertex map (cu:1634-1694 with the scans of cu:1758 and cu:1304):
 * leader flag v <= match[v]; cmap[leader] = number of leaders before it;
 * followers take their leader's id; leader[c], cvwgt[c] (the pair sum of
 * cu:1061-1066) and eoff[c] = exclusive prefix of deg(leader)+deg(follower).
 * Returns n' (cnvtxs). */
int32_t or_build_cmap(int32_t n, const int32_t *xadj, const int32_t *vwgt, const int32_t *match,
                      int32_t *cmap, int32_t *leader, int32_t *cvwgt, int32_t *eoff) {
  int32_t c = 0;
  int64_t off = 0;
  for (int32_t v = 0; v < n; ++v) {
    int32_t u = match[v];
    if (v <= u) {
      cmap[v] = c;
      if (leader) leader[c] = v;
      if (cvwgt) cvwgt[c] = (int32_t)((uint32_t)vwgt[v] + (u != v ? (uint32_t)vwgt[u] : 0u));
      if (eoff) eoff[c] = (int32_t)off;
      off += (xadj[v + 1] - xadj[v]) + (u != v ? xadj[u + 1] - xadj[u] : 0);
      ++c;
    }
  }
  if (eoff) eoff[c] = (int32_t)off;
  for (int32_t v = 0; v < n; ++v)
    if (v > match[v]) cmap[v] = cmap[match[v]];
  return c;
}

typedef struct { int32_t key, w; } or_kv;
static int kv_cmp(const void *pa, const void *pb) {
  const or_kv *a = (const or_kv *)pa, *b = (const or_kv *)pb;
  return a->key < b->key ? -1 : (a->key > b->key);
}

/* Contraction given match and cmap (the contract of cu:1006-1271): row c
 * gathers (cmap[x], w) over the leader's then the follower's entries
 * (cu:1014-1020), drops self loops (cu:1100, 1222), sorts by coarse id
 * (bb_segsort, cu:1332) and merges equal ids, summing weights (cu:1196-1271).
 * cxadj has n'+1 entries; cadjncy/cadjwgt capacity m.  Returns m'. */
int64_t or_contract(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *adjwgt,
                    const int32_t *match, const int32_t *cmap, int32_t cnvtxs, const int32_t *leader,
                    int32_t *cxadj, int32_t *cadjncy, int32_t *cadjwgt) {
  (void)n;
  int64_t out = 0;
  int32_t maxrow = 0;
  for (int32_t c = 0; c < cnvtxs; ++c) {
    int32_t l = leader[c], f = match[l];
    int32_t len = (xadj[l + 1] - xadj[l]) + (f != l ? xadj[f + 1] - xadj[f] : 0);
    if (len > maxrow) maxrow = len;
  }
  or_kv *row = (or_kv *)malloc(sizeof(or_kv) * (size_t)(maxrow ? maxrow : 1));
  cxadj[0] = 0;
  for (int32_t c = 0; c < cnvtxs; ++c) {
    int32_t l = leader[c], f = match[l], len = 0;
    for (int pass = 0; pass < 2; ++pass) {
      int32_t v = pass ? f : l;
      if (pass && f == l) break;
      for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) {
        int32_t k = cmap[adjncy[j]];
        if (k == c) continue;
        row[len].key = k; row[len].w = adjwgt[j]; ++len;
      }
    }
    qsort(row, (size_t)len, sizeof(or_kv), kv_cmp);
    for (int32_t i = 0; i < len; ++i) {
      if (i > 0 && row[i].key == row[i - 1].key) {
        cadjwgt[out - 1] = (int32_t)((uint32_t)cadjwgt[out - 1] + (uint32_t)row[i].w);
      } else {
        cadjncy[out] = row[i].key; cadjwgt[out] = row[i].w; ++out;
      }
    }
    cxadj[c + 1] = (int32_t)out;
  }
  free(row);
  return out;
}

/* ---------------------------------------------------------------------- */
/* Restatement of the reference's CPU coarsening (cu:639-692, 737-918).     */
/* ---------------------------------------------------------------------- */
static int32_t rand_in_range(int32_t max) { return (int32_t)((uint32_t)rand() % (uint32_t)max); }

/* cu:639-668: identity then nvtxs/8 rounds of 4-wide random swaps. */
static void rand_perm(int32_t n, int32_t *p, int32_t nshuffles) {
  for (int32_t i = 0; i < n; ++i) p[i] = i;
  if (n < 10) {
    for (int32_t i = 0; i < n; ++i) {
      int32_t v = rand_in_range(n), u = rand_in_range(n), t = p[v];
      p[v] = p[u]; p[u] = t;
    }
  } else {
    for (int32_t i = 0; i < nshuffles; ++i) {
      int32_t v = rand_in_range(n - 3), u = rand_in_range(n - 3), t;
      t = p[v + 0]; p[v + 0] = p[u + 2]; p[u + 2] = t;
      t = p[v + 1]; p[v + 1] = p[u + 3]; p[u + 3] = t;
      t = p[v + 2]; p[v + 2] = p[u + 0]; p[u + 0] = t;
      t = p[v + 3]; p[v + 3] = p[u + 1]; p[u + 1] = t;
    }
  }
}

/* cu:830-887: visit order = random permutation bucketed by clipped degree;
 * each unmatched vertex takes its first heaviest unmatched neighbour within
 * the cap; cmap in leader order.  Uses the C library rand() stream, which the
 * caller seeds with srand().  Returns n'. */
int32_t or_ref_cpu_match(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *adjwgt,
                         const int32_t *vwgt, int32_t maxvwgt, int32_t *match, int32_t *cmap) {
  int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  int32_t *tperm = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  int32_t *d = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  rand_perm(n, tperm, n / 8);
  int32_t aved = (int32_t)(0.7 * (xadj[n] / n));
  int32_t *counts = (int32_t *)calloc((size_t)aved + 2, sizeof(int32_t));
  for (int32_t i = 0; i < n; ++i) {
    int32_t dg = xadj[i + 1] - xadj[i];
    d[i] = dg > aved ? aved : dg;
    counts[d[i]]++;
  }
  /* counting sort by d, stable in tperm order (cu:671-687) */
  for (int32_t i = 1; i < aved + 1; ++i) counts[i] += counts[i - 1];
  for (int32_t i = aved + 1; i > 0; --i) counts[i] = counts[i - 1];
  counts[0] = 0;
  for (int32_t ii = 0; ii < n; ++ii) { int32_t i = tperm[ii]; perm[counts[d[i]]++] = i; }
  for (int32_t v = 0; v < n; ++v) match[v] = -1;
  int32_t cn = 0;
  for (int32_t pi = 0; pi < n; ++pi) {
    int32_t i = perm[pi];
    if (match[i] != -1) continue;
    int32_t maxidx = i, maxwgt = -1;
    for (int32_t j = xadj[i]; j < xadj[i + 1]; ++j) {
      int32_t k = adjncy[j];
      if (match[k] == -1 && maxwgt < adjwgt[j] && vwgt[i] + vwgt[k] <= maxvwgt) { maxidx = k; maxwgt = adjwgt[j]; }
      if (maxidx == i && 3 * vwgt[i] < maxvwgt) maxidx = -1;
    }
    if (maxidx != -1) { cmap[i] = cmap[maxidx] = cn++; match[i] = maxidx; match[maxidx] = i; }
  }
  cn = 0;
  for (int32_t i = 0; i < n; ++i) {
    if (match[i] == -1) { match[i] = i; cmap[i] = cn++; }
    else if (i <= match[i]) { cmap[i] = cmap[match[i]] = cn++; }
  }
  free(perm); free(tperm); free(d); free(counts);
  return cn;
}

/* cu:737-825: hash-table contraction, rows in first-seen order; the self
 * loop is removed only for matched pairs (cu:800-804).  Returns m'. */
int64_t or_ref_cpu_contract(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *adjwgt,
                            const int32_t *vwgt, const int32_t *match, const int32_t *cmap, int32_t cnvtxs,
                            int32_t *cxadj, int32_t *cvwgt, int32_t *cadjncy, int32_t *cadjwgt) {
  int32_t *htable = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cnvtxs ? cnvtxs : 1));
  for (int32_t i = 0; i < cnvtxs; ++i) htable[i] = -1;
  int64_t cne = 0;
  int32_t c = 0;
  cxadj[0] = 0;
  for (int32_t v = 0; v < n; ++v) {
    int32_t u = match[v];
    if (u < v) continue;
    int32_t *rk = cadjncy + cne, *rw = cadjwgt + cne, ne = 0;
    cvwgt[c] = vwgt[v];
    for (int pass = 0; pass < 2; ++pass) {
      int32_t x = pass ? u : v;
      if (pass && u == v) break;
      if (pass) cvwgt[c] += vwgt[u];
      for (int32_t j = xadj[x]; j < xadj[x + 1]; ++j) {
        int32_t k = cmap[adjncy[j]], m = htable[k];
        if (m == -1) { rk[ne] = k; rw[ne] = adjwgt[j]; htable[k] = ne++; }
        else rw[m] += adjwgt[j];
      }
    }
    if (u != v) {
      int32_t j = htable[c];
      if (j != -1) { --ne; rk[j] = rk[ne]; rw[j] = rw[ne]; htable[c] = -1; }
    }
    for (int32_t j = 0; j < ne; ++j) htable[rk[j]] = -1;
    cne += ne;
    cxadj[++c] = (int32_t)cne;
  }
  free(htable);
  return cne;
}

/* ---------------------------------------------------------------------- */
/* One k-way refinement pass of the reference (cu:3236-3514), with the part */
/* groups run one after another in part order (the reference runs them as  */
/* concurrent threads).  Boundary: weight to other parts > weight to own;   */
/* target: first part id of largest connection if it beats the own part;    */
/* groups by target in vertex order; phase 1 moves to higher part ids,      */
/* phase 2 to lower, each only if both parts stay in their windows.         */
/* Returns the number of moves.                                             */
/* ---------------------------------------------------------------------- */
int64_t or_refine_kway(int32_t n, const int32_t *xadj, const int32_t *adjncy, const int32_t *adjwgt,
                       const int32_t *vwgt, int32_t k, int32_t *where) {
  int64_t tv = 0;
  for (int32_t v = 0; v < n; ++v) tv += vwgt[v];
  const float tp = (float)(1.0 / k);
  const float x = tp * (float)(int32_t)tv;
  const int32_t mx = (int32_t)(x * 1.03f), mn = (int32_t)(x / 1.03f);
  int64_t *pw = (int64_t *)calloc((size_t)k, sizeof(int64_t));
  int64_t *acc = (int64_t *)calloc((size_t)k, sizeof(int64_t));
  int32_t *target = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  int32_t *flag = (int32_t *)calloc((size_t)(n ? n : 1), sizeof(int32_t));
  int32_t *cnt = (int32_t *)calloc((size_t)k + 1, sizeof(int32_t));
  int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  for (int32_t v = 0; v < n; ++v) pw[where[v]] += vwgt[v];
  for (int32_t v = 0; v < n; ++v) {
    const int32_t me = where[v];
    int64_t mw = 0, ow = 0;
    for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) {
      if (where[adjncy[j]] == me) mw += adjwgt[j];
      else ow += adjwgt[j];
    }
    target[v] = me;
    if (ow > mw) {
      flag[v] = 1;
      for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) acc[where[adjncy[j]]] += adjwgt[j];
      int64_t best = acc[me];
      int32_t bp = me;
      for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) {
        const int32_t p = where[adjncy[j]];
        if (acc[p] > best || (acc[p] == best && bp != me && p < bp)) { best = acc[p]; bp = p; }
      }
      target[v] = bp;
      cnt[bp + 1]++;
      for (int32_t j = xadj[v]; j < xadj[v + 1]; ++j) acc[where[adjncy[j]]] = 0;
    }
  }
  for (int32_t t = 0; t < k; ++t) cnt[t + 1] += cnt[t];
  for (int32_t v = 0; v < n; ++v)
    if (flag[v]) order[cnt[target[v]]++] = v;   /* stable: vertex order within a group */
  for (int32_t t = k; t > 0; --t) cnt[t] = cnt[t - 1];
  cnt[0] = 0;
  int64_t moves = 0;
  for (int phase = 0; phase < 2; ++phase)
    for (int32_t t = 0; t < k; ++t)
      for (int32_t i = cnt[t]; i < cnt[t + 1]; ++i) {
        const int32_t v = order[i], me = where[v], w = vwgt[v];
        if (phase == 0 ? me >= t : me <= t) continue;
        if (pw[t] + w >= mn && pw[t] + w <= mx && pw[me] - w >= mn && pw[me] - w <= mx) {
          pw[t] += w;
          pw[me] -= w;
          where[v] = t;
          ++moves;
        }
      }
  free(pw); free(acc); free(target); free(flag); free(cnt); free(order);
  return moves;
}

/* ------------------------------------------------------------------------
 * or_gen_rmat: the R-MAT workload generator, restated from the library's
 * cm_gen_rmat (so that the CPU reference arm of the benchmark builds its
 * input without loading the product library).  Pair e of the edge list draws
 * one 64-bit splitmix64 hash per two levels from a counter; each 32-bit half
 * picks a quadrant by the thresholds a, a+b, a+b+c (most significant level
 * first); self loops and duplicates are dropped, the rest symmetrised, rows
 * sorted; weights are a hash of the undirected edge in [wmin, wmax].  The
 * arrays are malloc'd (release with or_free); returns m, or -1.
 * ---------------------------------------------------------------------- */
static uint64_t or_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static void or_radix_u64(uint64_t *a, uint64_t *tmp, int64_t n) {
  size_t *cnt = (size_t *)malloc(sizeof(size_t) << 16);
  for (int shift = 0; shift < 64; shift += 16) {
    memset(cnt, 0, sizeof(size_t) << 16);
    for (int64_t i = 0; i < n; ++i) cnt[(a[i] >> shift) & 0xffff]++;
    size_t s = 0;
    for (int d = 0; d < (1 << 16); ++d) { size_t t = cnt[d]; cnt[d] = s; s += t; }
    for (int64_t i = 0; i < n; ++i) tmp[cnt[(a[i] >> shift) & 0xffff]++] = a[i];
    uint64_t *x = a; a = tmp; tmp = x;  /* four passes: the result ends in the caller's a */
    (void)x;
  }
  free(cnt);
}

int64_t or_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed, int32_t wmin,
                    int32_t wmax, int32_t **xadj_out, int32_t **adjncy_out, int32_t **adjwgt_out) {
  if (scale < 1 || scale > 30 || edge_factor < 1 || wmin < 1 || wmax < wmin) return -1;
  const int64_t n = (int64_t)1 << scale, ne = (int64_t)edge_factor << scale;
  const uint64_t ta = (uint64_t)(a * 4294967296.0), tb = (uint64_t)((a + b) * 4294967296.0),
                 tc = (uint64_t)((a + b + c) * 4294967296.0);
  const uint64_t s0 = or_mix64(seed ^ 0x52414D4147454E31ull);
  uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * ne), *tmp = (uint64_t *)malloc(sizeof(uint64_t) * ne);
  if (!keys || !tmp) { free(keys); free(tmp); return -1; }
  for (int64_t e = 0; e < ne; ++e) {
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; l += 2) {
      const uint64_t r = or_mix64(s0 + (uint64_t)e * 32 + (uint64_t)(l >> 1));
      for (int h = 0; h < 2 && l + h < scale; ++h) {
        const uint64_t x = h ? (r >> 32) : (r & 0xffffffffu);
        const uint64_t bu = x >= tb, bv = (x >= ta && x < tb) || x >= tc;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
    }
    const uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
    keys[e] = lo == hi ? ~0ull : ((lo << 32) | hi);
  }
  or_radix_u64(keys, tmp, ne);
  free(tmp);
  int64_t w = 0;
  for (int64_t i = 0; i < ne && keys[i] != ~0ull; ++i)
    if (w == 0 || keys[i] != keys[w - 1]) keys[w++] = keys[i];
  const int64_t m = 2 * w;
  int32_t *xadj = (int32_t *)calloc(n + 1, sizeof(int32_t));
  int32_t *adjncy = (int32_t *)malloc(sizeof(int32_t) * (m > 0 ? m : 1));
  int32_t *adjwgt = (int32_t *)malloc(sizeof(int32_t) * (m > 0 ? m : 1));
  int32_t *pos = (int32_t *)malloc(sizeof(int32_t) * n);
  if (!xadj || !adjncy || !adjwgt || !pos) { free(keys); free(xadj); free(adjncy); free(adjwgt); free(pos); return -1; }
  for (int64_t i = 0; i < w; ++i) { xadj[(keys[i] >> 32) + 1]++; xadj[(keys[i] & 0xffffffffu) + 1]++; }
  for (int64_t i = 0; i < n; ++i) { xadj[i + 1] += xadj[i]; pos[i] = xadj[i]; }
  const uint64_t wseed = or_mix64(seed ^ 0x5745494748543031ull), span = (uint64_t)(wmax - wmin) + 1;
  for (int64_t i = 0; i < w; ++i) {
    const int32_t lo = (int32_t)(keys[i] >> 32), hi = (int32_t)(keys[i] & 0xffffffffu);
    const int32_t wt = wmin + (int32_t)(or_mix64(wseed ^ keys[i]) % span);
    int32_t p = pos[lo]++;
    adjncy[p] = hi; adjwgt[p] = wt;
    p = pos[hi]++;
    adjncy[p] = lo; adjwgt[p] = wt;
  }
  free(keys);
  free(pos);
  *xadj_out = xadj;
  *adjncy_out = adjncy;
  *adjwgt_out = adjwgt;
  return m;
}

void or_free(void *p) { free(p); }
