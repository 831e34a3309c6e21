// cm_match.cu -- deterministic heavy-edge matching.
//
// Replaces (cuMetis.cu) initcuda_match (1411), the per-level bb_segsort of
// every adjacency row by weight (1723, used only to find each row's maximum),
// cuda_shem2 (1563-1595, racy plain stores), cuda_cleanv (1600) and findc1
// (1621).  Eligibility follows cuda_shem2: a pair (v,k) may match if
// vwgt[v]+vwgt[k] <= maxvwgt and one end is light (3*vwgt < maxvwgt).
//
// Rule: every vertex prefers its heaviest eligible unmatched neighbour, ties
// to the lower vertex id (CM_MATCH_HEM) or to the lower edge hash
// (CM_MATCH_HEM_HASH, then lower id).  Both orders are strict total orders on
// edges, so mutual-proposal rounds converge to the unique greedy matching of
// that order whatever the schedule.
//
// k_match_prep initialises the state, k_match_first runs the first round's
// scans at high occupancy, and one persistent cooperative kernel (1024-thread
// blocks, at most one per SM) runs the rounds; a round has three phases
// separated by grid barriers (block barriers once a round fits one block, the
// tail mode), and k_match_finish makes the unmatched vertices singletons:
//   A  full scans: every vertex in the round's scan list computes its kTop
//      best eligible unmatched candidates (cached) and points at the first.
//      Rows of <= kSerialDeg entries: one lane each; longer rows: kChunk-entry
//      chunks, one warp each, the last chunk of a row merging the chunk lists.
//   B  commits: a vertex whose pointer changed this round (scanned, or updated
//      from its cache) and whose target points back forms a pair.
//   C  filter of the active list (unmatched vertices with a candidate): a
//      vertex whose target got matched takes the next unmatched entry of its
//      cached list (candidates only disappear and eligibility is fixed, so the
//      cached order stays exact); only an exhausted, incomplete cache sends it
//      back to phase A for a full scan.
// m2[v] < 0 encodes "unmatched, vwgt = -1 - m2[v]": one 4-byte gather per
// neighbour answers both "matched?" and the weight cap.
#include <climits>

#include <algorithm>

#include "cm_ctx.h"

namespace cm {
namespace {

// Threads per block of the persistent round kernel and the blocks per SM it
// is compiled for (its grid is every resident block, up to the graph's need).
#ifndef CM_MATCH_THREADS
#define CM_MATCH_THREADS 1024
#endif
#ifndef CM_MATCH_MINBLOCKS
#define CM_MATCH_MINBLOCKS 1
#endif
constexpr int kMatchThreads = CM_MATCH_THREADS, kMatchMinBlocks = CM_MATCH_MINBLOCKS;
constexpr int64_t kWorkPerBlock = 32768;  // vertices + entries per block of the matching grid
// Rows of at most kSerialDeg entries are scanned by one lane, longer rows in
// kChunk-entry warp work items (tuning parameters, set through the build).
#ifndef CM_SERIAL_DEG
#define CM_SERIAL_DEG 16
#endif
#ifndef CM_MATCH_CHUNK
#define CM_MATCH_CHUNK 256
#endif
constexpr int kSerialDeg = CM_SERIAL_DEG;
constexpr int kChunk = CM_MATCH_CHUNK;
static_assert(kSerialDeg == 8 || kSerialDeg == 16, "CM_SERIAL_DEG: 8 or 16");
static_assert(kChunk == 128 || kChunk == 256 || kChunk == 512, "CM_MATCH_CHUNK: 128, 256 or 512");
constexpr int kTop = 4;          // cached candidates per vertex
// Tail mode (one block runs the remaining rounds) once a round has at most
// kTailItems vertices to scan, commit or filter and kTailChunks row chunks.
#ifndef CM_TAIL_ITEMS
#define CM_TAIL_ITEMS 4096
#endif
#ifndef CM_TAIL_CHUNKS
#define CM_TAIL_CHUNKS 64
#endif
constexpr long long kTailItems = CM_TAIL_ITEMS;
constexpr int kTailChunks = CM_TAIL_CHUNKS;
constexpr int kNotScanned = -2;  // top[v*kTop] before the first scan
constexpr int kUnknown = -3;     // cache slot not computed (the first scan keeps only the best)
// Candidates the first-round scans keep when every edge is eligible: short
// rows (one lane each) and chunked rows.  1 keeps only the best (later
// rescans fill the cache); kTop fills the cache at once.
#ifndef CM_FIRST_KEEP_SHORT
#define CM_FIRST_KEEP_SHORT 2
#endif
#ifndef CM_FIRST_KEEP_CHUNK
#define CM_FIRST_KEEP_CHUNK 2
#endif
constexpr int kFirstKeepShort = CM_FIRST_KEEP_SHORT, kFirstKeepChunk = CM_FIRST_KEEP_CHUNK;

struct Slot {      // lists feeding one round (double-buffered by round parity)
  int *small;      // full scans, rows <= kSerialDeg
  int *big_v, *big_base, *big_done;  // full scans, longer rows: vertex, first chunk, chunks done
  int4 *desc;      // per chunk: (vertex, first entry, end entry, row index or -1 if one chunk)
  int *upd;        // pointers already updated from the cache
  int *act;        // active list for the round's phase C
};

struct MatchArgs {
  int n;
  const int *xadj, *adjncy, *adjwgt, *vwgt;
  long long maxvwgt;
  int mode;
  int *m2, *ptr, *stamp, *top;
  Slot slot[2];
  int *nsmall, *nupd, *nact;     // [2] each
  unsigned long long *big;       // [2] = (rows << 32 | chunks)
  int *vmax;                     // largest vertex weight (zeroed before the launch)
  int *tick;                     // [2 slots][phase A chunks, phase C spans] work tickets
  int *part;                     // per chunk: kTop x (w, h, k)
  int max_rounds;
  DevStatus *st;
  unsigned long long *trace;     // optional: row 0 header, row r+1 = round r
  int trace_rows;
  // Several independent graphs side by side (a batch): vgid[v] = v's graph,
  // whose weight cap is gcap[g] and whose first vertex is gbase[g] (the edge
  // hash of the tie rule is taken on graph-local ids, so a graph matches the
  // same alone and in a batch).  Null for one graph.
  const int *vgid, *gbase, *gcap;
};

// Candidates.  Lex mode (ties to the lower id) packs (weight, ~id) into one
// 64-bit key, larger = better, 0 = none.  Hash mode compares (weight desc,
// edge hash asc, id asc) field by field.
template <bool H> struct Cand;
template <> struct Cand<false> {
  unsigned long long key = 0ull;
  __device__ __forceinline__ static Cand make(int v, int k, int w, int hb) {
    (void)v;
    (void)hb;
    Cand c;
    c.key = ((unsigned long long)((unsigned)w ^ 0x80000000u) << 32) | (unsigned)(~(unsigned)k);
    return c;
  }
  __device__ __forceinline__ bool valid() const { return key != 0ull; }
  __device__ __forceinline__ int id() const { return valid() ? (int)~(unsigned)key : -1; }
  __device__ __forceinline__ bool better(const Cand &o) const { return key > o.key; }
  __device__ __forceinline__ bool same(const Cand &o) const { return key == o.key; }
  __device__ __forceinline__ Cand warp_best() const {
    const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(key >> 32));
    const unsigned lo = __reduce_max_sync(0xffffffffu, (unsigned)(key >> 32) == hi ? (unsigned)key : 0u);
    Cand r;
    r.key = ((unsigned long long)hi << 32) | lo;
    return r;
  }
  // p: 16-byte aligned slot of kPartInts ints
  __device__ __forceinline__ void store(int *p) const { *reinterpret_cast<unsigned long long *>(p) = key; }
  __device__ __forceinline__ static Cand load(const int *p) {
    Cand c;
    c.key = __ldcg(reinterpret_cast<const unsigned long long *>(p));
    return c;
  }
};
template <> struct Cand<true> {
  int w = 0;
  unsigned h = 0u;
  int k = INT_MAX;  // INT_MAX = none
  __device__ __forceinline__ static Cand make(int v, int k, int w, int hb) {
    Cand c;
    c.w = w;
    c.k = k;
    c.h = edge_hash((unsigned)(min(v, k) - hb), (unsigned)(max(v, k) - hb));
    return c;
  }
  __device__ __forceinline__ bool valid() const { return k != INT_MAX; }
  __device__ __forceinline__ int id() const { return valid() ? k : -1; }
  __device__ __forceinline__ bool better(const Cand &o) const {
    if (k == INT_MAX) return false;
    if (o.k == INT_MAX) return true;
    if (w != o.w) return w > o.w;
    if (h != o.h) return h < o.h;
    return k < o.k;
  }
  __device__ __forceinline__ bool same(const Cand &o) const { return k == o.k && w == o.w && h == o.h; }
  __device__ __forceinline__ Cand warp_best() const {
    const unsigned full = 0xffffffffu;
    const int wmax = __reduce_max_sync(full, valid() ? w : INT_MIN);
    const bool atw = valid() && w == wmax;
    const unsigned hmin = __reduce_min_sync(full, atw ? h : 0xffffffffu);
    const bool ath = atw && h == hmin;
    const unsigned kmin = __reduce_min_sync(full, ath ? (unsigned)k : 0xffffffffu);
    Cand r;
    r.w = wmax;
    r.h = hmin;
    r.k = kmin == 0xffffffffu ? INT_MAX : (int)kmin;
    return r;
  }
  __device__ __forceinline__ void store(int *p) const { *reinterpret_cast<int4 *>(p) = make_int4(w, (int)h, k, 0); }
  __device__ __forceinline__ static Cand load(const int *p) {
    const int4 x = __ldcg(reinterpret_cast<const int4 *>(p));
    Cand c;
    c.w = x.x;
    c.h = (unsigned)x.y;
    c.k = x.z;
    return c;
  }
};
constexpr int kPartInts = 4;  // ints per stored candidate slot (16 bytes, one vector access)

// Sorted (best first) list of up to KK candidates held in registers.
template <bool H, int KK>
struct TopK {
  Cand<H> c[KK];
  __device__ __forceinline__ void insert(const Cand<H> &x) {
    if (!x.better(c[KK - 1])) return;
    Cand<H> cur = x;
#pragma unroll
    for (int i = 0; i < KK; ++i) {
      if (cur.better(c[i])) { Cand<H> t = c[i]; c[i] = cur; cur = t; }
    }
  }
  // Edge (v, k) of weight w.  In hash mode the edge hash is computed only when
  // the weight can still enter the list (a lighter edge loses to the last
  // entry whatever its hash); the result is that of insert(make(v, k, w, hb)).
  // hb: the first vertex of v's graph (0 for one graph).
  __device__ __forceinline__ void insert_edge(int v, int k, int w, int hb) {
    if constexpr (H) {
      if (c[KK - 1].valid() && w < c[KK - 1].w) return;
    }
    insert(Cand<H>::make(v, k, w, hb));
  }
};

// First vertex of v's graph (the hash base of the tie rule) and its weight cap.
__device__ __forceinline__ int hash_base(const MatchArgs &a, int v) { return a.vgid ? __ldg(a.gbase + __ldg(a.vgid + v)) : 0; }
__device__ __forceinline__ long long weight_cap(const MatchArgs &a, int v) {
  return a.vgid ? (long long)__ldg(a.gcap + __ldg(a.vgid + v)) : a.maxvwgt;
}

template <bool H>
__device__ __forceinline__ bool eligible(const MatchArgs &a, long long vw, int v, int k, int s) {
  if (k == v || s >= 0) return false;  // self or matched
  const long long vk = -1ll - s;
  const long long cap = weight_cap(a, v);
  if (vw + vk > cap) return false;
  return 3 * vw < cap || 3 * vk < cap;
}

// Merges the lanes' sorted lists into the warp's best KK (all lanes get it).
template <bool H, int KK>
__device__ __forceinline__ TopK<H, KK> warp_topk(const TopK<H, KK> &t) {
  TopK<H, KK> out;
  int head = 0;
#pragma unroll
  for (int i = 0; i < KK; ++i) {
    Cand<H> mine;
#pragma unroll
    for (int j = 0; j < KK; ++j)
      if (j == head) mine = t.c[j];
    const Cand<H> win = mine.warp_best();
    out.c[i] = win;
    if (win.valid() && mine.same(win)) ++head;
  }
  return out;
}

// The warp's best KK of the cnt candidates stored at slots slot(t), t < cnt,
// of the chunk partial lists (four loads in flight per lane).
template <bool H, int KK, typename F>
__device__ __forceinline__ TopK<H, KK> merge_parts(const MatchArgs &a, int cnt, F slot) {
  const int lane = threadIdx.x & 31;
  TopK<H, KK> acc;
  for (int t0 = lane; t0 < cnt; t0 += 128) {
    Cand<H> c[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int t = t0 + 32 * i;
      if (t < cnt) c[i] = Cand<H>::load(a.part + slot(t) * kPartInts);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) acc.insert(c[i]);
  }
  return warp_topk(acc);
}

// Per-lane best KK over entries [b, e) (e - b <= kChunk) of v's row; all loads
// of the chunk are issued before any is used.
template <bool H, int KK>
__device__ __forceinline__ TopK<H, KK> lane_scan(const MatchArgs &a, int v, long long vw, int b, int e,
                                                 bool all_elig = false) {
  const int lane = threadIdx.x & 31;
  constexpr int U = kChunk / 32;
  const int nu = (e - b + 31) >> 5;  // slots holding entries (warp-uniform): the others are skipped
  int k[U], w[U], s[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int j = b + lane + 32 * u;
    k[u] = -1;
    w[u] = 0;
    if (u < nu && j < e) {
      k[u] = a.adjncy[j];
      w[u] = a.adjwgt[j];
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) s[u] = (u < nu && k[u] >= 0 && !all_elig) ? __ldcg(a.m2 + k[u]) : -1;
  TopK<H, KK> t;
  const int hb = hash_base(a, v);
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (u < nu && k[u] >= 0 && (all_elig ? k[u] != v : eligible<H>(a, vw, v, k[u], s[u])))
      t.insert_edge(v, k[u], w[u], hb);
  return t;
}

// Inserts x into the descending list tw (the KK largest values seen, with
// repeats).
template <int KK>
__device__ __forceinline__ void wlist_insert(int (&tw)[KK], int x) {
#pragma unroll
  for (int i = 0; i < KK; ++i) {
    const int hi = max(tw[i], x);
    x = min(tw[i], x);
    tw[i] = hi;
  }
}

// The warp's best KK candidates over entries [b, e) (e - b <= kChunk) of v's
// row; every lane gets the list.  Hash order: most entries are lighter than
// the chunk's KK-th heaviest eligible entry and can never enter the list, so
// a weight threshold W is found first and only entries of weight >= W get an
// edge hash and a full comparison.  W is the KK-th largest weight of the
// union of the lanes' own KK heaviest (a sub-multiset of the chunk), so at
// least KK entries weigh >= W and the chunk's best KK are all among them.
// The qualifying entries (usually KK plus the ties at W) are packed one per
// lane through the warp's 32-entry buffer wbuf; more than 32 of them (many
// equal weights) take the per-lane lists instead.
template <bool H, int KK>
__device__ __forceinline__ TopK<H, KK> chunk_best(const MatchArgs &a, int v, long long vw, int b, int e, bool all_elig,
                                                  int2 *wbuf) {
  if constexpr (!H) {
    (void)wbuf;
    return warp_topk(lane_scan<H, KK>(a, v, vw, b, e, all_elig));
  } else {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    constexpr int U = kChunk / 32;
    const int nu = (e - b + 31) >> 5;  // slots holding entries (warp-uniform): the others are skipped
    int k[U], w[U], s[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = b + lane + 32 * u;
      k[u] = -1;
      w[u] = 0;
      if (u < nu && j < e) {
        k[u] = a.adjncy[j];
        w[u] = a.adjwgt[j];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) s[u] = (u < nu && k[u] >= 0 && !all_elig) ? __ldcg(a.m2 + k[u]) : -1;
    // k[u] = -1 marks an entry that is not an eligible candidate
    int tw[KK], rem = 0;
#pragma unroll
    for (int i = 0; i < KK; ++i) tw[i] = INT_MIN;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (u >= nu) break;
      if (k[u] >= 0 && !(all_elig ? k[u] != v : eligible<H>(a, vw, v, k[u], s[u]))) k[u] = -1;
      if (k[u] >= 0) {
        wlist_insert(tw, w[u]);
        ++rem;
      }
    }
    rem = min(rem, KK);
    // threshold: pop the lanes' list heads in descending order until KK
    // entries are taken (or every list is empty: then all eligible entries
    // qualify, W being the lightest of them)
    int W = INT_MIN, taken = 0;
#pragma unroll
    for (int r = 0; r < KK; ++r) {
      const bool has = rem > 0;
      if (!__ballot_sync(full, has)) break;
      const int mine = has ? tw[0] : INT_MIN;
      const int mx = __reduce_max_sync(full, mine);
      const bool pop = has && mine == mx;
      taken += __popc(__ballot_sync(full, pop));
      W = mx;
      if (pop) {
#pragma unroll
        for (int i = 0; i + 1 < KK; ++i) tw[i] = tw[i + 1];
        --rem;
      }
      if (taken >= KK) break;
    }
    int total = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (u >= nu) break;
      total += __popc(__ballot_sync(full, k[u] >= 0 && w[u] >= W));
    }
    const int hb = hash_base(a, v);
    TopK<H, KK> out;
    if (total > 32) {
      TopK<H, KK> t;
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (u < nu && k[u] >= 0 && w[u] >= W) t.insert_edge(v, k[u], w[u], hb);
      out = warp_topk(t);
    } else {
      const unsigned below = (1u << lane) - 1u;
      int base = 0;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (u >= nu) break;
        const bool q = k[u] >= 0 && w[u] >= W;
        const unsigned bal = __ballot_sync(full, q);
        if (q) wbuf[base + __popc(bal & below)] = make_int2(k[u], w[u]);
        base += __popc(bal);
      }
      __syncwarp();
      Cand<H> mine;
      if (lane < total) {
        const int2 x = wbuf[lane];
        mine = Cand<H>::make(v, x.x, x.y, hb);
      }
      __syncwarp();  // the buffer is free for the warp's next chunk
#pragma unroll
      for (int i = 0; i < KK; ++i) {
        const Cand<H> win = mine.warp_best();
        out.c[i] = win;
        if (win.valid() && mine.same(win)) mine = Cand<H>();
      }
    }
    // Identical entries (parallel edges of equal weight) count once in the
    // list but each in `taken`: a list left short although lighter entries
    // exist is recomputed over every eligible entry, so that a short list
    // still means "no other candidate".
    if (taken >= KK && !out.c[KK - 1].valid()) {
      TopK<H, KK> t;
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (u < nu && k[u] >= 0) t.insert_edge(v, k[u], w[u], hb);
      out = warp_topk(t);
    }
    return out;
  }
}

// Writes v's cached candidate ids and points v at the first.  A first scan
// (KK == 1) marks the rest of the cache unknown; a full list marks unused
// slots "none" (the cache then holds every candidate).
template <bool H, int KK>
__device__ __forceinline__ void store_top(const MatchArgs &a, int v, const TopK<H, KK> &t) {
  int q[kTop];
#pragma unroll
  for (int i = 0; i < kTop; ++i) q[i] = i < KK ? t.c[i].id() : (t.c[0].valid() ? kUnknown : -1);
  reinterpret_cast<int4 *>(a.top)[v] = make_int4(q[0], q[1], q[2], q[3]);
  a.ptr[v] = q[0];
}

__device__ __forceinline__ unsigned long long warp_excl_scan_u64(unsigned long long v, unsigned long long *total) {
  const unsigned long long inc = warp_inclusive_scan_u64(v);
  *total = __shfl_sync(0xffffffffu, inc, 31);
  return inc - v;
}

// Warp-aggregated append of x to list[counter]; convergent call.
__device__ __forceinline__ void warp_append(int *list, int *counter, bool take, int x) {
  const unsigned mask = __ballot_sync(0xffffffffu, take);
  if (!mask) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (take) list[base + __popc(mask & ((1u << lane) - 1))] = x;
}

// Chunk descriptors of the rows queued by the lanes with `take` set (row x of
// deg entries from xs, nch chunks from desc[cb], row index idx): a one-chunk
// row's lane writes its descriptor, and the warp writes each longer row's
// descriptors together.  Convergent.
__device__ __forceinline__ void write_descs(int4 *desc, bool take, int x, int xs, int deg, int nch, int idx, int cb) {
  const int lane = threadIdx.x & 31;
  if (take && nch == 1) desc[cb] = make_int4(x, xs, xs + deg, -1);
  unsigned bm = __ballot_sync(0xffffffffu, take && nch > 1);
  while (bm) {
    const int src = __ffs(bm) - 1;
    bm &= bm - 1;
    const int rx = __shfl_sync(0xffffffffu, x, src), rs = __shfl_sync(0xffffffffu, xs, src);
    const int rd = __shfl_sync(0xffffffffu, deg, src), rn = __shfl_sync(0xffffffffu, nch, src);
    const int ri = __shfl_sync(0xffffffffu, idx, src), rc = __shfl_sync(0xffffffffu, cb, src);
    for (int j = lane; j < rn; j += 32)
      desc[rc + j] = make_int4(rx, rs + j * kChunk, min(rs + rd, rs + (j + 1) * kChunk), ri);
  }
}

// Queues x (row of `deg` entries starting at xs) for a full scan in slot
// `par`; convergent.
__device__ __forceinline__ void append_scan(const MatchArgs &a, int par, bool take, int x, int xs, int deg) {
  const Slot &S = a.slot[par];
  warp_append(S.small, a.nsmall + par, take && deg <= kSerialDeg, x);
  const bool bg = take && deg > kSerialDeg;
  if (!__any_sync(0xffffffffu, bg)) return;
  const int lane = threadIdx.x & 31;
  const int nch = bg ? (deg + kChunk - 1) / kChunk : 0;
  const unsigned long long mine = bg ? ((1ull << 32) | (unsigned long long)nch) : 0ull;
  unsigned long long tot;
  const unsigned long long ex = warp_excl_scan_u64(mine, &tot);
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(a.big + par, tot);
  base = __shfl_sync(0xffffffffu, base, 0) + ex;
  const int idx = (int)(base >> 32), cb = (int)(base & 0xffffffffu);
  if (bg) {
    S.big_v[idx] = x;
    S.big_base[idx] = cb;
    S.big_done[idx] = 0;
  }
  write_descs(S.desc, bg, x, xs, deg, nch, idx, cb);
}

constexpr int kCU = 4;  // vertices per thread in phase C

// Phase C's appends for a block (all threads call it): every thread offers
// up to kCU vertices to the next round's active list (keep), cache-update
// list (upd) and scan lists (scan: the short-row list or, for longer rows,
// the chunk list with one descriptor per kChunk entries).  One block-wide
// scan of the packed per-thread counts (four 16-bit fields, block totals
// <= kMatchThreads * kCU) and of the chunk counts, then one atomicAdd per
// list, issued side by side by four lanes.
static_assert(kMatchThreads * kCU < 65536, "phase C counts are packed in 16-bit fields");
__device__ __forceinline__ void phase_c_append(const MatchArgs &a, int np, const bool (&keep)[kCU],
                                               const bool (&upd)[kCU], const bool (&scan)[kCU], const int (&x)[kCU],
                                               const int (&xs)[kCU], const int (&deg)[kCU],
                                               unsigned long long *sh_cw, int *sh_cc, unsigned long long *sh_cb) {
  constexpr int NW = kMatchThreads / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Slot &N = a.slot[np];
  unsigned long long c4 = 0ull;
  int cch = 0, nch[kCU];
#pragma unroll
  for (int u = 0; u < kCU; ++u) {
    const bool sm = scan[u] && deg[u] <= kSerialDeg, bg = scan[u] && deg[u] > kSerialDeg;
    c4 += (unsigned long long)keep[u] | ((unsigned long long)upd[u] << 16) | ((unsigned long long)sm << 32) |
          ((unsigned long long)bg << 48);
    nch[u] = bg ? (deg[u] + kChunk - 1) / kChunk : 0;
    cch += nch[u];
  }
  unsigned long long i4 = c4;
  int ic = cch;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y4 = __shfl_up_sync(0xffffffffu, i4, o);
    const int yc = __shfl_up_sync(0xffffffffu, ic, o);
    if (lane >= o) {
      i4 += y4;
      ic += yc;
    }
  }
  if (lane == 31) {
    sh_cw[warp] = i4;
    sh_cc[warp] = ic;
  }
  __syncthreads();
  if (warp == 0) {
    const unsigned long long v4 = lane < NW ? sh_cw[lane] : 0ull;
    const int vc = lane < NW ? sh_cc[lane] : 0;
    unsigned long long j4 = v4;
    int jc = vc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y4 = __shfl_up_sync(0xffffffffu, j4, o);
      const int yc = __shfl_up_sync(0xffffffffu, jc, o);
      if (lane >= o) {
        j4 += y4;
        jc += yc;
      }
    }
    const unsigned long long t4 = __shfl_sync(0xffffffffu, j4, 31);
    const int tc = __shfl_sync(0xffffffffu, jc, 31);
    if (lane < NW) {
      sh_cw[lane] = j4 - v4;
      sh_cc[lane] = jc - vc;
    }
    const int f = (int)((t4 >> (16 * (lane & 3))) & 0xffffull);
    unsigned long long gb = 0ull;
    if (lane == 0 && f) gb = (unsigned long long)atomicAdd(a.nact + np, f);
    if (lane == 1 && f) gb = (unsigned long long)atomicAdd(a.nupd + np, f);
    if (lane == 2 && f) gb = (unsigned long long)atomicAdd(a.nsmall + np, f);
    if (lane == 3 && (f || tc)) gb = atomicAdd(a.big + np, ((unsigned long long)f << 32) | (unsigned)tc);
    if (lane < 4) sh_cb[lane] = gb;
  }
  __syncthreads();
  const unsigned long long e4 = sh_cw[warp] + (i4 - c4);
  int pk = (int)sh_cb[0] + (int)(e4 & 0xffffull);
  int pu = (int)sh_cb[1] + (int)((e4 >> 16) & 0xffffull);
  int ps = (int)sh_cb[2] + (int)((e4 >> 32) & 0xffffull);
  int pb = (int)(sh_cb[3] >> 32) + (int)(e4 >> 48);
  int pc = (int)(sh_cb[3] & 0xffffffffull) + sh_cc[warp] + (ic - cch);
#pragma unroll
  for (int u = 0; u < kCU; ++u) {
    if (keep[u]) N.act[pk++] = x[u];
    if (upd[u]) N.upd[pu++] = x[u];
    if (scan[u] && deg[u] <= kSerialDeg) N.small[ps++] = x[u];
    const int idx = pb, cb = pc;
    if (nch[u] > 0) {
      ++pb;
      pc += nch[u];
      N.big_v[idx] = x[u];
      N.big_base[idx] = cb;
      N.big_done[idx] = 0;
    }
    write_descs(N.desc, nch[u] > 0, x[u], xs[u], deg[u], nch[u], idx, cb);
  }
  __syncthreads();  // the shared counts are free for the next call
}

// Phase A of a round: full scans of the rows whose candidates must be
// recomputed -- rows of <= kSerialDeg entries one lane each (the whole vertex
// range in the first round), longer rows as kChunk-entry warp chunks with a
// last-chunk merge.  `first`: the first round (keeps kFirstKeep* candidates);
// `skip_gather`: first round with every edge eligible (no neighbour state).
template <bool H>
__device__ __forceinline__ void phase_a(const MatchArgs &a, const Slot &S, bool first, bool skip_gather,
                                        long long nsmall, int nchunks, int gwarp, int nwarps, int lane, int2 *wbuf,
                                        int *tick) {
  for (long long b0 = (long long)gwarp * 32; b0 < nsmall; b0 += (long long)nwarps * 32) {
    const long long i = b0 + lane;
    if (i >= nsmall) continue;
    const int v = first ? (int)i : __ldcg(S.small + i);
    const int xs = a.xadj[v], deg = a.xadj[v + 1] - xs;
    if (first && (deg == 0 || deg > kSerialDeg)) continue;
    if (skip_gather) {  // first round, every edge eligible: ids and weights only, 8 at a time
      constexpr int kHalf = kSerialDeg / 2;
      const int hb = hash_base(a, v);
      TopK<H, kFirstKeepShort> tk;
#pragma unroll 1
      for (int t0 = 0; t0 < deg; t0 += kHalf) {
        int k[kHalf], w[kHalf];
#pragma unroll
        for (int t = 0; t < kHalf; ++t) {
          k[t] = t0 + t < deg ? a.adjncy[xs + t0 + t] : -1;
          w[t] = t0 + t < deg ? a.adjwgt[xs + t0 + t] : 0;
        }
#pragma unroll
        for (int t = 0; t < kHalf; ++t)
          if (k[t] >= 0 && k[t] != v) tk.insert_edge(v, k[t], w[t], hb);
      }
      store_top(a, v, tk);
      continue;
    }
    const int sv = __ldcg(a.m2 + v);
    if (sv >= 0) continue;
    const long long vw = -1ll - sv;
    int k[kSerialDeg], s[kSerialDeg];
#pragma unroll
    for (int t = 0; t < kSerialDeg; ++t) k[t] = t < deg ? a.adjncy[xs + t] : -1;
#pragma unroll
    for (int t = 0; t < kSerialDeg; ++t) s[t] = (k[t] >= 0 && !skip_gather) ? __ldcg(a.m2 + k[t]) : -1;
    if (first) {
      TopK<H, 1> tk;
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t)
        if (k[t] >= 0 && (skip_gather ? k[t] != v : eligible<H>(a, vw, v, k[t], s[t])))
          tk.insert_edge(v, k[t], a.adjwgt[xs + t], hash_base(a, v));
      store_top(a, v, tk);
    } else {
      TopK<H, kTop> tk;
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t)
        if (k[t] >= 0 && (skip_gather ? k[t] != v : eligible<H>(a, vw, v, k[t], s[t])))
          tk.insert_edge(v, k[t], a.adjwgt[xs + t], hash_base(a, v));
      store_top(a, v, tk);
    }
  }
  // Chunk loop driver: chunks taken from a ticket when one is given (rows of
  // very different lengths and the last chunk's merge make a fixed
  // assignment uneven; the next ticket and its descriptor are fetched before
  // the current chunk is scanned), else round robin over the warps.
  auto drive = [&](auto &&scan) {
    if (tick != nullptr) {
      int q = 0;
      if (lane == 0) q = atomicAdd(tick, 1);
      q = __shfl_sync(0xffffffffu, q, 0);
      int4 d = q < nchunks ? __ldcg(S.desc + q) : make_int4(0, 0, 0, 0);
      while (q < nchunks) {
        int qn = 0;
        if (lane == 0) qn = atomicAdd(tick, 1);
        qn = __shfl_sync(0xffffffffu, qn, 0);
        const int4 dn = qn < nchunks ? __ldcg(S.desc + qn) : d;
        scan(q, d);
        q = qn;
        d = dn;
      }
    } else {
      int4 d = gwarp < nchunks ? __ldcg(S.desc + gwarp) : make_int4(0, 0, 0, 0);
      for (int q = gwarp; q < nchunks; q += nwarps) {
        const int4 dn = q + nwarps < nchunks ? __ldcg(S.desc + q + nwarps) : d;
        scan(q, d);
        d = dn;
      }
    }
  };
  if (skip_gather) {
    // First round, every edge eligible: no neighbour state; multi-chunk rows
    // merge one partial per chunk.
    drive([&](int q, const int4 &d) {
      const int v = d.x, i = d.w;
      constexpr int KC = kFirstKeepChunk;
      const TopK<H, KC> r1 = chunk_best<H, KC>(a, v, 0, d.y, d.z, true, wbuf);
      if (i < 0) {
        if (lane == 0) store_top(a, v, r1);
        return;
      }
      const int nch = (a.xadj[v + 1] - a.xadj[v] + kChunk - 1) / kChunk;
      int last = 0;
      if (lane < KC) {
        Cand<H> mine = r1.c[0];
#pragma unroll
        for (int t = 1; t < KC; ++t)
          if (lane == t) mine = r1.c[t];
        mine.store(a.part + ((size_t)q * kTop + lane) * kPartInts);
      }
      if (lane == 0) {
        __threadfence();
        last = atomicAdd(S.big_done + i, 1) == nch - 1;
      }
      last = __shfl_sync(0xffffffffu, last, 0);
      if (last) {
        __threadfence();
        const int base = __ldcg(S.big_base + i);
        const TopK<H, KC> rr =
            merge_parts<H, KC>(a, nch * KC, [&](int t) { return (size_t)(base + t / KC) * kTop + t % KC; });
        if (lane == 0) store_top(a, v, rr);
      }
    });
    return;
  }
  // Scans with the neighbours' state.  A vertex of a scan list is unmatched
  // (the lists are built after the previous round's commits), so its row's
  // loads are issued together with its own state.
  auto scan_chunk = [&](int q, const int4 &d) {
    const int v = d.x, i = d.w;
    const int sv = __ldcg(a.m2 + v);
    const long long vw = -1ll - sv;
    TopK<H, kTop> r;
    if (first) {
      const TopK<H, 1> r1 = chunk_best<H, 1>(a, v, vw, d.y, d.z, skip_gather, wbuf);
      r.c[0] = r1.c[0];
    } else {
      r = chunk_best<H, kTop>(a, v, vw, d.y, d.z, false, wbuf);
    }
    if (sv >= 0) return;  // (not expected) uniform per warp, and alike for all chunks of the row
    if (i < 0) {  // the row's only chunk
      if (lane == 0) {
        if (first) {
          TopK<H, 1> r1;
          r1.c[0] = r.c[0];
          store_top(a, v, r1);
        } else {
          store_top(a, v, r);
        }
      }
      return;
    }
    const int nch = (a.xadj[v + 1] - a.xadj[v] + kChunk - 1) / kChunk;
    int last = 0;
    if (lane < kTop) {
      Cand<H> mine = r.c[0];
#pragma unroll
      for (int t = 1; t < kTop; ++t)
        if (lane == t) mine = r.c[t];
      mine.store(a.part + ((size_t)q * kTop + lane) * kPartInts);
    }
    if (lane == 0) {
      __threadfence();
      last = atomicAdd(S.big_done + i, 1) == nch - 1;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {  // merge the row's chunk lists
      __threadfence();
      const int base = __ldcg(S.big_base + i);
      const TopK<H, kTop> rr = merge_parts<H, kTop>(a, nch * kTop, [&](int t) { return (size_t)base * kTop + t; });
      if (lane == 0) {
        if (first) {
          TopK<H, 1> r1;
          r1.c[0] = rr.c[0];
          store_top(a, v, r1);
        } else {
          store_top(a, v, rr);
        }
      }
    }
  };
  drive(scan_chunk);
}

// Before the rounds: initial state of every vertex (unmatched, no
// candidate), the largest vertex weight, and the first round's chunk list of
// rows longer than kSerialDeg.  The list counters are zeroed by the host.
constexpr int kPrepThreads = 256;
// Resident blocks per SM the first-round kernel is compiled for (register cap).
#ifndef CM_FIRST_MINBLOCKS
#define CM_FIRST_MINBLOCKS 8
#endif
constexpr int kFirstMinBlocks = CM_FIRST_MINBLOCKS;
template <bool H>
__global__ void __launch_bounds__(kPrepThreads) k_match_prep(MatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const int n = a.n;
  int wmax = 0;
  for (long long b0 = (long long)gwarp * 32; b0 < n; b0 += (long long)nwarps * 32) {
    const long long v = b0 + lane;
    int xs = 0, deg = 0;
    if (v < n) {
      const int vw0 = a.vwgt[v];
      wmax = max(wmax, vw0);
      a.m2[v] = -1 - vw0;
      a.ptr[v] = -1;
      a.stamp[v] = 0;
      a.top[v * kTop] = kNotScanned;
      xs = a.xadj[v];
      deg = a.xadj[v + 1] - xs;
    }
    append_scan(a, 0, deg > kSerialDeg, (int)v, xs, deg);
  }
  wmax = __reduce_max_sync(0xffffffffu, wmax);
  if (lane == 0 && wmax > 0) atomicMax(a.vmax, wmax);
}

// Phase A of the first round, as an ordinary launch with more warps per SM
// than the persistent kernel can hold.  When even the two heaviest vertices
// may pair and are light (2 vmax <= maxvwgt, 3 vmax < maxvwgt), every edge is
// eligible while nothing is matched, and the scans skip the neighbour state.
// Both forms are launched (the choice is made on the device, from vmax); the
// one that does not apply returns at once.  Separate kernels keep each form's
// register allocation to its own needs.
template <bool H, bool ALL>
__global__ void __launch_bounds__(kPrepThreads, kFirstMinBlocks) k_match_first(MatchArgs a) {
  const long long vmax = __ldcg(a.vmax);
  const bool all_elig = 2 * vmax <= a.maxvwgt && 3 * vmax < a.maxvwgt;
  if (all_elig != ALL) return;
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const int nchunks = (int)(__ldcg(a.big) & 0xffffffffu);
  __shared__ int2 sh_q[kPrepThreads / 32][32];
  phase_a<H>(a, a.slot[0], true, ALL, a.n, nchunks, gwarp, nwarps, lane, sh_q[threadIdx.x >> 5], nullptr);
}

template <bool H>
__global__ void __launch_bounds__(kMatchThreads, kMatchMinBlocks) k_match(MatchArgs a) {
  __shared__ int2 sh_q[kMatchThreads / 32][32];  // per warp: packed candidates of a chunk scan
  __shared__ unsigned long long sh_cw[kMatchThreads / 32];  // phase C appends: per-warp packed counts
  __shared__ int sh_cc[kMatchThreads / 32];                 // ... and chunk counts
  __shared__ unsigned long long sh_cb[4];                   // ... and the lists' bases
  __shared__ int sh_tk;                                     // phase C: the block's ticket
  const int lane = threadIdx.x & 31;
  const long long gthread = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const int gwarp = (int)(gthread >> 5);
  const int nwarps = (int)(nthreads >> 5);
  const int n = a.n;
  DevStatus *st = a.st;
  const bool tracer = a.trace != nullptr && gthread == 0;
  auto trace = [&](int row, int col, unsigned long long v) {
    if (tracer && row < a.trace_rows) a.trace[row * 8 + col] = v;
  };
  trace(0, 0, global_timer_ns());

  // Tail mode: once a round's lists are small enough for one block, the
  // other blocks return and block 0 runs the remaining rounds alone with
  // block barriers instead of grid barriers (the rounds converge to the same
  // matching whatever the schedule).  All blocks decide it alike: from the
  // counters, read after a grid barrier.
  bool tail = false;
  int round = 0;
  for (;; ++round) {
    const int par = round & 1;
    const Slot &S = a.slot[par];
    // round 0: the short-row scan list and the active list are the vertex range
    const long long nsmall = round == 0 ? n : __ldcg(a.nsmall + par);
    const int nupd = __ldcg(a.nupd + par);
    const long long nact = round == 0 ? n : __ldcg(a.nact + par);
    const unsigned long long bc = __ldcg(a.big + par);
    const int nbig = (int)(bc >> 32), nchunks = (int)(bc & 0xffffffffu);
    if (!tail && round > 0 && nsmall + nbig + nupd <= kTailItems && nchunks <= kTailChunks && nact <= kTailItems) {
      tail = true;
      if (blockIdx.x != 0) return;
    }
    // this round's thread, warp and block indices (block 0 alone in tail mode)
    const long long gth = tail ? (long long)threadIdx.x : gthread;
    const long long nth = tail ? (long long)blockDim.x : nthreads;
    const int gw = tail ? (int)(threadIdx.x >> 5) : gwarp;
    const int nw = tail ? (int)(blockDim.x >> 5) : nwarps;
    auto barrier = [&]() -> bool {
      if (!tail) return grid_barrier(st, gridDim.x);
      __syncthreads();
      return ld_relaxed(&st->error) == 0;
    };
    if (round == 0) trace(0, 1, global_timer_ns());
    trace(round + 1, 0, global_timer_ns());
    trace(round + 1, 4, (unsigned long long)nsmall);
    trace(round + 1, 5, (unsigned long long)nbig);
    trace(round + 1, 6, (unsigned long long)nchunks);
    trace(round + 1, 7, (unsigned long long)nupd);
    if (nsmall == 0 && nbig == 0 && nupd == 0) break;
    if (round >= a.max_rounds) {
      if (gth == 0) record_error(st, CM_ERR_LIMIT, ERR_SITE_ROUNDS);
      break;
    }
    if (gth == 0) {  // the next round's lists and tickets start empty
      a.nsmall[par ^ 1] = 0;
      a.nupd[par ^ 1] = 0;
      a.nact[par ^ 1] = 0;
      a.big[par ^ 1] = 0;
      a.tick[2 * (par ^ 1)] = 0;
      a.tick[2 * (par ^ 1) + 1] = 0;
    }
    // A vertex's first scan keeps only its best candidate (most vertices never
    // need more); a rescan fills the whole cache.
    const bool first = round == 0;

    // ---- phase A: full scans (the first round's ran in k_match_first) ---------
    if (!first) phase_a<H>(a, S, false, false, nsmall, nchunks, gw, nw, lane, sh_q[threadIdx.x >> 5], a.tick + 2 * par);
    if (!barrier()) return;
    trace(round + 1, 1, global_timer_ns());

    // ---- phase B: commit mutual pairs ----------------------------------------
    // Candidates that changed this round: short scans, chunked scans, cache
    // updates (in the first round every vertex, once).
    const long long tot_b = first ? n : nsmall + nbig + nupd;
    for (long long i = gth; i < tot_b; i += nth) {
      int v;
      if (i < nsmall) {
        v = first ? (int)i : __ldcg(S.small + i);
      } else if (i < nsmall + nbig) {
        v = __ldcg(S.big_v + (i - nsmall));
      } else {
        v = __ldcg(S.upd + (i - nsmall - nbig));
      }
      const int p = __ldcg(a.ptr + v);
      if (p < 0 || __ldcg(a.m2 + v) >= 0 || __ldcg(a.ptr + p) != v) continue;
      // Both ends changed this round: the lower id commits.
      if (p < v && __ldcg(a.stamp + p) == round) continue;
      a.m2[v] = p;
      a.m2[p] = v;
    }
    if (!barrier()) return;
    trace(round + 1, 2, global_timer_ns());

    // ---- phase C: filter the active list, refresh stale pointers -------------
    // Blocks take kMatchThreads * kCU consecutive entries (block-wide appends).
    // Blocks take kMatchThreads * kCU consecutive entries at a time from a
    // ticket (a fixed assignment leaves most blocks idle once the list spans
    // only one or two spans per block).
    const long long span = (long long)kMatchThreads * kCU;
    for (;;) {
      if (threadIdx.x == 0) sh_tk = atomicAdd(a.tick + 2 * par + 1, 1);
      __syncthreads();
      const long long b0 = (long long)sh_tk * span;
      __syncthreads();
      if (b0 >= nact) break;
      int x[kCU], p[kCU], sx[kCU], sp[kCU];
#pragma unroll
      for (int u = 0; u < kCU; ++u) {
        const long long i = b0 + threadIdx.x + (long long)kMatchThreads * u;
        x[u] = i < nact ? (first ? (int)i : __ldcg(S.act + i)) : -1;
      }
#pragma unroll
      for (int u = 0; u < kCU; ++u) {
        sx[u] = x[u] >= 0 ? __ldcg(a.m2 + x[u]) : 0;
        p[u] = x[u] >= 0 ? __ldcg(a.ptr + x[u]) : -1;
      }
#pragma unroll
      for (int u = 0; u < kCU; ++u)
        if (sx[u] >= 0 || p[u] < 0) x[u] = -1;  // matched, or no candidate: out for good
#pragma unroll
      for (int u = 0; u < kCU; ++u) sp[u] = x[u] >= 0 ? __ldcg(a.m2 + p[u]) : -1;
      bool keep[kCU], upd[kCU], scan[kCU];
      int xs[kCU], deg[kCU];
#pragma unroll
      for (int u = 0; u < kCU; ++u) {
        keep[u] = upd[u] = scan[u] = false;
        xs[u] = deg[u] = 0;
        const int xv = x[u];
        if (xv < 0) continue;
        if (sp[u] < 0) {
          keep[u] = true;                    // waiting on an unmatched candidate
          continue;
        }
        // from L2: phase A of this kernel rewrites the caches on other SMs
        const int4 c = __ldcg(reinterpret_cast<const int4 *>(a.top) + xv);
        const int cs[kTop] = {c.x, c.y, c.z, c.w};
        int sm[kTop];
#pragma unroll
        for (int t = 0; t < kTop; ++t) sm[t] = cs[t] >= 0 ? __ldcg(a.m2 + cs[t]) : 0;
        // first unmatched cached candidate; -1 = no candidate left, kUnknown or
        // a full cache exhausted = rescan
        int np = -2;
#pragma unroll
        for (int t = kTop - 1; t >= 0; --t) {
          if (cs[t] >= 0 && sm[t] < 0) np = cs[t];
          else if (cs[t] == -1) np = -1;
          else if (cs[t] == kUnknown) np = -2;
        }
        if (np >= 0) {
          a.ptr[xv] = np;
          keep[u] = upd[u] = true;
        } else if (np == -1) {
          a.ptr[xv] = -1;                    // the cache held every candidate: none left
        } else {
          keep[u] = scan[u] = true;
          xs[u] = a.xadj[xv];
          deg[u] = a.xadj[xv + 1] - xs[u];
        }
        if (upd[u] || scan[u]) atomicMax(a.stamp + xv, round + 1);
      }
      phase_c_append(a, par ^ 1, keep, upd, scan, x, xs, deg, sh_cw, sh_cc, sh_cb);
    }
    if (!barrier()) return;
    trace(round + 1, 3, global_timer_ns());
  }
  // (unmatched vertices become singletons in k_match_finish)
  if (gthread == 0) st->rounds = round;
  trace(0, 3, global_timer_ns());
  trace(0, 4, (unsigned long long)round);
}

// After the rounds: every vertex still unmatched is a singleton.
__global__ void k_match_finish(int n, int *__restrict__ m2) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
    if (m2[v] < 0) m2[v] = (int)v;
}

// ---------------------------------------------------------------------------
// CM_MATCH_RACY: one unsynchronised proposal pass and its cleanup, as the
// reference's cuda_shem2 (cu:1563-1595) + cuda_cleanv (cu:1600) + findc1
// (cu:1621).  A light vertex (3 vwgt < cap) that nobody has claimed takes,
// among its neighbours that already point at it or are unmatched within the
// weight cap, the heaviest one (the reference walks its row sorted by weight,
// heaviest first, and stops at the first such neighbour), and writes both
// ends with plain stores; concurrent writers race.  The cleanup then turns
// every vertex whose partner does not point back into a singleton.  The
// result is a legal matching, not a maximal one, and depends on the schedule.
// One warp per vertex (the reference uses one thread per vertex).
// ---------------------------------------------------------------------------
constexpr int kRacyThreads = 256;

__global__ void k_racy_init(int n, int *__restrict__ m) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
    m[v] = -1;
}

__global__ void __launch_bounds__(kRacyThreads) k_racy_propose(MatchArgs a) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (kRacyThreads / 32);
  volatile int *m = a.m2;
  for (long long v = (long long)blockIdx.x * (kRacyThreads / 32) + (threadIdx.x >> 5); v < a.n; v += warps) {
    const long long cap = weight_cap(a, (int)v);
    const long long vw = a.vwgt[v];
    if (!(3 * vw < cap)) continue;
    if (m[v] != -1) continue;  // already claimed
    // heaviest candidate; equal weights by the edge hash (both ends of an
    // edge rank it alike, which the reference's unstable weight sort leaves
    // to chance)
    const int hb = hash_base(a, (int)v);
    int bw = INT_MIN, bk = -1;
    unsigned bh = 0xffffffffu;
    for (int j = a.xadj[v] + lane; j < a.xadj[v + 1]; j += 32) {
      const int k = a.adjncy[j];
      if (k == v) continue;
      const int mk = m[k];
      const bool ok = mk == (int)v || (mk == -1 && vw + a.vwgt[k] <= cap);
      if (!ok) continue;
      const int w = a.adjwgt[j];
      const unsigned h = edge_hash((unsigned)(min((int)v, k) - hb), (unsigned)(max((int)v, k) - hb));
      if (w > bw || (w == bw && h < bh)) {
        bw = w;
        bh = h;
        bk = k;
      }
    }
    const int top = __reduce_max_sync(0xffffffffu, bk >= 0 ? bw : INT_MIN);
    const unsigned hmin = __reduce_min_sync(0xffffffffu, (bk >= 0 && bw == top) ? bh : 0xffffffffu);
    const unsigned holders = __ballot_sync(0xffffffffu, bk >= 0 && bw == top && bh == hmin);
    if (holders == 0) continue;
    const int k = __shfl_sync(0xffffffffu, bk, __ffs(holders) - 1);
    if (lane == 0 && m[v] == -1) {
      m[v] = k;
      if (m[k] != (int)v) m[k] = (int)v;
    }
  }
}

// s[v] = 1 if v keeps its partner (unmatched, or the partner points back).
__global__ void k_racy_clean(int n, const int *__restrict__ m, int *__restrict__ s) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int u = m[v];
    s[v] = (u == -1 || m[u] == (int)v) ? 1 : 0;
  }
}

__global__ void k_racy_apply(int n, int *__restrict__ m, const int *__restrict__ s) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
    if (s[v] == 0 || m[v] == -1) m[v] = (int)v;
}

int64_t max_chunks(int64_t n, int64_t m) { return m / kChunk + n + 64; }

}  // namespace

size_t match_ws_bytes(int64_t n, int64_t m) {
  const int64_t ch = max_chunks(n, m);
  size_t b = (size_t)n * 4 * (3 + kTop);                      // ptr, stamp, top (+slack)
  b += 2 * ((size_t)n * 4 * 6 + (size_t)ch * 16);             // two slots
  b += (size_t)ch * 4 * kPartInts * kTop;                     // chunk partial lists
  return b + 64 * 256;
}

int launch_match(cm_ctx *ctx, const cm_graph *g, int32_t maxvwgt, int32_t mode, int32_t *d_match, cudaStream_t s,
                 const int32_t *vgid, const int32_t *gbase, const int32_t *gcap) {
  const int n = g->nvtxs;
  if (n == 0) return CM_OK;
  if (mode != CM_MATCH_HEM && mode != CM_MATCH_HEM_HASH && mode != CM_MATCH_RACY)
    return cm_fail(CM_ERR_INVALID, "cm_match: unknown mode %d", mode);
  if (mode == CM_MATCH_RACY) {
    MatchArgs a{};
    a.n = n;
    a.xadj = g->xadj; a.adjncy = g->adjncy; a.adjwgt = g->adjwgt; a.vwgt = g->vwgt;
    a.maxvwgt = maxvwgt;
    a.m2 = d_match;
    a.vgid = vgid;
    a.gbase = gbase;
    a.gcap = gcap;
    int *flags = (int *)ws_take(ctx, (size_t)n * 4);
    if (!flags) return cm_fail(CM_ERR_NOMEM, "cm_match: workspace too small");
    const unsigned vg = (unsigned)std::min<int64_t>((int64_t)ctx->num_sms * 8, n / 256 + 1);
    const unsigned wg = (unsigned)std::min<int64_t>((int64_t)ctx->num_sms * 16, n / (kRacyThreads / 32) + 1);
    stage_begin(ctx, s);
    k_racy_init<<<vg, 256, 0, s>>>(n, d_match);
    k_racy_propose<<<wg, kRacyThreads, 0, s>>>(a);
    k_racy_clean<<<vg, 256, 0, s>>>(n, d_match, flags);
    k_racy_apply<<<vg, 256, 0, s>>>(n, d_match, flags);
    stage_end(ctx, CM_STAGE_MATCH, s);
    ctx->launches += 4;
    cudaMemsetAsync(&ctx->d_status->rounds, 0, sizeof(int), s);
    return check_launch(ctx, "cm_match (racy)");
  }
  const int64_t ch = max_chunks(n, g->nedges);
  MatchArgs a;
  a.n = n;
  a.xadj = g->xadj; a.adjncy = g->adjncy; a.adjwgt = g->adjwgt; a.vwgt = g->vwgt;
  a.maxvwgt = maxvwgt;  // with graphs side by side: the smallest cap (it gates the all-eligible first round)
  a.mode = mode;
  a.m2 = d_match;
  a.vgid = vgid;
  a.gbase = gbase;
  a.gcap = gcap;
  bool ok = true;
  auto take = [&](size_t bytes) {
    void *p = ws_take(ctx, bytes);
    ok = ok && p != nullptr;
    return (int *)p;
  };
  a.ptr = take((size_t)n * 4);
  a.stamp = take((size_t)n * 4);
  a.top = take((size_t)n * 4 * kTop);
  for (int p = 0; p < 2; ++p) {
    Slot &S = a.slot[p];
    S.small = take((size_t)n * 4);
    S.big_v = take((size_t)n * 4);
    S.big_base = take((size_t)n * 4);
    S.big_done = take((size_t)n * 4);
    S.desc = (int4 *)take((size_t)ch * 16);
    S.upd = take((size_t)n * 4);
    S.act = take((size_t)n * 4);
  }
  a.part = take((size_t)ch * 4 * kPartInts * kTop);
  int *ctrs = take(320);  // list counters of both slots and the largest vertex weight
  if (!ok) return cm_fail(CM_ERR_NOMEM, "cm_match: workspace too small");
  a.nsmall = ctrs;
  a.nupd = ctrs + 16;
  a.nact = ctrs + 32;
  a.big = (unsigned long long *)(ctrs + 48);
  a.vmax = ctrs + 64;
  a.tick = ctrs + 72;
  cudaMemsetAsync(ctrs, 0, 320, s);
  a.max_rounds = n + 8;
  a.st = ctx->d_status;
  a.trace = ctx->d_trace;
  a.trace_rows = ctx->trace_rows;
  const int hm = mode == CM_MATCH_HEM_HASH ? 1 : 0;
  const void *fn = hm ? (const void *)k_match<true> : (const void *)k_match<false>;
  int &per_sm = ctx->match_blocks_per_sm[hm];  // queried once per context and tie order
  if (per_sm == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kMatchThreads, 0);
  if (per_sm < 1) {
    per_sm = 0;
    return cm_fail(CM_ERR_CUDA, "cm_match: kernel cannot be resident");
  }
  // Small graphs take a few SMs, so that kernels of other contexts (other
  // streams) can run beside this one; the kernel is grid-size agnostic.
  const int64_t want = (n + g->nedges) / kWorkPerBlock + 1;
  const int grid = (int)std::min<int64_t>((int64_t)ctx->num_sms * per_sm, want);
  void *args[] = {(void *)&a};
  stage_begin(ctx, s);
  const unsigned pgrid = (unsigned)std::min<int64_t>((int64_t)ctx->num_sms * 8, n / kPrepThreads + 1);
  const unsigned fgrid = (unsigned)std::min<int64_t>((int64_t)ctx->num_sms * 8, want * 4);
  if (mode == CM_MATCH_HEM_HASH) {
    k_match_prep<true><<<pgrid, kPrepThreads, 0, s>>>(a);
    k_match_first<true, true><<<fgrid, kPrepThreads, 0, s>>>(a);
    k_match_first<true, false><<<fgrid, kPrepThreads, 0, s>>>(a);
  } else {
    k_match_prep<false><<<pgrid, kPrepThreads, 0, s>>>(a);
    k_match_first<false, true><<<fgrid, kPrepThreads, 0, s>>>(a);
    k_match_first<false, false><<<fgrid, kPrepThreads, 0, s>>>(a);
  }
  ctx->launches += 3;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kMatchThreads), args, 0, s);
  if (e != cudaSuccess) {
    stage_end(ctx, CM_STAGE_MATCH, s);
    return cuda_status(e, "cm_match launch");
  }
  k_match_finish<<<(unsigned)std::min<int64_t>((int64_t)ctx->num_sms * 4, n / 256 + 1), 256, 0, s>>>(n, d_match);
  stage_end(ctx, CM_STAGE_MATCH, s);
  ctx->launches += 2;
  return CM_OK;
}

}  // namespace cm
