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
// One persistent cooperative kernel (one 1024-thread block per SM) runs all
// rounds; a round has three phases separated by grid barriers:
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

#include "cm_ctx.h"

namespace cm {
namespace {

constexpr int kMatchThreads = 1024;
constexpr int kSerialDeg = 16;   // rows scanned by one lane
constexpr int kChunk = 256;      // entries per warp work item
constexpr int kTop = 4;          // cached candidates per vertex
constexpr int kNotScanned = -2;  // top[v*kTop] before the first scan

struct Slot {      // lists feeding one round (double-buffered by round parity)
  int *small;      // full scans, rows <= kSerialDeg
  int *big_v, *big_base, *big_done, *big_map;   // full scans, longer rows (chunked)
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
  int *part;                     // per chunk: kTop x (w, h, k)
  int max_rounds;
  DevStatus *st;
  unsigned long long *trace;     // optional: row 0 header, row r+1 = round r
  int trace_rows;
};

struct Cand {
  int w;
  unsigned h;
  int k;  // INT_MAX = none
};

__device__ __forceinline__ bool better(const Cand &a, const Cand &b) {
  if (a.k == INT_MAX) return false;
  if (b.k == INT_MAX) return true;
  if (a.w != b.w) return a.w > b.w;
  if (a.h != b.h) return a.h < b.h;
  return a.k < b.k;
}

// Sorted (best first) list of up to kTop candidates held in registers.
struct TopK {
  Cand c[kTop];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int i = 0; i < kTop; ++i) c[i] = Cand{0, 0u, INT_MAX};
  }
  __device__ __forceinline__ void insert(const Cand &x) {
    if (!better(x, c[kTop - 1])) return;
    Cand cur = x;
#pragma unroll
    for (int i = 0; i < kTop; ++i) {
      if (better(cur, c[i])) { Cand t = c[i]; c[i] = cur; cur = t; }
    }
  }
};

__device__ __forceinline__ bool eligible_cand(const MatchArgs &a, int v, long long vw, int k, int w, int s, Cand &out) {
  if (k == v || s >= 0) return false;  // self or matched
  const long long vk = -1ll - s;
  if (vw + vk > a.maxvwgt) return false;
  if (!(3 * vw < a.maxvwgt || 3 * vk < a.maxvwgt)) return false;
  out.w = w;
  out.k = k;
  out.h = a.mode == CM_MATCH_HEM_HASH ? edge_hash((unsigned)min(v, k), (unsigned)max(v, k)) : 0u;
  return true;
}

__device__ __forceinline__ Cand warp_best(const Cand &c) {
  const unsigned full = 0xffffffffu;
  const bool valid = c.k != INT_MAX;
  const int wmax = __reduce_max_sync(full, valid ? c.w : INT_MIN);
  const bool atw = valid && c.w == wmax;
  const unsigned hmin = __reduce_min_sync(full, atw ? c.h : 0xffffffffu);
  const bool ath = atw && c.h == hmin;
  const unsigned kmin = __reduce_min_sync(full, ath ? (unsigned)c.k : 0xffffffffu);
  Cand r;
  r.w = wmax;
  r.h = hmin;
  r.k = kmin == 0xffffffffu ? INT_MAX : (int)kmin;
  return r;
}

// Merges the lanes' sorted lists into the warp's best kTop (all lanes get it).
__device__ __forceinline__ TopK warp_topk(TopK t) {
  TopK out;
  int head = 0;
#pragma unroll
  for (int i = 0; i < kTop; ++i) {
    Cand mine = Cand{0, 0u, INT_MAX};
#pragma unroll
    for (int j = 0; j < kTop; ++j)
      if (j == head) mine = t.c[j];
    const Cand win = warp_best(mine);
    out.c[i] = win;
    if (win.k != INT_MAX && mine.k == win.k && mine.w == win.w && mine.h == win.h) ++head;
  }
  return out;
}

// Per-lane kTop over entries [b, e) (e - b <= kChunk) of v's row; all loads of
// the chunk are issued before any is used.
__device__ __forceinline__ TopK lane_scan(const MatchArgs &a, int v, long long vw, int b, int e) {
  const int lane = threadIdx.x & 31;
  constexpr int U = kChunk / 32;
  int k[U], w[U], s[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int j = b + lane + 32 * u;
    k[u] = j < e ? a.adjncy[j] : -1;
    w[u] = j < e ? a.adjwgt[j] : 0;
  }
#pragma unroll
  for (int u = 0; u < U; ++u) s[u] = k[u] >= 0 ? __ldcg(a.m2 + k[u]) : 0;
  TopK t;
  t.clear();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    Cand c;
    if (k[u] >= 0 && eligible_cand(a, v, vw, k[u], w[u], s[u], c)) t.insert(c);
  }
  return t;
}

__device__ __forceinline__ void store_top(const MatchArgs &a, int v, const TopK &t) {
  int4 q;
  q.x = t.c[0].k == INT_MAX ? -1 : t.c[0].k;
  q.y = t.c[1].k == INT_MAX ? -1 : t.c[1].k;
  q.z = t.c[2].k == INT_MAX ? -1 : t.c[2].k;
  q.w = t.c[3].k == INT_MAX ? -1 : t.c[3].k;
  reinterpret_cast<int4 *>(a.top)[v] = q;
  a.ptr[v] = q.x;
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

// Queues x (row of `deg` entries) for a full scan in slot `par`; convergent.
__device__ __forceinline__ void append_scan(const MatchArgs &a, int par, bool take, int x, int deg) {
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
  if (bg) {
    const int idx = (int)(base >> 32), cb = (int)(base & 0xffffffffu);
    S.big_v[idx] = x;
    S.big_base[idx] = cb;
    S.big_done[idx] = 0;
    for (int j = 0; j < nch; ++j) S.big_map[cb + j] = idx;
  }
}

__global__ void __launch_bounds__(kMatchThreads, 1) k_match(MatchArgs a) {
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

  if (gthread == 0) {
    a.nsmall[0] = a.nsmall[1] = a.nupd[0] = a.nupd[1] = a.nact[0] = a.nact[1] = 0;
    a.big[0] = a.big[1] = 0;
  }
  for (long long v = gthread; v < n; v += nthreads) {
    a.m2[v] = -1 - a.vwgt[v];
    a.ptr[v] = -1;
    a.stamp[v] = 0;
    a.top[v * kTop] = kNotScanned;
  }
  if (!grid_barrier(st, gridDim.x)) return;
  // Round 0 scans every vertex that has a neighbour: short rows straight from
  // the vertex range, longer rows through the chunk list built here.
  for (long long b0 = (long long)gwarp * 32; b0 < n; b0 += (long long)nwarps * 32) {
    const long long v = b0 + lane;
    const int deg = v < n ? a.xadj[v + 1] - a.xadj[v] : 0;
    append_scan(a, 0, deg > kSerialDeg, (int)v, deg);
  }
  if (!grid_barrier(st, gridDim.x)) return;

  int round = 0;
  for (;; ++round) {
    const int par = round & 1;
    const Slot &S = a.slot[par];
    const Slot &N = a.slot[par ^ 1];
    // round 0: the short-row scan list and the active list are the vertex range
    const long long nsmall = round == 0 ? n : __ldcg(a.nsmall + par);
    const int nupd = __ldcg(a.nupd + par);
    const long long nact = round == 0 ? n : __ldcg(a.nact + par);
    const unsigned long long bc = __ldcg(a.big + par);
    const int nbig = (int)(bc >> 32), nchunks = (int)(bc & 0xffffffffu);
    if (round == 0) trace(0, 1, global_timer_ns());
    trace(round + 1, 0, global_timer_ns());
    trace(round + 1, 4, (unsigned long long)nsmall);
    trace(round + 1, 5, (unsigned long long)nbig);
    trace(round + 1, 6, (unsigned long long)nchunks);
    trace(round + 1, 7, (unsigned long long)nupd);
    if (nsmall == 0 && nbig == 0 && nupd == 0) break;
    if (round >= a.max_rounds) {
      if (gthread == 0) record_error(st, CM_ERR_LIMIT, ERR_SITE_ROUNDS);
      break;
    }
    if (gthread == 0) {  // the next round's lists start empty
      a.nsmall[par ^ 1] = 0;
      a.nupd[par ^ 1] = 0;
      a.nact[par ^ 1] = 0;
      a.big[par ^ 1] = 0;
    }

    // ---- phase A: full scans -------------------------------------------------
    for (long long b0 = (long long)gwarp * 32; b0 < nsmall; b0 += (long long)nwarps * 32) {
      const long long i = b0 + lane;
      if (i >= nsmall) continue;
      const int v = round == 0 ? (int)i : __ldcg(S.small + i);
      const int xs = a.xadj[v], deg = a.xadj[v + 1] - xs;
      if (round == 0 && (deg == 0 || deg > kSerialDeg)) continue;
      const int sv = __ldcg(a.m2 + v);
      if (sv >= 0) continue;
      const long long vw = -1ll - sv;
      int k[kSerialDeg], s[kSerialDeg];
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t) k[t] = t < deg ? a.adjncy[xs + t] : -1;
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t) s[t] = k[t] >= 0 ? __ldcg(a.m2 + k[t]) : 0;
      TopK tk;
      tk.clear();
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t) {
        Cand c;
        if (k[t] >= 0 && eligible_cand(a, v, vw, k[t], a.adjwgt[xs + t], s[t], c)) tk.insert(c);
      }
      store_top(a, v, tk);
    }
    for (int q = gwarp; q < nchunks; q += nwarps) {
      const int i = __ldcg(S.big_map + q);
      const int v = __ldcg(S.big_v + i);
      const int sv = __ldcg(a.m2 + v);
      if (sv >= 0) continue;  // uniform per warp
      const int xs = a.xadj[v], xe = a.xadj[v + 1];
      const int nch = (xe - xs + kChunk - 1) / kChunk;
      const int j = q - __ldcg(S.big_base + i);
      const int b = xs + j * kChunk, e = min(xe, b + kChunk);
      const TopK r = warp_topk(lane_scan(a, v, -1ll - sv, b, e));
      if (nch == 1) {
        if (lane == 0) store_top(a, v, r);
        continue;
      }
      int last = 0;
      if (lane < kTop) {
        Cand mine = r.c[0];
#pragma unroll
        for (int t = 1; t < kTop; ++t)
          if (lane == t) mine = r.c[t];
        int *p = a.part + ((size_t)q * kTop + lane) * 3;
        p[0] = mine.w;
        p[1] = (int)mine.h;
        p[2] = mine.k;
      }
      if (lane == 0) {
        __threadfence();
        last = atomicAdd(S.big_done + i, 1) == nch - 1;
      }
      last = __shfl_sync(0xffffffffu, last, 0);
      if (last) {  // merge the row's chunk lists
        __threadfence();
        const int base = __ldcg(S.big_base + i);
        TopK acc;
        acc.clear();
        for (int t = lane; t < nch * kTop; t += 32) {
          const int *p = a.part + ((size_t)base * kTop + t) * 3;
          Cand o;
          o.w = __ldcg(p);
          o.h = (unsigned)__ldcg(p + 1);
          o.k = __ldcg(p + 2);
          acc.insert(o);
        }
        const TopK rr = warp_topk(acc);
        if (lane == 0) store_top(a, v, rr);
      }
    }
    if (!grid_barrier(st, gridDim.x)) return;
    trace(round + 1, 1, global_timer_ns());

    // ---- phase B: commit mutual pairs ----------------------------------------
    // Candidates that changed this round: short scans, chunked scans, cache updates.
    const long long tot_b = nsmall + nbig + nupd;
    for (long long i = gthread; i < tot_b; i += nthreads) {
      int v;
      if (i < nsmall) {
        v = round == 0 ? (int)i : __ldcg(S.small + i);
        if (round == 0) {
          const int deg = a.xadj[v + 1] - a.xadj[v];
          if (deg == 0 || deg > kSerialDeg) continue;
        }
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
    if (!grid_barrier(st, gridDim.x)) return;
    trace(round + 1, 2, global_timer_ns());

    // ---- phase C: filter the active list, refresh stale pointers -------------
    for (long long b0 = (long long)gwarp * 32; b0 < nact; b0 += (long long)nwarps * 32) {
      const long long i = b0 + lane;
      int x = -1;
      if (i < nact) {
        x = round == 0 ? (int)i : __ldcg(S.act + i);
        if (__ldcg(a.m2 + x) >= 0) x = -1;  // matched
      }
      const int p = x >= 0 ? __ldcg(a.ptr + x) : -1;
      if (p < 0) x = -1;                   // no candidate: out for good
      bool keep = false, upd = false, scan = false;
      int deg = 0;
      if (x >= 0) {
        if (__ldcg(a.m2 + p) < 0) {
          keep = true;                     // waiting on an unmatched candidate
        } else {
          const int4 c = reinterpret_cast<const int4 *>(a.top)[x];
          const int cs[kTop] = {c.x, c.y, c.z, c.w};
          int sm[kTop];
#pragma unroll
          for (int t = 0; t < kTop; ++t) sm[t] = cs[t] >= 0 ? __ldcg(a.m2 + cs[t]) : 0;
          int np = -1;
#pragma unroll
          for (int t = kTop - 1; t >= 0; --t)
            if (cs[t] >= 0 && sm[t] < 0) np = cs[t];
          if (np >= 0) {
            a.ptr[x] = np;
            keep = upd = true;
          } else if (cs[kTop - 1] < 0) {
            a.ptr[x] = -1;                 // cache held every candidate: none left
          } else {
            keep = scan = true;
            deg = a.xadj[x + 1] - a.xadj[x];
          }
        }
      }
      if (upd || scan) atomicMax(a.stamp + x, round + 1);
      warp_append(N.act, a.nact + (par ^ 1), keep, x);
      warp_append(N.upd, a.nupd + (par ^ 1), upd, x);
      append_scan(a, par ^ 1, scan, x, deg);
    }
    if (!grid_barrier(st, gridDim.x)) return;
    trace(round + 1, 3, global_timer_ns());
  }
  for (long long v = gthread; v < n; v += nthreads)
    if (__ldcg(a.m2 + v) < 0) a.m2[v] = (int)v;
  if (gthread == 0) st->rounds = round;
  trace(0, 3, global_timer_ns());
  trace(0, 4, (unsigned long long)round);
}

int64_t max_chunks(int64_t n, int64_t m) { return m / kChunk + n + 64; }

}  // namespace

size_t match_ws_bytes(int64_t n, int64_t m) {
  const int64_t ch = max_chunks(n, m);
  size_t b = (size_t)n * 4 * (3 + kTop);                      // ptr, stamp, top (+slack)
  b += 2 * ((size_t)n * 4 * 6 + (size_t)ch * 4);              // two slots
  b += (size_t)ch * 4 * 3 * kTop;                             // chunk partial lists
  return b + 64 * 256;
}

int launch_match(cm_ctx *ctx, const cm_graph *g, int32_t maxvwgt, int32_t mode, int32_t *d_match, cudaStream_t s) {
  const int n = g->nvtxs;
  if (n == 0) return CM_OK;
  if (mode != CM_MATCH_HEM && mode != CM_MATCH_HEM_HASH)
    return cm_fail(CM_ERR_UNSUPPORTED, "cm_match: mode %d not available", mode);
  const int64_t ch = max_chunks(n, g->nedges);
  MatchArgs a;
  a.n = n;
  a.xadj = g->xadj; a.adjncy = g->adjncy; a.adjwgt = g->adjwgt; a.vwgt = g->vwgt;
  a.maxvwgt = maxvwgt;
  a.mode = mode;
  a.m2 = d_match;
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
    S.big_map = take((size_t)ch * 4);
    S.upd = take((size_t)n * 4);
    S.act = take((size_t)n * 4);
  }
  a.part = take((size_t)ch * 4 * 3 * kTop);
  a.nsmall = take(64);
  a.nupd = take(64);
  a.nact = take(64);
  a.big = (unsigned long long *)take(64);
  if (!ok) return cm_fail(CM_ERR_NOMEM, "cm_match: workspace too small");
  a.max_rounds = n + 8;
  a.st = ctx->d_status;
  a.trace = ctx->d_trace;
  a.trace_rows = ctx->trace_rows;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_match, kMatchThreads, 0);
  if (per_sm < 1) return cm_fail(CM_ERR_CUDA, "cm_match: kernel cannot be resident");
  const int grid = ctx->num_sms * per_sm;
  void *args[] = {(void *)&a};
  stage_begin(ctx, s);
  cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_match, dim3(grid), dim3(kMatchThreads), args, 0, s);
  stage_end(ctx, CM_STAGE_MATCH, s);
  if (e != cudaSuccess) return cuda_status(e, "cm_match launch");
  ctx->launches++;
  return CM_OK;
}

}  // namespace cm
