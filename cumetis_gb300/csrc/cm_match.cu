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
// rounds.  A round has three phases separated by grid barriers:
//   A  (m2[] frozen)  every vertex of the round's work recomputes ptr[v], its
//      best candidate.  Rows of <= kSerialDeg entries: one lane each.  Longer
//      rows: kChunk-entry chunks, one warp each (edge-balanced across the
//      grid); the last chunk of a row to finish reduces the chunk bests.
//   B  (ptr[] frozen) mutual pointers commit (m2[v]=p, m2[p]=v).  A pair whose
//      two rows are short wakes its neighbours x with ptr[x] in the pair at
//      once; longer pairs queue their rows as wake chunks.
//   C  wake chunks: neighbours with ptr[x] in the pair join the next round.
// Vertices whose candidate is still unmatched keep their pointer and wait.
// m2[v] < 0 encodes "unmatched, vwgt = -1 - m2[v]": one 4-byte gather per
// neighbour answers both "matched?" and the weight cap.
#include <climits>

#include "cm_ctx.h"

namespace cm {
namespace {

constexpr int kMatchThreads = 1024;
constexpr int kSerialDeg = 16;   // rows scanned by one lane
constexpr int kChunk = 256;      // entries per warp work item

struct Slot {      // work of one round (double-buffered by round parity)
  int *small;      // vertices with rows <= kSerialDeg
  int *big_v, *big_base, *big_done;  // longer rows, first chunk index, chunks done
  int *big_map;    // chunk -> index into big_v
};

struct MatchArgs {
  int n;
  const int *xadj, *adjncy, *adjwgt, *vwgt;
  long long maxvwgt;
  int mode;
  int *m2, *ptr, *stamp;
  Slot slot[2];
  int *wk_x, *wk_v, *wk_p, *wk_base, *wk_map;   // wake items of the current round
  int *nsmall;                   // nsmall[0..1]
  unsigned long long *big;       // big[0..1] = (rows << 32 | chunks)
  unsigned long long *wk;        // (items << 32 | chunks)
  int *part_w, *part_k;          // per chunk partial best
  unsigned *part_h;
  int max_rounds;
  DevStatus *st;
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

__device__ __forceinline__ void eval(const MatchArgs &a, int v, long long vw, int k, int w, int s, Cand &best) {
  if (k == v || s >= 0) return;  // self or matched
  const long long vk = -1ll - s;
  if (vw + vk > a.maxvwgt) return;
  if (!(3 * vw < a.maxvwgt || 3 * vk < a.maxvwgt)) return;
  Cand c;
  c.w = w;
  c.k = k;
  c.h = a.mode == CM_MATCH_HEM_HASH ? edge_hash((unsigned)min(v, k), (unsigned)max(v, k)) : 0u;
  if (better(c, best)) best = c;
}

// Per-lane best over entries [b, e) (e - b <= kChunk) of v's row; all loads
// of the chunk are issued before any is used.
__device__ __forceinline__ Cand lane_scan(const MatchArgs &a, int v, long long vw, int b, int e) {
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
  Cand c{0, 0u, INT_MAX};
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (k[u] >= 0) eval(a, v, vw, k[u], w[u], s[u], c);
  return c;
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

__device__ __forceinline__ unsigned long long warp_excl_scan_u64(unsigned long long v, unsigned long long *total) {
  const unsigned long long inc = warp_inclusive_scan_u64(v);
  *total = __shfl_sync(0xffffffffu, inc, 31);
  return inc - v;
}

// Adds vertex x (row of `deg` entries) to slot S's work; all lanes call it
// convergently (warp-aggregated counters).
__device__ __forceinline__ void append_work(const MatchArgs &a, int par, bool take, int x, int deg) {
  const Slot &S = a.slot[par];
  const int lane = threadIdx.x & 31;
  const bool sm = take && deg <= kSerialDeg;
  const unsigned mask = __ballot_sync(0xffffffffu, sm);
  if (mask) {
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(a.nsmall + par, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (sm) S.small[base + __popc(mask & ((1u << lane) - 1))] = x;
  }
  const bool bg = take && deg > kSerialDeg;
  if (__any_sync(0xffffffffu, bg)) {
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
}

// Queues x's row as wake chunks for the pair (v, p); convergent call.
__device__ __forceinline__ void append_wake(const MatchArgs &a, bool take, int x, int deg, int v, int p) {
  const int lane = threadIdx.x & 31;
  const bool t = take && deg > 0;
  if (!__any_sync(0xffffffffu, t)) return;
  const int nch = t ? (deg + kChunk - 1) / kChunk : 0;
  const unsigned long long mine = t ? ((1ull << 32) | (unsigned long long)nch) : 0ull;
  unsigned long long tot;
  const unsigned long long ex = warp_excl_scan_u64(mine, &tot);
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(a.wk, tot);
  base = __shfl_sync(0xffffffffu, base, 0) + ex;
  if (t) {
    const int idx = (int)(base >> 32), cb = (int)(base & 0xffffffffu);
    a.wk_x[idx] = x;
    a.wk_v[idx] = v;
    a.wk_p[idx] = p;
    a.wk_base[idx] = cb;
    for (int j = 0; j < nch; ++j) a.wk_map[cb + j] = idx;
  }
}

__device__ __forceinline__ bool wakes(const MatchArgs &a, int x, int v, int p) {
  if (x == v || x == p) return false;
  const int px = __ldcg(a.ptr + x);
  return (px == v || px == p) && __ldcg(a.m2 + x) < 0;
}

// Puts x into round nr's work unless already there (stamp); convergent.
__device__ __forceinline__ void push_next(const MatchArgs &a, int nr, bool want, int x) {
  bool push = false;
  if (want) push = atomicMax(a.stamp + x, nr) < nr;
  int deg = 0;
  if (push) deg = a.xadj[x + 1] - a.xadj[x];
  append_work(a, nr & 1, push, x, deg);
}

__global__ void __launch_bounds__(kMatchThreads, 1) k_match(MatchArgs a) {
  const int lane = threadIdx.x & 31;
  const long long gthread = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const int gwarp = (int)(gthread >> 5);
  const int nwarps = (int)(nthreads >> 5);
  const int n = a.n;
  DevStatus *st = a.st;

  if (gthread == 0) {
    a.nsmall[0] = a.nsmall[1] = 0;
    a.big[0] = a.big[1] = 0;
    a.wk[0] = 0;
  }
  for (long long v = gthread; v < n; v += nthreads) {
    a.m2[v] = -1 - a.vwgt[v];
    a.ptr[v] = -1;
    a.stamp[v] = 0;
  }
  if (!grid_barrier(st, gridDim.x)) return;
  // round 0 works on every vertex that has a neighbour
  for (long long b0 = (long long)gwarp * 32; b0 < n; b0 += (long long)nwarps * 32) {
    const long long v = b0 + lane;
    const int deg = v < n ? a.xadj[v + 1] - a.xadj[v] : 0;
    append_work(a, 0, deg > 0, (int)v, deg);
  }
  if (!grid_barrier(st, gridDim.x)) return;

  int round = 0;
  for (;; ++round) {
    const int par = round & 1;
    const Slot &S = a.slot[par];
    const int nsmall = __ldcg(a.nsmall + par);
    const unsigned long long bc = __ldcg(a.big + par);
    const int nbig = (int)(bc >> 32), nchunks = (int)(bc & 0xffffffffu);
    if (nsmall == 0 && nbig == 0) break;
    if (round >= a.max_rounds) {
      if (gthread == 0) record_error(st, CM_ERR_LIMIT, ERR_SITE_ROUNDS);
      break;
    }
    if (gthread == 0) {  // next round's slot and this round's wake list start empty
      a.nsmall[par ^ 1] = 0;
      a.big[par ^ 1] = 0;
      a.wk[0] = 0;
    }

    // ---- phase A: candidates ----------------------------------------------
    for (long long b0 = (long long)gwarp * 32; b0 < nsmall; b0 += (long long)nwarps * 32) {
      const long long i = b0 + lane;
      if (i >= nsmall) continue;
      const int v = __ldcg(S.small + i);
      const int sv = __ldcg(a.m2 + v);
      if (sv >= 0) continue;
      const long long vw = -1ll - sv;
      const int xs = a.xadj[v], deg = a.xadj[v + 1] - xs;
      int k[kSerialDeg], s[kSerialDeg];
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t) k[t] = t < deg ? a.adjncy[xs + t] : -1;
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t) s[t] = k[t] >= 0 ? __ldcg(a.m2 + k[t]) : 0;
      Cand best{0, 0u, INT_MAX};
#pragma unroll
      for (int t = 0; t < kSerialDeg; ++t)
        if (k[t] >= 0 && s[t] < 0) eval(a, v, vw, k[t], a.adjwgt[xs + t], s[t], best);
      a.ptr[v] = best.k == INT_MAX ? -1 : best.k;
    }
    for (int q = gwarp; q < nchunks; q += nwarps) {
      const int i = __ldcg(S.big_map + q);
      const int v = __ldcg(S.big_v + i);
      const int sv = __ldcg(a.m2 + v);
      if (sv >= 0) continue;  // matched: nothing to recompute (uniform per warp)
      const int xs = a.xadj[v], xe = a.xadj[v + 1];
      const int nch = (xe - xs + kChunk - 1) / kChunk;
      const int j = q - __ldcg(S.big_base + i);
      const int b = xs + j * kChunk, e = min(xe, b + kChunk);
      const Cand r = warp_best(lane_scan(a, v, -1ll - sv, b, e));
      if (nch == 1) {
        if (lane == 0) a.ptr[v] = r.k == INT_MAX ? -1 : r.k;
        continue;
      }
      int last = 0;
      if (lane == 0) {
        a.part_w[q] = r.w;
        a.part_h[q] = r.h;
        a.part_k[q] = r.k;
        __threadfence();
        last = atomicAdd(S.big_done + i, 1) == nch - 1;
      }
      last = __shfl_sync(0xffffffffu, last, 0);
      if (last) {  // reduce this row's chunk bests
        __threadfence();
        const int base = __ldcg(S.big_base + i);
        Cand cc{0, 0u, INT_MAX};
        for (int t = lane; t < nch; t += 32) {
          Cand o;
          o.k = __ldcg(a.part_k + base + t);
          o.w = __ldcg(a.part_w + base + t);
          o.h = __ldcg(a.part_h + base + t);
          if (better(o, cc)) cc = o;
        }
        const Cand rr = warp_best(cc);
        if (lane == 0) a.ptr[v] = rr.k == INT_MAX ? -1 : rr.k;
      }
    }
    if (!grid_barrier(st, gridDim.x)) return;

    // ---- phase B: commit mutual pairs --------------------------------------
    const long long total = (long long)nsmall + nbig;
    for (long long b0 = (long long)gwarp * 32; b0 < total; b0 += (long long)nwarps * 32) {
      const long long i = b0 + lane;
      int v = -1, p = -1;
      if (i < total) {
        v = i < nsmall ? __ldcg(S.small + i) : __ldcg(S.big_v + (i - nsmall));
        p = __ldcg(a.ptr + v);
        bool commit = p >= 0 && __ldcg(a.m2 + v) < 0 && __ldcg(a.ptr + p) == v;
        // Both ends in this round's work: the lower id commits.
        if (commit && p < v && __ldcg(a.stamp + p) == round) commit = false;
        if (commit) {
          a.m2[v] = p;
          a.m2[p] = v;
        } else {
          v = -1;
        }
      }
      int xv = 0, dv = 0, xp = 0, dp = 0;
      if (v >= 0) {
        xv = a.xadj[v]; dv = a.xadj[v + 1] - xv;
        xp = a.xadj[p]; dp = a.xadj[p + 1] - xp;
      }
      const bool serial = v >= 0 && dv + dp <= kSerialDeg;
      // long pairs: queue both rows as wake chunks for phase C
      append_wake(a, v >= 0 && !serial, v, dv, v, p);
      append_wake(a, v >= 0 && !serial, p, dp, v, p);
      const int smax = __reduce_max_sync(0xffffffffu, serial ? dv + dp : 0);
      for (int t = 0; t < smax; ++t) {
        bool want = false;
        int x = 0;
        if (serial && t < dv + dp) {
          x = t < dv ? a.adjncy[xv + t] : a.adjncy[xp + t - dv];
          want = wakes(a, x, v, p);
        }
        push_next(a, round + 1, want, x);
      }
    }
    if (!grid_barrier(st, gridDim.x)) return;

    // ---- phase C: wake chunks ----------------------------------------------
    const unsigned long long wc = __ldcg(a.wk);
    const int wchunks = (int)(wc & 0xffffffffu);
    for (int q = gwarp; q < wchunks; q += nwarps) {
      const int i = __ldcg(a.wk_map + q);
      const int x = __ldcg(a.wk_x + i), v = __ldcg(a.wk_v + i), p = __ldcg(a.wk_p + i);
      const int j = q - __ldcg(a.wk_base + i);
      const int xs = a.xadj[x], xe = a.xadj[x + 1];
      const int b = xs + j * kChunk, e = min(xe, b + kChunk);
      constexpr int U = kChunk / 32;
      int y[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = b + lane + 32 * u;
        y[u] = t < e ? a.adjncy[t] : -1;
      }
      bool want[U];
#pragma unroll
      for (int u = 0; u < U; ++u) want[u] = y[u] >= 0 && wakes(a, y[u], v, p);
#pragma unroll
      for (int u = 0; u < U; ++u) push_next(a, round + 1, want[u], y[u] >= 0 ? y[u] : 0);
    }
    if (!grid_barrier(st, gridDim.x)) return;
  }
  for (long long v = gthread; v < n; v += nthreads)
    if (__ldcg(a.m2 + v) < 0) a.m2[v] = (int)v;
  if (gthread == 0) st->rounds = round;
}

int64_t max_chunks(int64_t n, int64_t m) { return m / kChunk + n + 64; }

}  // namespace

size_t match_ws_bytes(int64_t n, int64_t m) {
  const int64_t ch = max_chunks(n, m);
  size_t b = (size_t)n * 4 * 3;                               // ptr, stamp (+slack)
  b += 2 * ((size_t)n * 4 * 4 + (size_t)ch * 4);              // two slots
  b += (size_t)n * 4 * 4 + (size_t)ch * 4;                    // wake items + map
  b += (size_t)ch * 4 * 3;                                    // partials
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
  for (int p = 0; p < 2; ++p) {
    Slot &S = a.slot[p];
    S.small = take((size_t)n * 4);
    S.big_v = take((size_t)n * 4);
    S.big_base = take((size_t)n * 4);
    S.big_done = take((size_t)n * 4);
    S.big_map = take((size_t)ch * 4);
  }
  a.wk_x = take((size_t)n * 4);
  a.wk_v = take((size_t)n * 4);
  a.wk_p = take((size_t)n * 4);
  a.wk_base = take((size_t)n * 4);
  a.wk_map = take((size_t)ch * 4);
  a.part_w = take((size_t)ch * 4);
  a.part_k = take((size_t)ch * 4);
  a.part_h = (unsigned *)take((size_t)ch * 4);
  a.nsmall = take(64);
  a.big = (unsigned long long *)take(64);
  a.wk = (unsigned long long *)take(64);
  if (!ok) return cm_fail(CM_ERR_NOMEM, "cm_match: workspace too small");
  a.max_rounds = n + 8;
  a.st = ctx->d_status;
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
