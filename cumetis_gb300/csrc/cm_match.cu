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
// that order, independent of scheduling.
//
// One persistent cooperative kernel runs all rounds.  A round is two phases
// separated by grid barriers:
//   A  every frontier vertex recomputes ptr[v] = its best candidate
//      (m2[] frozen);
//   B  mutual pointers commit (m2[v]=p, m2[p]=v); the neighbours x of each
//      newly matched pair with ptr[x] in the pair join the next frontier
//      (ptr[] frozen).
// Vertices whose candidate is still unmatched keep their pointer and wait.
// m2[v] < 0 encodes "unmatched, vwgt = -1 - m2[v]", so one 4-byte gather per
// neighbour answers both "matched?" and the weight cap.
// Lanes handle one frontier vertex each when its row has <= kSerialDeg
// entries; longer rows are scanned by the whole warp (coalesced loads).
#include <climits>

#include "cm_ctx.h"

namespace cm {
namespace {

constexpr int kMatchThreads = 256;
constexpr int kSerialDeg = 16;

struct MatchArgs {
  int n;
  const int *xadj, *adjncy, *adjwgt, *vwgt;
  long long maxvwgt;
  int mode;
  int *m2;      // result (the caller's match array, used as working state)
  int *ptr;     // current candidate of every vertex
  int *stamp;   // last round whose frontier holds the vertex
  int *fr[2];   // frontiers of odd/even rounds (round 0 is all vertices)
  int *ctr;     // ctr[0], ctr[1]: frontier sizes
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

__device__ __forceinline__ void consider(const MatchArgs &a, int v, long long vw, int j, Cand &best) {
  const int k = a.adjncy[j];
  if (k == v) return;
  const int s = __ldcg(a.m2 + k);
  if (s >= 0) return;  // matched
  const long long vk = -1ll - s;
  if (vw + vk > a.maxvwgt) return;
  if (!(3 * vw < a.maxvwgt || 3 * vk < a.maxvwgt)) return;
  Cand c;
  c.w = a.adjwgt[j];
  c.k = k;
  c.h = a.mode == CM_MATCH_HEM_HASH ? edge_hash((unsigned)min(v, k), (unsigned)max(v, k)) : 0u;
  if (better(c, best)) best = c;
}

// Warp-wide best of per-lane candidates (all lanes participate).
__device__ __forceinline__ int warp_best(const Cand &c) {
  const unsigned full = 0xffffffffu;
  const bool valid = c.k != INT_MAX;
  const int wmax = __reduce_max_sync(full, valid ? c.w : INT_MIN);
  const bool atw = valid && c.w == wmax;
  const unsigned hmin = __reduce_min_sync(full, atw ? c.h : 0xffffffffu);
  const bool ath = atw && c.h == hmin;
  const unsigned kmin = __reduce_min_sync(full, ath ? (unsigned)c.k : 0xffffffffu);
  return kmin == 0xffffffffu ? -1 : (int)kmin;
}

__device__ __forceinline__ void push_next(const MatchArgs &a, int round, bool want, int x) {
  // Warp-aggregated, deduplicated by stamp; called convergently by all lanes.
  bool push = false;
  if (want) push = atomicMax(a.stamp + x, round + 1) < round + 1;
  const unsigned mask = __ballot_sync(0xffffffffu, push);
  if (!mask) return;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == __ffs(mask) - 1) base = atomicAdd(a.ctr + ((round + 1) & 1), __popc(mask));
  base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
  if (push) a.fr[(round + 1) & 1][base + __popc(mask & ((1u << lane) - 1))] = x;
}

__global__ void __launch_bounds__(kMatchThreads) k_match(MatchArgs a) {
  const int lane = threadIdx.x & 31;
  const long long gthread = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const int gwarp = (int)(gthread >> 5);
  const int nwarps = (int)(nthreads >> 5);
  const int n = a.n;
  DevStatus *st = a.st;

  for (long long v = gthread; v < n; v += nthreads) {
    a.m2[v] = -1 - a.vwgt[v];
    a.ptr[v] = -1;
    a.stamp[v] = 0;
  }
  if (gthread == 0) { a.ctr[0] = 0; a.ctr[1] = 0; }
  if (!grid_barrier(st, gridDim.x)) return;

  int round = 0;
  for (;; ++round) {
    const int count = round == 0 ? n : __ldcg(a.ctr + (round & 1));
    if (count == 0) break;
    if (round >= a.max_rounds) {
      if (gthread == 0) record_error(st, CM_ERR_LIMIT, ERR_SITE_ROUNDS);
      break;
    }
    const int *front = a.fr[round & 1];
    if (gthread == 0) a.ctr[(round + 1) & 1] = 0;

    // ---- phase A: recompute candidates --------------------------------
    for (long long base = (long long)gwarp * 32; base < count; base += (long long)nwarps * 32) {
      const long long i = base + lane;
      int v = -1, xs = 0, deg = 0;
      if (i < count) {
        v = round == 0 ? (int)i : __ldcg(front + i);
        if (__ldcg(a.m2 + v) < 0) {
          xs = a.xadj[v];
          deg = a.xadj[v + 1] - xs;
        } else {
          v = -1;
        }
      }
      const long long vw = v >= 0 ? -1ll - __ldcg(a.m2 + v) : 0;
      Cand best{0, 0u, INT_MAX};
      const bool serial = v >= 0 && deg <= kSerialDeg;
      if (serial) {
        for (int j = xs; j < xs + deg; ++j) consider(a, v, vw, j, best);
        a.ptr[v] = best.k == INT_MAX ? -1 : best.k;
      }
      unsigned longs = __ballot_sync(0xffffffffu, v >= 0 && !serial);
      while (longs) {
        const int src = __ffs(longs) - 1;
        longs &= longs - 1;
        const int vv = __shfl_sync(0xffffffffu, v, src);
        const int xx = __shfl_sync(0xffffffffu, xs, src);
        const int dd = __shfl_sync(0xffffffffu, deg, src);
        const long long ww = __shfl_sync(0xffffffffu, vw, src);
        Cand c{0, 0u, INT_MAX};
        for (int j = xx + lane; j < xx + dd; j += 32) consider(a, vv, ww, j, c);
        const int b = warp_best(c);
        if (lane == 0) a.ptr[vv] = b;
      }
    }
    if (!grid_barrier(st, gridDim.x)) return;

    // ---- phase B: commit mutual pairs, wake waiting neighbours ---------
    for (long long base = (long long)gwarp * 32; base < count; base += (long long)nwarps * 32) {
      const long long i = base + lane;
      int v = -1, p = -1;
      if (i < count) {
        v = round == 0 ? (int)i : __ldcg(front + i);
        p = __ldcg(a.ptr + v);
        bool commit = p >= 0 && __ldcg(a.m2 + v) < 0 && __ldcg(a.ptr + p) == v;
        // Both ends in this frontier: the lower id commits.
        if (commit && p < v && __ldcg(a.stamp + p) == round) commit = false;
        if (commit) {
          a.m2[v] = p;
          a.m2[p] = v;
        } else {
          v = -1;
        }
      }
      // Wake neighbours x of v and p with ptr[x] in {v, p}.
      int xv = 0, dv = 0, xp = 0, dp = 0;
      if (v >= 0) {
        xv = a.xadj[v]; dv = a.xadj[v + 1] - xv;
        xp = a.xadj[p]; dp = a.xadj[p + 1] - xp;
      }
      const bool serial = v >= 0 && dv + dp <= kSerialDeg;
      const int smax = __reduce_max_sync(0xffffffffu, serial ? dv + dp : 0);
      for (int t = 0; t < smax; ++t) {
        bool want = false;
        int x = 0;
        if (serial && t < dv + dp) {
          x = t < dv ? a.adjncy[xv + t] : a.adjncy[xp + t - dv];
          if (x != v && x != p) {
            const int px = __ldcg(a.ptr + x);
            want = (px == v || px == p) && __ldcg(a.m2 + x) < 0;
          }
        }
        push_next(a, round, want, x);
      }
      unsigned longs = __ballot_sync(0xffffffffu, v >= 0 && !serial);
      while (longs) {
        const int src = __ffs(longs) - 1;
        longs &= longs - 1;
        const int vv = __shfl_sync(0xffffffffu, v, src), pp = __shfl_sync(0xffffffffu, p, src);
        const int x0 = __shfl_sync(0xffffffffu, xv, src), d0 = __shfl_sync(0xffffffffu, dv, src);
        const int x1 = __shfl_sync(0xffffffffu, xp, src), d1 = __shfl_sync(0xffffffffu, dp, src);
        for (int t0 = 0; t0 < d0 + d1; t0 += 32) {
          const int t = t0 + lane;
          bool want = false;
          int x = 0;
          if (t < d0 + d1) {
            x = t < d0 ? a.adjncy[x0 + t] : a.adjncy[x1 + t - d0];
            if (x != vv && x != pp) {
              const int px = __ldcg(a.ptr + x);
              want = (px == vv || px == pp) && __ldcg(a.m2 + x) < 0;
            }
          }
          push_next(a, round, want, x);
        }
      }
    }
    if (!grid_barrier(st, gridDim.x)) return;
  }
  for (long long v = gthread; v < n; v += nthreads)
    if (__ldcg(a.m2 + v) < 0) a.m2[v] = (int)v;
  if (gthread == 0) st->rounds = round;
}

}  // namespace

size_t match_ws_bytes(int64_t n, int64_t) { return (size_t)n * 4 * 4 + 1024; }

int launch_match(cm_ctx *ctx, const cm_graph *g, int32_t maxvwgt, int32_t mode, int32_t *d_match, cudaStream_t s) {
  const int n = g->nvtxs;
  if (n == 0) return CM_OK;
  if (mode != CM_MATCH_HEM && mode != CM_MATCH_HEM_HASH)
    return cm_fail(CM_ERR_UNSUPPORTED, "cm_match: mode %d not available", mode);
  MatchArgs a;
  a.n = n;
  a.xadj = g->xadj; a.adjncy = g->adjncy; a.adjwgt = g->adjwgt; a.vwgt = g->vwgt;
  a.maxvwgt = maxvwgt;
  a.mode = mode;
  a.m2 = d_match;
  a.ptr = (int *)ws_take(ctx, (size_t)n * 4);
  a.stamp = (int *)ws_take(ctx, (size_t)n * 4);
  a.fr[0] = (int *)ws_take(ctx, (size_t)n * 4);
  a.fr[1] = (int *)ws_take(ctx, (size_t)n * 4);
  a.ctr = (int *)ws_take(ctx, 64);
  if (!a.ptr || !a.stamp || !a.fr[0] || !a.fr[1] || !a.ctr) return cm_fail(CM_ERR_NOMEM, "cm_match: workspace too small");
  a.max_rounds = n / 2 + 4;
  a.st = ctx->d_status;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_match, kMatchThreads, 0);
  if (per_sm < 1) per_sm = 1;
  long long want = ((long long)n + kMatchThreads - 1) / kMatchThreads;
  int grid = (int)std::min<long long>((long long)ctx->num_sms * per_sm, std::max<long long>(1, want));
  void *args[] = {(void *)&a};
  stage_begin(ctx, s);
  cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_match, dim3(grid), dim3(kMatchThreads), args, 0, s);
  stage_end(ctx, CM_STAGE_MATCH, s);
  if (e != cudaSuccess) return cuda_status(e, "cm_match launch");
  ctx->launches++;
  return CM_OK;
}

}  // namespace cm
