// cm_refine.cu -- k-way refinement and projection on the device, and the
// whole partition driver (coarsen -> initial partition -> refine/project per
// level).
//
// Replaces the uncoarsening half of cuMetis_kway_partition (cuMetis.cu:
// 3544-3616): cuMetis_uncoarsen (3494-3514) with cuMetis_findgraphbndinfo
// (3389-3418), Find_real_bnd_info (3236-3262), find_kayparams (3267-3306),
// the bb_segsort of boundary vertices by target part (3406), findcsr
// (3322-3352), Exnode_part1/2 (3436-3488); cuMetis_kway_project / projectback
// (3067-3086); and cuMetis_PartGraph (3622-3664).
//
// One refinement pass, as in the reference (refine_pass = 1, cu:3319):
//   1. part weights pwgts[p] and the balance window of every part,
//      max = (int)(tpwgts * tvwgt * 1.03f), min = (int)(tpwgts * tvwgt / 1.03f)
//      with tpwgts = 1/k (Sum_maxmin_pwgts, cu:3424-3433);
//   2. a vertex is a boundary vertex when the weight of its edges to other
//      parts exceeds the weight to its own part; its target is the part with
//      the largest connection, the lowest such part id, unless no part beats
//      its own (find_kayparams' scan, cu:3290-3298);
//   3. boundary vertices grouped by target part -- here in vertex-id order
//      within a part (a stable counting sort), where the reference's
//      segmented sort leaves equal targets in an unspecified order;
//   4. per target part one thread walks its group in order and moves a vertex
//      when both parts stay inside their windows: first the moves towards a
//      higher part id, then (second launch) towards a lower one.
//      Part weights are updated with atomics while the part threads run, as
//      in the reference, so concurrent groups see each other's moves in
//      whatever order the hardware interleaves them.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <vector>

#include "cm_ctx.h"

namespace cm {
namespace {

constexpr int kRefThreads = 256;          // 8 warps; one warp per vertex
constexpr int kRefWarps = kRefThreads / 32;
constexpr int kSmemParts = 1024;          // per-warp part accumulators in shared memory up to this k
constexpr int kSortBlock = 1024;          // boundary entries per counting-sort block

// Part weights (atomics, shared-memory histogram when k is small).  With a
// coarser level given (cmap, cwhere), the kernel first projects it:
// where[v] = cwhere[cmap[v]] (cuMetis_kway_project fused into the pass).
__global__ void k_part_weights(int n, int *__restrict__ where, const int *__restrict__ vwgt, int nparts,
                               int *__restrict__ pwgts, const int *__restrict__ cmap, const int *__restrict__ cwhere) {
  extern __shared__ int h[];
  const bool sh = nparts <= 8192;
  if (sh)
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    int p;
    if (cmap) {
      p = cwhere[cmap[v]];
      where[v] = p;
    } else {
      p = where[v];
    }
    if (sh) atomicAdd(&h[p], vwgt[v]);
    else atomicAdd(&pwgts[p], vwgt[v]);
  }
  __syncthreads();
  if (sh)
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
      if (h[i]) atomicAdd(&pwgts[i], h[i]);
}

// Balance window of each part from the total vertex weight (Sum_maxmin_pwgts).
__global__ void k_part_bounds(int nparts, float tp, const int *__restrict__ pwgts, int *__restrict__ maxw,
                              int *__restrict__ minw) {
  __shared__ long long s_tot;
  if (threadIdx.x == 0) s_tot = 0;
  __syncthreads();
  long long t = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) t += pwgts[i];
  atomicAdd((unsigned long long *)&s_tot, (unsigned long long)t);
  __syncthreads();
  const int tvwgt = (int)s_tot;
  const float ub = 1.03f;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    maxw[i] = (int)(__fmul_rn(__fmul_rn(tp, (float)tvwgt), ub));
    minw[i] = (int)(__fdiv_rn(__fmul_rn(tp, (float)tvwgt), ub));
  }
}

// Boundary test and target part, one warp per vertex.  acc holds one zeroed
// int per part for this warp (shared memory when k <= kSmemParts, else a
// global slice); it is zero again when the warp moves on.
template <bool kShared>
__global__ void __launch_bounds__(kRefThreads)
k_boundary(int n, const int *__restrict__ xadj, const int *__restrict__ adjncy, const int *__restrict__ adjwgt,
           const int *__restrict__ where, int nparts, int *__restrict__ acc_global, int *__restrict__ flag,
           int *__restrict__ target) {
  extern __shared__ int acc_s[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long gw = (long long)blockIdx.x * kRefWarps + warp;
  const long long nw = (long long)gridDim.x * kRefWarps;
  int *acc = kShared ? acc_s + warp * nparts : acc_global + gw * nparts;
  if (kShared) {
    for (int i = threadIdx.x; i < kRefWarps * nparts; i += kRefThreads) acc_s[i] = 0;
    __syncthreads();
  }
  for (long long v = gw; v < n; v += nw) {
    const int xs = xadj[v], xe = xadj[v + 1], me = where[v];
    int mw = 0, ow = 0;
    for (int j = xs + lane; j < xe; j += 32) {
      const int w = adjwgt[j];
      if (where[adjncy[j]] == me) mw += w;
      else ow += w;
    }
    mw = __reduce_add_sync(0xffffffffu, mw);
    ow = __reduce_add_sync(0xffffffffu, ow);
    const bool bnd = ow > mw;
    int t = me;
    if (bnd) {
      for (int j = xs + lane; j < xe; j += 32) atomicAdd(&acc[where[adjncy[j]]], adjwgt[j]);
      __syncwarp();
      int bw = INT_MIN, bp = INT_MAX;
      for (int j = xs + lane; j < xe; j += 32) {
        const int p = where[adjncy[j]];
        const int w = acc[p];
        if (w > bw || (w == bw && p < bp)) {
          bw = w;
          bp = p;
        }
      }
      const int wmax = __reduce_max_sync(0xffffffffu, bw);
      const int pmin = __reduce_min_sync(0xffffffffu, bw == wmax ? bp : INT_MAX);
      const int mew = acc[me];
      t = wmax > mew ? pmin : me;
      __syncwarp();
      for (int j = xs + lane; j < xe; j += 32) acc[where[adjncy[j]]] = 0;
      __syncwarp();
    }
    if (lane == 0) {
      flag[v] = bnd ? 1 : 0;
      target[v] = t;
    }
  }
}

// Exclusive scan of flags[0..n) into pos[0..n] (decoupled look-back over
// 2048-entry tiles); pos[n] = total.
constexpr int kScanThreads = 256, kScanItems = 8;
__global__ void __launch_bounds__(kScanThreads)
k_scan_flags(const int *__restrict__ flags, int n, int *__restrict__ pos, unsigned long long *lb, DevStatus *st) {
  __shared__ int s_tile;
  __shared__ unsigned long long s_warp[kScanThreads / 32];
  __shared__ unsigned long long s_excl;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(lb, 1ull);
  __syncthreads();
  const int tile = s_tile;
  const long long base = (long long)tile * kScanThreads * kScanItems + (long long)threadIdx.x * kScanItems;
  int v[kScanItems];
  unsigned long long sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? flags[base + i] : 0;
    sum += (unsigned)v[i];
  }
  const unsigned long long inc = warp_inclusive_scan_u64(sum);
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const unsigned long long x = lane < kScanThreads / 32 ? s_warp[lane] : 0ull;
    const unsigned long long xi = warp_inclusive_scan_u64(x);
    const unsigned long long agg = __shfl_sync(0xffffffffu, xi, kScanThreads / 32 - 1);
    if (lane < kScanThreads / 32) s_warp[lane] = xi - x;
    const unsigned long long ex = lookback_exclusive(lb, tile, agg, st);
    if (lane == 0) s_excl = ex;
  }
  __syncthreads();
  unsigned long long run = s_excl + s_warp[wid] + inc - sum;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i >= n) break;
    pos[base + i] = (int)run;
    run += (unsigned)v[i];
    if (base + i == n - 1) pos[n] = (int)run;
  }
}

// Boundary list in vertex order: bnd_v[pos[v]] = v, bnd_t[...] = target[v].
__global__ void k_compact(int n, const int *__restrict__ flag, const int *__restrict__ pos,
                          const int *__restrict__ target, int *__restrict__ bnd_v, int *__restrict__ bnd_t) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
    if (flag[v]) {
      bnd_v[pos[v]] = (int)v;
      bnd_t[pos[v]] = target[v];
    }
}

// Stable counting sort of the boundary list by target part, three steps:
// per-block counts, per-part prefix over blocks, in-order scatter.
__global__ void k_sort_counts(const int *__restrict__ d_nb, const int *__restrict__ bnd_t, int nparts,
                              int *__restrict__ bhist) {
  const int nb = *d_nb;
  const long long b = blockIdx.x;
  for (long long i = b * kSortBlock + threadIdx.x; i < min((long long)nb, (b + 1) * kSortBlock); i += blockDim.x)
    atomicAdd(&bhist[b * nparts + bnd_t[i]], 1);
}

__global__ void k_sort_offsets(const int *__restrict__ d_nb, int nparts, int *__restrict__ bhist,
                               int *__restrict__ pcount) {
  const int nb = *d_nb;
  const int nblocks = (nb + kSortBlock - 1) / kSortBlock;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nparts; t += gridDim.x * blockDim.x) {
    int run = 0;
    for (int b = 0; b < nblocks; ++b) {
      const int c = bhist[(size_t)b * nparts + t];
      bhist[(size_t)b * nparts + t] = run;
      run += c;
    }
    pcount[t] = run;
  }
}

// pstart[t] = exclusive prefix of pcount (one block).
__global__ void k_part_starts(int nparts, const int *__restrict__ pcount, int *__restrict__ pstart) {
  __shared__ int scan[1024 / 32 + 1];
  int carry = 0;
  for (int b = 0; b < nparts; b += 1024) {
    const int t = b + threadIdx.x;
    const int c = t < nparts ? pcount[t] : 0;
    int tot;
    const int ex = block_exclusive_scan<1024>(c, scan, &tot);
    if (t < nparts) pstart[t] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) pstart[nparts] = carry;
}

// One warp per block of kSortBlock entries, in order: an entry's place is its
// part's start + the block's offset for the part + its rank among the part's
// earlier entries in the block.
__global__ void k_sort_scatter(const int *__restrict__ d_nb, const int *__restrict__ bnd_v,
                               const int *__restrict__ bnd_t, int nparts, int *__restrict__ bhist,
                               const int *__restrict__ pstart, int *__restrict__ sorted_v) {
  const int nb = *d_nb;
  const int lane = threadIdx.x & 31;
  const long long b = blockIdx.x;
  const long long lo = b * kSortBlock, hi = min((long long)nb, lo + kSortBlock);
  int *cnt = bhist + b * nparts;
  for (long long i0 = lo; i0 < hi; i0 += 32) {
    const long long i = i0 + lane;
    const bool ok = i < hi;
    const int t = ok ? bnd_t[i] : -1;
    const unsigned m = __match_any_sync(0xffffffffu, t);
    const int rank = __popc(m & ((1u << lane) - 1));
    int base = 0;
    if (ok) base = cnt[t];
    __syncwarp();
    if (ok) {
      sorted_v[pstart[t] + base + rank] = bnd_v[i];
      if (rank == 0) cnt[t] = base + __popc(m);
    }
    __syncwarp();
  }
}

// One thread per target part walks its group in order (Exnode_part1 when
// kUp, moves to a higher-or-equal part id; Exnode_part2 otherwise).
template <bool kUp>
__global__ void k_moves(int nparts, const int *__restrict__ pstart, const int *__restrict__ sorted_v,
                        const int *__restrict__ vwgt, const int *__restrict__ maxw, const int *__restrict__ minw,
                        int *pwgts, int *where, unsigned long long *moves) {
  const int to = blockIdx.x * blockDim.x + threadIdx.x;
  if (to >= nparts) return;
  unsigned long long nm = 0;
  const int tomax = maxw[to], tomin = minw[to];
  for (int i = pstart[to]; i < pstart[to + 1]; ++i) {
    const int v = sorted_v[i];
    const int vw = vwgt[v];
    const int me = where[v];
    // me == to would add and remove the same weight: a no-op move, skipped
    // (the reference applies it, leaving a transient in pwgts[me]).
    if (kUp ? (me >= to) : (me <= to)) continue;
    const int pto = *(volatile int *)&pwgts[to], pme = *(volatile int *)&pwgts[me];
    if (pto + vw >= tomin && pto + vw <= tomax && pme - vw >= minw[me] && pme - vw <= maxw[me]) {
      atomicAdd(&pwgts[to], vw);
      atomicSub(&pwgts[me], vw);
      where[v] = to;
      ++nm;
    }
  }
  if (nm) atomicAdd(moves, nm);
}

__global__ void k_project(int n, const int *__restrict__ cmap, const int *__restrict__ cwhere,
                          int *__restrict__ where) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
    where[v] = cwhere[cmap[v]];
}

// Sum of weights of cut entries (each undirected cut edge counted twice).
__global__ void k_cut(int n, const int *__restrict__ xadj, const int *__restrict__ adjncy,
                      const int *__restrict__ adjwgt, const int *__restrict__ where, unsigned long long *out) {
  const int lane = threadIdx.x & 31;
  const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  long long s = 0;
  for (long long v = gw; v < n; v += nw) {
    const int me = where[v];
    for (int j = xadj[v] + lane; j < xadj[v + 1]; j += 32)
      if (where[adjncy[j]] != me) s += adjwgt[j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0 && s) atomicAdd(out, (unsigned long long)s);
}

struct RefineWs {
  int *pwgts, *maxw, *minw, *flag, *target, *pos, *bnd_v, *bnd_t, *sorted_v, *bhist, *pcount, *pstart, *acc;
  unsigned long long *lb, *counters;  // counters[0] = moves, [1] = cut
  size_t bhist_ints, acc_ints, lb_words;
};

int grid_warps(cm_ctx *ctx) { return ctx->num_sms * 8 * kRefWarps; }

size_t refine_ws_bytes(cm_ctx *ctx, int64_t n, int nparts) {
  const int64_t nblocks = (n + kSortBlock - 1) / kSortBlock + 1;
  size_t b = 0;
  b += (size_t)(3 * nparts + 2 * (nparts + 1)) * 4 + 5 * 256;
  b += (size_t)(6 * n + 8) * 4 + 6 * 256;
  b += (size_t)nblocks * nparts * 4 + 256;
  if (nparts > kSmemParts) b += (size_t)grid_warps(ctx) * nparts * 4 + 256;
  b += (size_t)(n / (kScanThreads * kScanItems) + 4) * 8 + 256 + 64;
  return b + 4096;
}

int take_refine_ws(cm_ctx *ctx, int64_t n, int nparts, RefineWs &w) {
  const int64_t nblocks = (n + kSortBlock - 1) / kSortBlock + 1;
  w.pwgts = (int *)ws_take(ctx, (size_t)nparts * 4);
  w.maxw = (int *)ws_take(ctx, (size_t)nparts * 4);
  w.minw = (int *)ws_take(ctx, (size_t)nparts * 4);
  w.pcount = (int *)ws_take(ctx, (size_t)(nparts + 1) * 4);
  w.pstart = (int *)ws_take(ctx, (size_t)(nparts + 1) * 4);
  w.flag = (int *)ws_take(ctx, (size_t)n * 4 + 4);
  w.target = (int *)ws_take(ctx, (size_t)n * 4 + 4);
  w.pos = (int *)ws_take(ctx, (size_t)(n + 1) * 4);
  w.bnd_v = (int *)ws_take(ctx, (size_t)n * 4 + 4);
  w.bnd_t = (int *)ws_take(ctx, (size_t)n * 4 + 4);
  w.sorted_v = (int *)ws_take(ctx, (size_t)n * 4 + 4);
  w.bhist_ints = (size_t)nblocks * nparts;
  w.bhist = (int *)ws_take(ctx, w.bhist_ints * 4);
  w.acc_ints = nparts > kSmemParts ? (size_t)grid_warps(ctx) * nparts : 0;
  w.acc = w.acc_ints ? (int *)ws_take(ctx, w.acc_ints * 4) : nullptr;
  w.lb_words = (size_t)(n / (kScanThreads * kScanItems) + 4);
  w.lb = (unsigned long long *)ws_take(ctx, w.lb_words * 8);
  w.counters = (unsigned long long *)ws_take(ctx, 64);
  if (!w.pwgts || !w.maxw || !w.minw || !w.pcount || !w.pstart || !w.flag || !w.target || !w.pos || !w.bnd_v ||
      !w.bnd_t || !w.sorted_v || !w.bhist || (w.acc_ints && !w.acc) || !w.lb || !w.counters)
    return cm_fail(CM_ERR_NOMEM, "refine: workspace too small");
  return CM_OK;
}

// One refinement pass over level graph g (device) with partition where.
int refine_pass(cm_ctx *ctx, const cm_graph &g, int nparts, int32_t *where, RefineWs &w, cudaStream_t s,
                const int32_t *proj_cmap = nullptr, const int32_t *proj_cwhere = nullptr) {
  const int n = g.nvtxs;
  if (n == 0) return CM_OK;
  const int sms = ctx->num_sms;
  cudaMemsetAsync(w.pwgts, 0, (size_t)nparts * 4, s);
  const size_t hsh = nparts <= 8192 ? (size_t)nparts * 4 : 0;
  k_part_weights<<<sms * 4, 256, hsh, s>>>(n, where, g.vwgt, nparts, w.pwgts, proj_cmap, proj_cwhere);
  // tpwgts = 1.0 / nparts rounded to float, as cuMetis_set_graph_admin stores it (cu:384)
  k_part_bounds<<<1, 1024, 0, s>>>(nparts, (float)(1.0 / nparts), w.pwgts, w.maxw, w.minw);
  if (nparts <= kSmemParts) {
    const size_t sm = (size_t)kRefWarps * nparts * 4;
    if (sm > 48 * 1024)
      cudaFuncSetAttribute(k_boundary<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_boundary<true><<<sms * 8, kRefThreads, sm, s>>>(n, g.xadj, g.adjncy, g.adjwgt, where, nparts, nullptr, w.flag,
                                                     w.target);
  } else {
    cudaMemsetAsync(w.acc, 0, w.acc_ints * 4, s);
    k_boundary<false><<<sms * 8, kRefThreads, 0, s>>>(n, g.xadj, g.adjncy, g.adjwgt, where, nparts, w.acc, w.flag,
                                                     w.target);
  }
  cudaMemsetAsync(w.lb, 0, w.lb_words * 8, s);
  const int scan_tiles = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  k_scan_flags<<<scan_tiles, kScanThreads, 0, s>>>(w.flag, n, w.pos, w.lb, ctx->d_status);
  k_compact<<<sms * 4, 256, 0, s>>>(n, w.flag, w.pos, w.target, w.bnd_v, w.bnd_t);
  const int *d_nb = w.pos + n;
  const int sort_blocks = (n + kSortBlock - 1) / kSortBlock;
  cudaMemsetAsync(w.bhist, 0, (size_t)sort_blocks * nparts * 4, s);
  k_sort_counts<<<sort_blocks, 256, 0, s>>>(d_nb, w.bnd_t, nparts, w.bhist);
  k_sort_offsets<<<(nparts + 255) / 256, 256, 0, s>>>(d_nb, nparts, w.bhist, w.pcount);
  k_part_starts<<<1, 1024, 0, s>>>(nparts, w.pcount, w.pstart);
  k_sort_scatter<<<sort_blocks, 32, 0, s>>>(d_nb, w.bnd_v, w.bnd_t, nparts, w.bhist, w.pstart, w.sorted_v);
  const int mb = (nparts + 127) / 128;
  k_moves<true><<<mb, 128, 0, s>>>(nparts, w.pstart, w.sorted_v, g.vwgt, w.maxw, w.minw, w.pwgts, where,
                                   w.counters);
  k_moves<false><<<mb, 128, 0, s>>>(nparts, w.pstart, w.sorted_v, g.vwgt, w.maxw, w.minw, w.pwgts, where,
                                    w.counters);
  ctx->launches += 11;
  return check_launch(ctx, "refine");
}

int edge_cut_dev(cm_ctx *ctx, const cm_graph &g, const int32_t *where, unsigned long long *d_out, int64_t *cut,
                 cudaStream_t s) {
  cudaMemsetAsync(d_out, 0, 8, s);
  k_cut<<<ctx->num_sms * 8, 256, 0, s>>>(g.nvtxs, g.xadj, g.adjncy, g.adjwgt, where, d_out);
  ctx->launches++;
  unsigned long long h = 0;
  int rc = cuda_status(cudaMemcpyAsync(&h, d_out, 8, cudaMemcpyDeviceToHost, s), "cut readback");
  if (!rc) rc = stream_wait(ctx, s, "cut sync");
  if (!rc) *cut = (int64_t)(h / 2);
  return rc;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace
}  // namespace cm

using namespace cm;

extern "C" int cm_refine_kway(cm_ctx *ctx, const cm_graph *g_dev, int32_t nparts, int32_t *d_where,
                              int64_t *moves, void *stream) {
  if (!ctx || !g_dev || !d_where || nparts < 1 || g_dev->nvtxs < 0)
    return cm_fail(CM_ERR_INVALID, "cm_refine_kway: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, refine_ws_bytes(ctx, g_dev->nvtxs, nparts)))) return rc;
  RefineWs w;
  if ((rc = take_refine_ws(ctx, g_dev->nvtxs, nparts, w))) return rc;
  cudaMemsetAsync(w.counters, 0, 64, s);
  if ((rc = refine_pass(ctx, *g_dev, nparts, d_where, w, s))) return rc;
  if ((rc = take_device_error(ctx, s))) return rc;
  if (moves) {
    unsigned long long h = 0;
    if ((rc = cuda_status(cudaMemcpyAsync(&h, w.counters, 8, cudaMemcpyDeviceToHost, s), "moves readback")) ||
        (rc = stream_wait(ctx, s, "moves sync")))
      return rc;
    *moves = (int64_t)h;
  }
  return CM_OK;
}

extern "C" int cm_project(cm_ctx *ctx, int32_t n, const int32_t *d_cmap, const int32_t *d_cwhere, int32_t *d_where,
                          void *stream) {
  if (!ctx || n < 0 || (n > 0 && (!d_cmap || !d_cwhere || !d_where)))
    return cm_fail(CM_ERR_INVALID, "cm_project: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  if (n == 0) return CM_OK;
  k_project<<<ctx->num_sms * 4, 256, 0, (cudaStream_t)stream>>>(n, d_cmap, d_cwhere, d_where);
  ctx->launches++;
  return check_launch(ctx, "project");
}

extern "C" void cm_part_default_params(cm_part_params *p) {
  if (!p) return;
  p->seed = 1;
  // Hash-ordered ties: on unit-weight meshes the lowest-id order chains the
  // handshakes (hundreds of rounds per level) while hashed ties settle in a
  // few; both give deterministic heavy-edge matchings.
  p->match_mode = CM_MATCH_HEM_HASH;
  p->refine_passes = 1;
  p->coarsen_to = 0;
}

// Initial partition of the hierarchy's coarsest graph on the host, then per
// level, coarsest to finest, projection and refinement on the context's
// stream (cuMetis_kway_partition after cuMetis_coarsen, cu:3544-3616).  Takes
// the hierarchy (frees it); part receives the finest level's partition.
int part_hierarchy(cm_ctx *ctx, cm_hierarchy *h, int32_t nparts, const cm_part_params &P, int32_t *part,
                   int32_t *objval, cm_part_stats *stats) {
  cm_part_stats S = stats ? *stats : cm_part_stats{};
  int rc = set_device(ctx);
  if (rc) {
    cm_hierarchy_free(h);
    return rc;
  }
  cudaStream_t s = ctx->stream;
  const int32_t nvtxs = h->levels[0].g.nvtxs;
  auto t0 = std::chrono::steady_clock::now();
  const int L = cm_hierarchy_levels(h);
  S.levels = L;
  std::vector<cm_graph> lg(L);
  std::vector<const int32_t *> lcmap(L);
  for (int l = 0; l < L; ++l) cm_hierarchy_level(h, l, &lg[l], &lcmap[l], nullptr);
  S.coarsest_nvtxs = lg[L - 1].nvtxs;

  // Initial partition of the coarsest graph on the host.
  t0 = std::chrono::steady_clock::now();
  cm_graph coarsest{};
  if ((rc = cm_hierarchy_copy_level(h, L - 1, &coarsest, nullptr, nullptr))) {
    cm_hierarchy_free(h);
    return rc;
  }
  std::vector<int32_t> cwhere(std::max(coarsest.nvtxs, 1));
  int32_t initobj = 0;
  rc = cm_initial_partition(&coarsest, nparts, (uint32_t)P.seed, cwhere.data(), &initobj);
  cm_graph_free(&coarsest);
  if (rc) {
    cm_hierarchy_free(h);
    return rc;
  }
  S.init_ms = ms_since(t0);
  S.initial_cut = initobj;

  // Refinement and projection, coarsest to finest.
  t0 = std::chrono::steady_clock::now();
  int64_t total_n = 0;
  for (int l = 0; l < L; ++l) total_n += lg[l].nvtxs;
  int32_t *wbuf = nullptr;
  if ((rc = cuda_status(cudaMallocFromPoolAsync((void **)&wbuf, (size_t)std::max<int64_t>(total_n, 1) * 4, ctx->pool, s), "where alloc"))) {
    cm_hierarchy_free(h);
    return rc;
  }
  std::vector<int32_t *> wl(L);
  {
    int64_t off = 0;
    for (int l = 0; l < L; ++l) {
      wl[l] = wbuf + off;
      off += lg[l].nvtxs;
    }
  }
  auto finish = [&](int code) {
    cudaFreeAsync(wbuf, s);
    stream_wait(ctx, s, "free");
    cm_hierarchy_free(h);
    return code;
  };
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, refine_ws_bytes(ctx, nvtxs, nparts)))) return finish(rc);
  RefineWs w;
  if ((rc = take_refine_ws(ctx, nvtxs, nparts, w))) return finish(rc);
  cudaMemsetAsync(w.counters, 0, 64, s);
  cudaMemcpyAsync(wl[L - 1], cwhere.data(), (size_t)lg[L - 1].nvtxs * 4, cudaMemcpyHostToDevice, s);
  const int passes = std::max(1, P.refine_passes);
  for (int l = L - 1; l >= 0; --l) {
    // the first pass of a finer level projects the coarser partition itself
    for (int p = 0; p < passes; ++p) {
      const bool proj = l < L - 1 && p == 0;
      if ((rc = refine_pass(ctx, lg[l], nparts, wl[l], w, s, proj ? lcmap[l] : nullptr, proj ? wl[l + 1] : nullptr)))
        return finish(rc);
    }
  }
  if ((rc = take_device_error(ctx, s))) return finish(rc);
  int64_t cut = 0;
  if ((rc = edge_cut_dev(ctx, lg[0], wl[0], w.counters + 1, &cut, s))) return finish(rc);
  unsigned long long moves = 0;
  cudaMemcpyAsync(&moves, w.counters, 8, cudaMemcpyDeviceToHost, s);
  if ((rc = cuda_status(cudaMemcpyAsync(part, wl[0], (size_t)nvtxs * 4, cudaMemcpyDeviceToHost, s), "part readback")))
    return finish(rc);
  if ((rc = stream_wait(ctx, s, "part sync"))) return finish(rc);
  S.uncoarsen_ms = ms_since(t0);
  S.moves = (int64_t)moves;
  S.edge_cut = cut;
  if (objval) *objval = (int32_t)cut;
  if (stats) *stats = S;
  return finish(CM_OK);
}

extern "C" int cm_part_graph(cm_ctx *ctx, int32_t nvtxs, const int32_t *xadj, const int32_t *adjncy,
                             const int32_t *vwgt, const int32_t *adjwgt, int32_t nparts, const float *tpwgts,
                             const float *ubvec, int32_t *objval, int32_t *part, const cm_part_params *params,
                             cm_part_stats *stats) {
  (void)tpwgts;  // accepted and ignored, as by the reference (cu:370-394)
  (void)ubvec;
  if (!ctx || nvtxs < 0 || !part || nparts < 1 || (nvtxs > 0 && (!xadj || xadj[nvtxs] < 0 || (xadj[nvtxs] > 0 && !adjncy))))
    return cm_fail(CM_ERR_INVALID, "cm_part_graph: bad arguments");
  cm_part_params P;
  cm_part_default_params(&P);
  if (params) P = *params;
  const auto t_all = std::chrono::steady_clock::now();
  cm_part_stats S{};
  if (nvtxs == 0 || nparts == 1) {
    for (int i = 0; i < nvtxs; ++i) part[i] = 0;
    if (objval) *objval = 0;
    if (stats) *stats = S;
    return CM_OK;
  }
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;  // the context's own stream: concurrent contexts overlap
  const int64_t m = xadj[nvtxs];
  // Unit weights where the caller passes none (cuMetis_set_graph, cu:479-503).
  std::vector<int32_t> uv, ue;
  if (!vwgt) {
    uv.assign(nvtxs, 1);
    vwgt = uv.data();
  }
  if (!adjwgt) {
    ue.assign(std::max<int64_t>(m, 1), 1);
    adjwgt = ue.data();
  }
  cm_graph hg{nvtxs, (int32_t)m, const_cast<int32_t *>(xadj), const_cast<int32_t *>(adjncy), const_cast<int32_t *>(adjwgt),
              const_cast<int32_t *>(vwgt)};
  cm_coarsen_params cp;
  cm_coarsen_default_params(nvtxs, nparts, &cp);
  if (P.coarsen_to > 0) cp.coarsen_to = P.coarsen_to;
  cp.match_mode = P.match_mode;
  cm_hierarchy *h = nullptr;
  auto t0 = std::chrono::steady_clock::now();
  if ((rc = cm_coarsen(ctx, &hg, 0, &cp, &h, s))) return rc;
  S.coarsen_ms = ms_since(t0);
  rc = part_hierarchy(ctx, h, nparts, P, part, objval, &S);
  S.total_ms = ms_since(t_all);
  if (stats) *stats = S;
  return rc;
}

// Drop-in with the reference's parameter list (include/cuMetis.h:18-19): one
// context on the current device for the call.  Returns 1 on success like the
// reference, 0 on failure (message in cm_last_error()) where the reference
// would exit.
extern "C" int cuMetis_PartGraph(int *nvtxs, int *xadj, int *adjncy, int *vwgt, int *adjwgt, int *nparts,
                                 float *tpwgts, float *ubvec, int *objval, int *part) {
  if (!nvtxs || !nparts) {
    cm_fail(CM_ERR_INVALID, "cuMetis_PartGraph: null size arguments");
    return 0;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  cm_ctx *ctx = nullptr;
  if (cm_ctx_create(dev, &ctx) != CM_OK) return 0;
  const int rc = cm_part_graph(ctx, *nvtxs, xadj, adjncy, vwgt, adjwgt, *nparts, tpwgts, ubvec, objval, part,
                               nullptr, nullptr);
  cm_ctx_destroy(ctx);
  return rc == CM_OK ? 1 : 0;
}
