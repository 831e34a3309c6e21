// cm_batch.cu -- coarsening many independent graphs together.  No
// counterpart in the reference, which coarsens one graph per process
// (cuMetis.cu:3874).
//
// The active graphs of a batch are laid side by side as one graph whose
// vertex and entry ranges are the graphs' (a disjoint union), so that one
// matching and one contraction serve every graph of a level.  Per level:
//   join     every active graph's current level -> the union (ids shifted by
//            the graph's first vertex, entry offsets by its first entry);
//   match    the union with per-graph weight caps, the edge hash of the tie
//            rule taken on graph-local ids (a graph matches the same alone and
//            in a batch);
//   contract the union, unchanged: graphs stay contiguous, since the coarse
//            map keeps the leaders' order and a graph's first vertex always
//            leads its pair;
//   sizes    per graph its coarse vertex and entry ranges, read back at once;
//   split    every graph's coarse level into its own 0-based storage (one
//            slab per level for all graphs), and its match and cmap at the
//            finer level.
// Each graph then applies the stop rule of cuMetis_coarsen (cu:1843-1845) to
// its own sizes and leaves the batch once it stops; new graphs may join
// before any level.  The copies of join and split move every level twice; in
// exchange a level of thousands of graphs costs one set of launches.
#include <algorithm>
#include <cstring>
#include <vector>

#include "cm_batch.h"

namespace cm {
namespace {

// A graph's part of a join or split: `count` vertices or entries from
// `start`, of the graph at table index g.
struct Item {
  int g, kind, start, count;
};
enum : int { kItemVertices = 0, kItemEntries = 1, kItemFine = 2 };
constexpr int kItemVertexChunk = 4096, kItemEntryChunk = 8192, kItemThreads = 256;

// Per graph: its arrays (level l for a join; level l+1 and the finer level's
// match/cmap for a split) and its place in the union.
struct Desc {
  const int *xadj, *adjncy, *adjwgt, *vwgt;  // join: the graph's level; split: unused
  int *oxadj, *oadjncy, *oadjwgt, *ovwgt;    // split: the graph's coarse level
  int *omatch, *ocmap;                       // split: the finer level's match and cmap
  int n, m;                                  // join: the level; split: the coarse level
  int vbase, ebase;                          // the graph's first vertex / entry in the union
  int cbase, cebase;                         // split: its first coarse vertex / entry
  int nfine, pad;
};

__global__ void __launch_bounds__(kItemThreads)
k_join(const Item *__restrict__ items, int nitems, const Desc *__restrict__ D, int *__restrict__ xadj,
       int *__restrict__ adjncy, int *__restrict__ adjwgt, int *__restrict__ vwgt, int *__restrict__ vgid, int N,
       int M) {
  if (blockIdx.x == 0 && threadIdx.x == 0) xadj[N] = M;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const Item I = items[it];
    const Desc &d = D[I.g];
    if (I.kind == kItemVertices) {
      for (int t = threadIdx.x; t < I.count; t += kItemThreads) {
        const int i = I.start + t;
        xadj[d.vbase + i] = d.ebase + d.xadj[i];
        vwgt[d.vbase + i] = d.vwgt[i];
        vgid[d.vbase + i] = I.g;
      }
    } else {
      for (int t = threadIdx.x; t < I.count; t += kItemThreads) {
        const int j = I.start + t;
        adjncy[d.ebase + j] = d.adjncy[j] + d.vbase;
        adjwgt[d.ebase + j] = d.adjwgt[j];
      }
    }
  }
}

// Per graph g of the union: its coarse vertex range starts at cmap of its
// first vertex; out[g] = (first coarse vertex, coarse vertices, first coarse
// entry, coarse entries).
__global__ void k_batch_sizes(const int *__restrict__ vbase, int ng, const int *__restrict__ cmap,
                              const int *__restrict__ cxadj, const int *d_sizes, int4 *__restrict__ out) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int cb = cmap[vbase[g]];
    const int ce = g + 1 < ng ? cmap[vbase[g + 1]] : d_sizes[0];
    out[g] = make_int4(cb, ce - cb, cxadj[cb], cxadj[ce] - cxadj[cb]);
  }
}

__global__ void __launch_bounds__(kItemThreads)
k_split(const Item *__restrict__ items, int nitems, const Desc *__restrict__ D, const int *__restrict__ cxadj,
        const int *__restrict__ cadjncy, const int *__restrict__ cadjwgt, const int *__restrict__ cvwgt,
        const int *__restrict__ match, const int *__restrict__ cmap) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const Item I = items[it];
    const Desc &d = D[I.g];
    if (I.kind == kItemVertices) {
      if (I.start == 0 && threadIdx.x == 0) d.oxadj[d.n] = d.m;
      for (int t = threadIdx.x; t < I.count; t += kItemThreads) {
        const int i = I.start + t;
        d.oxadj[i] = cxadj[d.cbase + i] - d.cebase;
        d.ovwgt[i] = cvwgt[d.cbase + i];
      }
    } else if (I.kind == kItemEntries) {
      for (int t = threadIdx.x; t < I.count; t += kItemThreads) {
        const int j = I.start + t;
        d.oadjncy[j] = cadjncy[d.cebase + j] - d.cbase;
        d.oadjwgt[j] = cadjwgt[d.cebase + j];
      }
    } else {
      for (int t = threadIdx.x; t < I.count; t += kItemThreads) {
        const int v = I.start + t;
        d.omatch[v] = match[d.vbase + v] - d.vbase;
        d.ocmap[v] = cmap[d.vbase + v] - d.cbase;
      }
    }
  }
}

void add_items(std::vector<Item> &items, int g, int kind, int64_t count, int chunk) {
  for (int64_t s = 0; s < count; s += chunk) items.push_back({g, kind, (int)s, (int)std::min<int64_t>(chunk, count - s)});
}

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Bytes of one level of a graph of n vertices, m entries in a slab: xadj,
// vwgt, adjncy, adjwgt, match, cmap.
size_t level_bytes(int64_t n, int64_t m) {
  return a256((n + 1) * 4) + 3 * a256(std::max<int64_t>(n, 1) * 4) + 2 * a256(std::max<int64_t>(m, 1) * 4);
}
void carve_level(char *p, int64_t n, int64_t m, cm_level &L) {
  L.g.nvtxs = (int32_t)n;
  L.g.nedges = (int32_t)m;
  L.g.xadj = (int32_t *)p;
  p += a256((n + 1) * 4);
  L.g.vwgt = (int32_t *)p;
  p += a256(std::max<int64_t>(n, 1) * 4);
  L.g.adjncy = (int32_t *)p;
  p += a256(std::max<int64_t>(m, 1) * 4);
  L.g.adjwgt = (int32_t *)p;
  p += a256(std::max<int64_t>(m, 1) * 4);
  L.match = (int32_t *)p;
  p += a256(std::max<int64_t>(n, 1) * 4);
  L.cmap = (int32_t *)p;
  L.block = nullptr;
  L.owns_graph = true;
}

}  // namespace

BatchCoarsener::BatchCoarsener(cm_ctx *ctx, cudaStream_t s) : ctx_(ctx), s_(s) {}

BatchCoarsener::~BatchCoarsener() {
  for (auto &it : active_) cm_hierarchy_free(it.h);
}

int BatchCoarsener::add(int32_t count, const cm_graph *graphs, const cm_coarsen_params *params, const int64_t *tags,
                        std::vector<std::pair<int64_t, cm_hierarchy *>> &finished) {
  int rc = set_device(ctx_);
  if (rc) return rc;
  // Level 0 of every new graph in one slab, copied from the host.
  size_t total = 0;
  for (int i = 0; i < count; ++i) total += level_bytes(graphs[i].nvtxs, graphs[i].nedges);
  char *p = nullptr;
  if ((rc = cuda_status(cudaMallocFromPoolAsync((void **)&p, std::max<size_t>(total, 256), ctx_->pool, s_),
                        "batch level-0 alloc")))
    return rc;
  auto slab = std::make_shared<cm_slab>();
  slab->ptr = p;
  slab->device = ctx_->device;
  slab->stream = s_;
  for (int i = 0; i < count; ++i) {
    const cm_graph &g = graphs[i];
    const int64_t n = g.nvtxs, m = g.nedges;
    Active a;
    a.tag = tags[i];
    a.p = params[i];
    a.h = new cm_hierarchy();
    a.h->device = ctx_->device;
    a.h->stream = s_;
    a.h->slabs.push_back(slab);
    cm_level L;
    carve_level(p, n, m, L);
    p += level_bytes(n, m);
    cudaMemcpyAsync(L.g.xadj, g.xadj, (n + 1) * 4, cudaMemcpyHostToDevice, s_);
    if (n) cudaMemcpyAsync(L.g.vwgt, g.vwgt, n * 4, cudaMemcpyHostToDevice, s_);
    if (m) cudaMemcpyAsync(L.g.adjncy, g.adjncy, m * 4, cudaMemcpyHostToDevice, s_);
    if (m) cudaMemcpyAsync(L.g.adjwgt, g.adjwgt, m * 4, cudaMemcpyHostToDevice, s_);
    a.h->levels.push_back(L);
    int64_t tvwgt = 0, maxdeg = 0;
    for (int64_t v = 0; v < n; ++v) {
      tvwgt += g.vwgt[v];
      maxdeg = std::max<int64_t>(maxdeg, (int64_t)g.xadj[v + 1] - g.xadj[v]);
    }
    // maxvwgt = (int)(1.5 * tvwgt / Coarsen_threshold), cuMetis.cu:1828
    a.h->maxvwgt = a.p.maxvwgt > 0 ? a.p.maxvwgt : (int32_t)(1.5 * (double)tvwgt / a.p.coarsen_to);
    a.row_bound = 2 * maxdeg;
    if (n == 0) {  // nothing to coarsen: an empty coarse level, as cm_coarsen makes
      char *q = nullptr;
      if ((rc = cuda_status(cudaMallocFromPoolAsync((void **)&q, level_bytes(0, 0), ctx_->pool, s_), "batch alloc"))) {
        cm_hierarchy_free(a.h);
        return rc;
      }
      cm_level C;
      carve_level(q, 0, 0, C);
      C.block = q;
      cudaMemsetAsync(C.g.xadj, 0, 4, s_);
      a.h->levels.push_back(C);
      a.h->rounds.push_back(0);
      finished.push_back({a.tag, a.h});
      continue;
    }
    active_.push_back(a);
  }
  return cuda_status(cudaGetLastError(), "batch upload");
}

int BatchCoarsener::step(std::vector<std::pair<int64_t, cm_hierarchy *>> &finished) {
  int rc = set_device(ctx_);
  if (rc) return rc;
  // Groups: one tie order per union, sizes within the int32 CSR limits.
  std::vector<std::vector<int>> groups;
  for (int mode : {CM_MATCH_HEM, CM_MATCH_HEM_HASH, CM_MATCH_RACY}) {
    std::vector<int> cur;
    int64_t N = 0, M = 0;
    for (int i = 0; i < (int)active_.size(); ++i) {
      if (active_[i].p.match_mode != mode) continue;
      const cm_graph &g = active_[i].h->levels.back().g;
      if (!cur.empty() && (N + g.nvtxs > kMaxUnionVertices || M + g.nedges > kMaxUnionEntries)) {
        groups.push_back(cur);
        cur.clear();
        N = M = 0;
      }
      cur.push_back(i);
      N += g.nvtxs;
      M += g.nedges;
    }
    if (!cur.empty()) groups.push_back(cur);
  }
  std::vector<char> stop(active_.size(), 0);
  for (auto &grp : groups)
    if ((rc = level(grp, stop))) return rc;
  std::vector<Active> keep;
  for (size_t i = 0; i < active_.size(); ++i) {
    if (stop[i]) finished.push_back({active_[i].tag, active_[i].h});
    else keep.push_back(active_[i]);
  }
  active_.swap(keep);
  return CM_OK;
}

// One level of the graphs active_[grp[..]] (same tie order).
int BatchCoarsener::level(const std::vector<int> &grp, std::vector<char> &stop) {
  const int ng = (int)grp.size();
  cudaStream_t s = s_;
  int64_t N = 0, M = 0, row_bound = 0;
  int32_t min_cap = INT32_MAX;
  std::vector<int> vbase(ng + 1), ebase(ng + 1), gcap(ng);
  std::vector<Desc> D(ng);
  std::vector<Item> items;
  for (int k = 0; k < ng; ++k) {
    const Active &a = active_[grp[k]];
    const cm_graph &g = a.h->levels.back().g;
    vbase[k] = (int)N;
    ebase[k] = (int)M;
    gcap[k] = a.h->maxvwgt;
    min_cap = std::min(min_cap, a.h->maxvwgt);
    row_bound = std::max(row_bound, a.row_bound);
    Desc &d = D[k];
    std::memset(&d, 0, sizeof d);
    d.xadj = g.xadj;
    d.adjncy = g.adjncy;
    d.adjwgt = g.adjwgt;
    d.vwgt = g.vwgt;
    d.n = g.nvtxs;
    d.m = g.nedges;
    d.vbase = (int)N;
    d.ebase = (int)M;
    add_items(items, k, kItemVertices, g.nvtxs, kItemVertexChunk);
    add_items(items, k, kItemEntries, g.nedges, kItemEntryChunk);
    N += g.nvtxs;
    M += g.nedges;
  }
  vbase[ng] = (int)N;
  ebase[ng] = (int)M;

  // Union buffers from the context's pool: the union (with match, cmap and
  // graph ids), its coarse union, the tables.
  const size_t bN = a256((N + 1) * 4), bM = a256(std::max<int64_t>(M, 1) * 4);
  const size_t bItems = a256(std::max<size_t>(items.size(), 1) * sizeof(Item)), bD = a256(ng * sizeof(Desc));
  const size_t bG = a256((ng + 1) * 4), bSz = a256(ng * sizeof(int4));
  const size_t total = 10 * bN + 4 * bM + bItems + bD + 2 * bG + bSz + 256;
  char *base = nullptr;
  int rc = cuda_status(cudaMallocFromPoolAsync((void **)&base, total, ctx_->pool, s), "batch union alloc");
  if (rc) return rc;
  char *p = base;
  auto take = [&](size_t b) { char *q = p; p += b; return q; };
  cm_graph U{(int32_t)N, (int32_t)M, (int32_t *)take(bN), (int32_t *)take(bM), (int32_t *)take(bM),
             (int32_t *)take(bN)};
  int *vgid = (int *)take(bN), *match = (int *)take(bN), *cmap = (int *)take(bN);
  cm_graph C{(int32_t)N, (int32_t)M, (int32_t *)take(bN), (int32_t *)take(bM), (int32_t *)take(bM),
             (int32_t *)take(bN)};
  Item *d_items = (Item *)take(bItems);
  Desc *d_D = (Desc *)take(bD);
  int *d_vbase = (int *)take(bG), *d_gcap = (int *)take(bG);
  int4 *d_sz = (int4 *)take(bSz);
  (void)take(bN);  // spare
  auto release = [&](int code) {
    cudaFreeAsync(base, s);
    return code;
  };
  cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_D, D.data(), ng * sizeof(Desc), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_vbase, vbase.data(), (ng + 1) * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_gcap, gcap.data(), ng * 4, cudaMemcpyHostToDevice, s);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx_->num_sms * 8, items.size()));
  k_join<<<grid, kItemThreads, 0, s>>>(d_items, (int)items.size(), d_D, U.xadj, U.adjncy, U.adjwgt, U.vwgt, vgid,
                                       (int)N, (int)M);
  ctx_->launches++;
  if ((rc = check_launch(ctx_, "batch join"))) return release(rc);

  // One level of the union.
  ws_reset(ctx_);
  if ((rc = ws_ensure(ctx_, std::max(match_ws_bytes(N, M), contract_ws_bytes(N, M) + 1024) + 4096)))
    return release(rc);
  int32_t *sizes = (int32_t *)ws_take(ctx_, 64);
  const size_t ws_mark = ctx_->ws_used;
  if ((rc = launch_match(ctx_, &U, min_cap, active_[grp[0]].p.match_mode, match, s, vgid, d_vbase, d_gcap)))
    return release(rc);
  ctx_->ws_used = ws_mark;
  if ((rc = launch_contract(ctx_, &U, match, cmap, &C, sizes, s, row_bound))) return release(rc);
  k_batch_sizes<<<(unsigned)((ng + 255) / 256), 256, 0, s>>>(d_vbase, ng, cmap, C.xadj, sizes, d_sz);
  ctx_->launches++;
  std::vector<int4> sz(ng);
  cudaMemcpyAsync(ctx_->h_status, ctx_->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(sz.data(), d_sz, ng * sizeof(int4), cudaMemcpyDeviceToHost, s);
  if ((rc = stream_wait(ctx_, s, "batch level sync"))) return release(rc);
  if (ctx_->h_status->error) {
    rc = take_device_error(ctx_, s);
    return release(rc ? rc : CM_ERR_CUDA);
  }
  const int32_t rounds = ctx_->h_status->rounds;
  const int64_t next_bound = 2 * (int64_t)ctx_->h_status->max_row;

  // Every graph's coarse level in one slab; split the union into it.
  size_t stotal = 0;
  for (int k = 0; k < ng; ++k) stotal += level_bytes(sz[k].y, sz[k].w);
  char *sp = nullptr;
  if ((rc = cuda_status(cudaMallocFromPoolAsync((void **)&sp, std::max<size_t>(stotal, 256), ctx_->pool, s),
                        "batch level alloc")))
    return release(rc);
  auto slab = std::make_shared<cm_slab>();
  slab->ptr = sp;
  slab->device = ctx_->device;
  slab->stream = s;
  items.clear();
  for (int k = 0; k < ng; ++k) {
    Active &a = active_[grp[k]];
    cm_level &F = a.h->levels.back();
    cm_level L;
    carve_level(sp, sz[k].y, sz[k].w, L);
    sp += level_bytes(sz[k].y, sz[k].w);
    Desc &d = D[k];
    d.oxadj = L.g.xadj;
    d.oadjncy = L.g.adjncy;
    d.oadjwgt = L.g.adjwgt;
    d.ovwgt = L.g.vwgt;
    d.omatch = F.match;
    d.ocmap = F.cmap;
    d.n = sz[k].y;
    d.m = sz[k].w;
    d.cbase = sz[k].x;
    d.cebase = sz[k].z;
    d.nfine = F.g.nvtxs;
    add_items(items, k, kItemVertices, sz[k].y, kItemVertexChunk);
    add_items(items, k, kItemEntries, sz[k].w, kItemEntryChunk);
    add_items(items, k, kItemFine, F.g.nvtxs, kItemVertexChunk);
    const int64_t n = F.g.nvtxs, cn = sz[k].y, cm_ = sz[k].w;
    a.h->levels.push_back(L);  // F is not used past this point
    a.h->slabs.push_back(slab);
    a.h->rounds.push_back(rounds);
    a.row_bound = next_bound;
    // stop rule of cuMetis_coarsen (cu:1843-1845), per graph
    const bool go_on = cn > a.p.coarsen_to && (double)cn < a.p.shrink * (double)n && cm_ > cn / 2 &&
                       (int)a.h->levels.size() - 1 < a.p.max_levels;
    stop[grp[k]] = go_on ? 0 : 1;
  }
  Item *d_items2 = nullptr;
  if ((rc = cuda_status(cudaMallocFromPoolAsync((void **)&d_items2, std::max<size_t>(items.size(), 1) * sizeof(Item),
                                                ctx_->pool, s),
                        "batch split items")))
    return release(rc);
  cudaMemcpyAsync(d_items2, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_D, D.data(), ng * sizeof(Desc), cudaMemcpyHostToDevice, s);
  const unsigned grid2 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx_->num_sms * 8, items.size()));
  k_split<<<grid2, kItemThreads, 0, s>>>(d_items2, (int)items.size(), d_D, C.xadj, C.adjncy, C.adjwgt, C.vwgt, match,
                                         cmap);
  ctx_->launches++;
  rc = check_launch(ctx_, "batch split");
  cudaFreeAsync(d_items2, s);
  // host tables above are pageable: the copies have been staged before the
  // calls returned, so the vectors may go
  return release(rc);
}

}  // namespace cm

using namespace cm;

extern "C" int cm_coarsen_batch(cm_ctx *ctx, int32_t ngraphs, const cm_graph *graphs,
                                const cm_coarsen_params *params, cm_hierarchy **out, void *stream) {
  if (!ctx || ngraphs < 0 || (ngraphs > 0 && (!graphs || !params || !out)))
    return cm_fail(CM_ERR_INVALID, "cm_coarsen_batch: bad arguments");
  for (int i = 0; i < ngraphs; ++i) {
    const cm_graph &g = graphs[i];
    if (g.nvtxs < 0 || g.nedges < 0 || (g.nvtxs > 0 && (!g.xadj || !g.vwgt)) || (g.nedges > 0 && (!g.adjncy || !g.adjwgt)) ||
        params[i].coarsen_to < 1)
      return cm_fail(CM_ERR_INVALID, "cm_coarsen_batch: bad graph or parameters at %d", i);
    out[i] = nullptr;
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  BatchCoarsener B(ctx, s);
  std::vector<int64_t> tags(ngraphs);
  for (int i = 0; i < ngraphs; ++i) tags[i] = i;
  std::vector<std::pair<int64_t, cm_hierarchy *>> fin;
  int rc = B.add(ngraphs, graphs, params, tags.data(), fin);
  while (rc == CM_OK && !B.empty()) rc = B.step(fin);
  for (auto &f : fin) out[f.first] = f.second;
  if (rc != CM_OK) {
    for (int i = 0; i < ngraphs; ++i) {
      cm_hierarchy_free(out[i]);
      out[i] = nullptr;
    }
    return rc;
  }
  return cuda_status(cudaStreamSynchronize(s), "cm_coarsen_batch sync");
}
