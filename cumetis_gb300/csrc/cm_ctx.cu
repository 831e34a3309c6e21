// cm_ctx.cu -- device context, workspace, C-ABI entry points for one level
// (cm_match, cm_build_cmap, cm_contract) and the multilevel driver
// (cm_coarsen), which replaces cuMetis_coarsen (cuMetis.cu:1824-1850).
//
// Differences from the reference's level loop, by design:
//   - no cudaMalloc/cudaFree inside a level: per-level graphs come from the
//     context's stream-ordered pool (cudaMallocFromPoolAsync) and scratch from the context
//     workspace, sized once for the input;
//   - no host round trips inside a level: matching, cmap, contraction run
//     back to back on one stream; one 8-byte readback of (n', m') per level
//     feeds the stop rule (cuMetis.cu:1843-1845);
//   - the fine graph is never modified (the reference sorts each level's
//     adjacency by weight in place, cuMetis.cu:1723).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cm_ctx.h"

namespace cm {

int cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return CM_OK;
  if (e == cudaErrorMemoryAllocation) return cm_fail(CM_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return cm_fail(CM_ERR_UNSUPPORTED, "%s: %s", what, cudaGetErrorString(e));
  return cm_fail(CM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(cm_ctx *, const char *what) { return cuda_status(cudaGetLastError(), what); }

void *ws_take(cm_ctx *ctx, size_t bytes) {
  size_t off = (ctx->ws_used + 255) & ~(size_t)255;
  if (off + bytes > ctx->ws_bytes) return nullptr;
  ctx->ws_used = off + bytes;
  return ctx->ws + off;
}

int ws_ensure(cm_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->ws_bytes) return CM_OK;
  int rc = cuda_status(cudaDeviceSynchronize(), "workspace grow (sync)");
  if (rc) return rc;
  if (ctx->ws) cudaFree(ctx->ws);
  ctx->ws = nullptr;
  ctx->ws_bytes = 0;
  rc = cuda_status(cudaMalloc(&ctx->ws, bytes), "workspace grow");
  if (rc) return rc;
  ctx->ws_bytes = bytes;
  return CM_OK;
}

namespace {
cudaEvent_t pool_event(cm_ctx *ctx) {
  if (!ctx->ev_pool.empty()) {
    cudaEvent_t e = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void drain_pending(cm_ctx *ctx) {
  for (auto &p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
      ctx->stage_ms[p.stage] += ms;
    ctx->ev_pool.push_back(p.a);
    ctx->ev_pool.push_back(p.b);
  }
  ctx->pending.clear();
}
}  // namespace

void stage_begin(cm_ctx *ctx, cudaStream_t s) {
  if (!ctx->timing) return;
  ctx->ev_open = pool_event(ctx);
  cudaEventRecord(ctx->ev_open, s);
}

void stage_end(cm_ctx *ctx, int stage, cudaStream_t s) {
  if (!ctx->timing || !ctx->ev_open) return;
  cudaEvent_t b = pool_event(ctx);
  cudaEventRecord(b, s);
  ctx->pending.push_back({stage, ctx->ev_open, b});
  ctx->ev_open = nullptr;
  if (ctx->pending.size() > 4096) drain_pending(ctx);
}

int set_device(cm_ctx *ctx) { return cuda_status(cudaSetDevice(ctx->device), "cudaSetDevice"); }

int stream_wait(cm_ctx *ctx, cudaStream_t s, const char *what) {
  if (!ctx->blocking_waits || !ctx->wait_ev) return cuda_status(cudaStreamSynchronize(s), what);
  int rc = cuda_status(cudaEventRecord(ctx->wait_ev, s), what);
  return rc ? rc : cuda_status(cudaEventSynchronize(ctx->wait_ev), what);
}

// Reads the device status, clears its error, returns it as a CM status.
int take_device_error(cm_ctx *ctx, cudaStream_t s) {
  int rc = cuda_status(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s),
                       "status readback");
  if (rc) return rc;
  rc = stream_wait(ctx, s, "stream sync");
  if (rc) return rc;
  const int err = ctx->h_status->error, site = ctx->h_status->error_site;
  if (err) {
    // Clear the whole block (error word and grid-barrier state): a kernel that
    // gave up may have left the barrier counter mid-way.
    cudaMemsetAsync(ctx->d_status, 0, sizeof(DevStatus), s);
    cudaStreamSynchronize(s);
    static const char *sites[] = {"", "grid barrier wait", "look-back wait", "round limit", "index bounds",
                                  "match is not an involution / out of range"};
    return cm_fail(err, "device reported error %d at %s", err, (site >= 0 && site <= 5) ? sites[site] : "?");
  }
  return CM_OK;
}

namespace {

size_t level_ws_bytes(int64_t n, int64_t m) {
  // matching and contraction run one after the other and share the workspace
  return std::max(match_ws_bytes(n, m), contract_ws_bytes(n, m) + 1024);
}

bool bad_graph(const cm_graph *g) {
  return !g || g->nvtxs < 0 || g->nedges < 0 ||
         (g->nvtxs > 0 && (!g->xadj || !g->vwgt)) || (g->nedges > 0 && (!g->adjncy || !g->adjwgt));
}

// One warp resolving look-back tile 1 while tile 0 never publishes: the
// production wait (lookback_resolve) must give up after its time limit and
// record CM_ERR_LIMIT.
__global__ void k_selftest_wait(unsigned long long *status, DevStatus *st) {
  lookback_exclusive(status, 1, 1ull, st);
}

// Input statistics of a device graph: out[0] = the vertex weights' sum,
// out[1] = the largest degree (bounds the contraction's expanded rows).
__global__ void k_input_stats(const int *vwgt, const int *xadj, long long n, unsigned long long *out) {
  unsigned long long s = 0, d = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    s += (unsigned long long)(long long)vwgt[i];
    d = max(d, (unsigned long long)(unsigned)(xadj[i + 1] - xadj[i]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    d = max(d, __shfl_xor_sync(0xffffffffu, d, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, s);
    atomicMax(out + 1, d);
  }
}

}  // namespace
}  // namespace cm

using namespace cm;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" int cm_ctx_create(int device, cm_ctx **out) {
  if (!out) return cm_fail(CM_ERR_INVALID, "cm_ctx_create: null out");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return cm_fail(CM_ERR_UNSUPPORTED, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= count) return cm_fail(CM_ERR_INVALID, "device %d out of range (%d devices)", device, count);
  cm_ctx *ctx = new cm_ctx();
  ctx->device = device;
  int rc = set_device(ctx);
  cudaDeviceProp prop;
  if (!rc) rc = cuda_status(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  if (!rc && prop.major < 10) rc = cm_fail(CM_ERR_UNSUPPORTED, "device %d is sm_%d%d; libcm is built for sm_103a", device, prop.major, prop.minor);
  if (!rc) {
    ctx->num_sms = prop.multiProcessorCount;
    ctx->max_smem_optin = (int)prop.sharedMemPerBlockOptin;
    rc = cuda_status(cudaMalloc(&ctx->d_status, sizeof(DevStatus)), "status alloc");
  }
  if (!rc) rc = cuda_status(cudaMemset(ctx->d_status, 0, sizeof(DevStatus)), "status init");
  if (!rc) rc = cuda_status(cudaMallocHost(&ctx->h_status, sizeof(DevStatus)), "pinned status alloc");
  if (!rc) rc = cuda_status(cudaMallocHost(&ctx->h_small, 64), "pinned readback alloc");
  if (!rc) rc = cuda_status(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "context stream");
  for (int i = 0; i < cm_ctx::kAux && !rc; ++i) {
    rc = cuda_status(cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking), "aux stream");
    if (!rc) rc = cuda_status(cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming), "aux event");
  }
  if (!rc) rc = cuda_status(cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming), "fork event");
  if (!rc)
    rc = cuda_status(cudaEventCreateWithFlags(&ctx->wait_ev, cudaEventDisableTiming | cudaEventBlockingSync),
                     "wait event");
  if (!rc) {
    // The context's own pool; freed level buffers stay in it between calls.
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    rc = cuda_status(cudaMemPoolCreate(&ctx->pool, &props), "memory pool");
    if (!rc) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  if (rc) {
    cm_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return CM_OK;
}

extern "C" void cm_ctx_destroy(cm_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  drain_pending(ctx);
  for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->ws) cudaFree(ctx->ws);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->h_small) cudaFreeHost(ctx->h_small);
  if (ctx->d_trace) cudaFree(ctx->d_trace);
  for (int i = 0; i < cm_ctx::kAux; ++i) {
    if (ctx->aux[i]) cudaStreamDestroy(ctx->aux[i]);
    if (ctx->join_ev[i]) cudaEventDestroy(ctx->join_ev[i]);
  }
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->wait_ev) cudaEventDestroy(ctx->wait_ev);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);  // blocks still held by hierarchies keep it alive until freed
  delete ctx;
}

extern "C" void *cm_ctx_stream(const cm_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int cm_ctx_selftest_wait(cm_ctx *ctx, void *stream) {
  if (!ctx) return cm_fail(CM_ERR_INVALID, "cm_ctx_selftest_wait: null context");
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, 4096))) return rc;
  unsigned long long *status = (unsigned long long *)ws_take(ctx, 64);
  cudaMemsetAsync(status, 0, 64, s);
  k_selftest_wait<<<1, 32, 0, s>>>(status, ctx->d_status);
  ctx->launches++;
  if ((rc = check_launch(ctx, "selftest wait"))) return rc;
  return take_device_error(ctx, s);
}

extern "C" int cm_ctx_reserve(cm_ctx *ctx, int64_t nvtxs, int64_t nedges) {
  if (!ctx || nvtxs < 0 || nedges < 0) return cm_fail(CM_ERR_INVALID, "cm_ctx_reserve: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  return ws_ensure(ctx, level_ws_bytes(nvtxs, nedges) + 4096);
}

extern "C" int64_t cm_ctx_launch_count(const cm_ctx *ctx) { return ctx ? ctx->launches : -1; }

extern "C" int cm_ctx_set_stage_timing(cm_ctx *ctx, int enable) {
  if (!ctx) return cm_fail(CM_ERR_INVALID, "cm_ctx_set_stage_timing: null context");
  ctx->timing = enable != 0;
  return CM_OK;
}

extern "C" int cm_ctx_set_blocking_waits(cm_ctx *ctx, int enable) {
  if (!ctx) return cm_fail(CM_ERR_INVALID, "cm_ctx_set_blocking_waits: null context");
  ctx->blocking_waits = enable != 0;
  return CM_OK;
}

extern "C" int cm_ctx_stage_times(cm_ctx *ctx, double *ms, int32_t cap, int reset) {
  if (!ctx || (cap > 0 && !ms)) return cm_fail(CM_ERR_INVALID, "cm_ctx_stage_times: bad arguments");
  cudaSetDevice(ctx->device);
  drain_pending(ctx);
  for (int i = 0; i < cap && i < CM_STAGE_COUNT; ++i) ms[i] = ctx->stage_ms[i];
  if (reset)
    for (double &v : ctx->stage_ms) v = 0.0;
  return CM_OK;
}

extern "C" int cm_ctx_set_match_trace(cm_ctx *ctx, int32_t max_rounds) {
  if (!ctx || max_rounds < 0) return cm_fail(CM_ERR_INVALID, "cm_ctx_set_match_trace: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  if (ctx->d_trace) {
    cudaDeviceSynchronize();
    cudaFree(ctx->d_trace);
    ctx->d_trace = nullptr;
    ctx->trace_rows = 0;
  }
  if (max_rounds == 0) return CM_OK;
  const size_t bytes = (size_t)(max_rounds + 1) * 8 * sizeof(unsigned long long);
  if ((rc = cuda_status(cudaMalloc(&ctx->d_trace, bytes), "trace alloc"))) return rc;
  cudaMemset(ctx->d_trace, 0, bytes);
  ctx->trace_rows = max_rounds + 1;
  return CM_OK;
}

extern "C" int cm_ctx_match_trace(cm_ctx *ctx, int64_t *out, int32_t cap_rows, int32_t *rows_out) {
  if (!ctx || !out || cap_rows < 1) return cm_fail(CM_ERR_INVALID, "cm_ctx_match_trace: bad arguments");
  if (!ctx->d_trace) return cm_fail(CM_ERR_INVALID, "cm_ctx_match_trace: tracing is off");
  int rc = set_device(ctx);
  if (rc) return rc;
  const int rows = std::min(cap_rows, ctx->trace_rows);
  if ((rc = cuda_status(cudaDeviceSynchronize(), "trace sync"))) return rc;
  if ((rc = cuda_status(cudaMemcpy(out, ctx->d_trace, (size_t)rows * 64, cudaMemcpyDeviceToHost), "trace copy")))
    return rc;
  if (rows_out) *rows_out = std::min<int64_t>(rows, out[4] + 2);
  return CM_OK;
}

extern "C" const char *cm_stage_name(int32_t stage) {
  static const char *names[CM_STAGE_COUNT] = {"k_match", "k_cmap", "k_rows", "k_count_scan", "k_copy_rows"};
  return stage >= 0 && stage < CM_STAGE_COUNT ? names[stage] : "";
}

extern "C" int cm_ctx_sync(cm_ctx *ctx, void *stream) {
  if (!ctx) return cm_fail(CM_ERR_INVALID, "cm_ctx_sync: null context");
  int rc = set_device(ctx);
  if (rc) return rc;
  return take_device_error(ctx, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// one level
// ---------------------------------------------------------------------------
extern "C" int cm_match(cm_ctx *ctx, const cm_graph *g, int32_t maxvwgt, int32_t mode, int32_t *d_match,
                        int32_t *rounds_out, void *stream) {
  if (!ctx || bad_graph(g) || (g->nvtxs > 0 && !d_match)) return cm_fail(CM_ERR_INVALID, "cm_match: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, match_ws_bytes(g->nvtxs, g->nedges)))) return rc;
  if ((rc = launch_match(ctx, g, maxvwgt, mode, d_match, s))) return rc;
  if (rounds_out) {
    if ((rc = take_device_error(ctx, s))) return rc;
    *rounds_out = ctx->h_status->rounds;
  }
  return CM_OK;
}

extern "C" int cm_build_cmap(cm_ctx *ctx, int32_t nvtxs, const int32_t *d_xadj, const int32_t *d_vwgt,
                             const int32_t *d_match, int32_t *d_cmap, int32_t *d_leader, int32_t *d_cvwgt,
                             int32_t *d_eoff, int32_t *d_cnvtxs, void *stream) {
  if (!ctx || nvtxs < 0 || (nvtxs > 0 && (!d_xadj || !d_vwgt || !d_match || !d_cmap || !d_leader || !d_cvwgt)) ||
      !d_eoff || !d_cnvtxs)
    return cm_fail(CM_ERR_INVALID, "cm_build_cmap: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, cmap_ws_bytes(nvtxs)))) return rc;
  return launch_cmap(ctx, nvtxs, d_xadj, d_vwgt, d_match, d_cmap, d_leader, d_cvwgt, d_eoff, d_cnvtxs, nullptr, 0,
                     1, nullptr, nullptr, nullptr, nullptr, 0, nullptr, (cudaStream_t)stream);
}

extern "C" int cm_contract(cm_ctx *ctx, const cm_graph *fine, const int32_t *d_match, int32_t *d_cmap,
                           cm_graph *coarse, int32_t *d_sizes, void *stream) {
  if (!ctx || bad_graph(fine) || !coarse || !coarse->xadj || !d_sizes ||
      (fine->nvtxs > 0 && (!d_match || !d_cmap || !coarse->vwgt)) ||
      (fine->nedges > 0 && (!coarse->adjncy || !coarse->adjwgt)))
    return cm_fail(CM_ERR_INVALID, "cm_contract: bad arguments");
  int rc = set_device(ctx);
  if (rc) return rc;
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, contract_ws_bytes(fine->nvtxs, fine->nedges)))) return rc;
  return launch_contract(ctx, fine, d_match, d_cmap, coarse, d_sizes, (cudaStream_t)stream, INT64_MAX);
}

// ---------------------------------------------------------------------------
// multilevel coarsening
// ---------------------------------------------------------------------------
extern "C" void cm_coarsen_default_params(int32_t nvtxs, int32_t nparts, cm_coarsen_params *p) {
  if (!p) return;
  // k-way Coarsen_threshold = max(n / (20 log2 k), 30 k), cuMetis.cu:3634
  int lg = 0;
  for (int a = nparts; a > 1; a >>= 1) ++lg;
  int thr = lg > 0 ? nvtxs / (20 * lg) : nvtxs;
  p->coarsen_to = std::max(thr, 30 * std::max(nparts, 1));
  p->maxvwgt = 0;
  p->match_mode = CM_MATCH_HEM;
  p->max_levels = 64;
  p->shrink = 0.75;
}

namespace {
size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// One pooled block holding xadj(n+1), vwgt(n), adjncy(m), adjwgt(m), match(n), cmap(n).
int alloc_level(cm_level &L, int64_t n, int64_t m, cudaMemPool_t pool, cudaStream_t s) {
  const size_t bx = align256((n + 1) * 4), bv = align256(std::max<int64_t>(n, 1) * 4),
               be = align256(std::max<int64_t>(m, 1) * 4);
  const size_t total = bx + bv + 2 * be + 2 * bv;
  char *p = nullptr;
  int rc = cuda_status(cudaMallocFromPoolAsync((void **)&p, total, pool, s), "level alloc");
  if (rc) return rc;
  L.block = p;
  L.g.xadj = (int32_t *)p;
  L.g.vwgt = (int32_t *)(p + bx);
  L.g.adjncy = (int32_t *)(p + bx + bv);
  L.g.adjwgt = (int32_t *)(p + bx + bv + be);
  L.match = (int32_t *)(p + bx + bv + 2 * be);
  L.cmap = (int32_t *)(p + bx + 2 * bv + 2 * be);
  L.owns_graph = true;
  return CM_OK;
}
}  // namespace

extern "C" void cm_hierarchy_free(cm_hierarchy *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  for (auto &L : h->levels)
    if (L.block) cudaFreeAsync(L.block, h->stream);
  cudaStreamSynchronize(h->stream);
  delete h;  // shared slabs are released with their last hierarchy
}

extern "C" int cm_coarsen(cm_ctx *ctx, const cm_graph *g, int input_on_device, const cm_coarsen_params *params,
                          cm_hierarchy **out, void *stream) {
  if (!ctx || bad_graph(g) || !params || !out || params->coarsen_to < 1)
    return cm_fail(CM_ERR_INVALID, "cm_coarsen: bad arguments");
  *out = nullptr;
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n0 = g->nvtxs, m0 = g->nedges;
  ws_reset(ctx);
  if ((rc = ws_ensure(ctx, level_ws_bytes(n0, m0) + 4096))) return rc;

  cm_hierarchy *h = new cm_hierarchy();
  h->device = ctx->device;
  h->stream = s;
  auto fail = [&](int code) { cm_hierarchy_free(h); return code; };

  // Level 0 on the device.
  cm_level L0;
  int64_t tvwgt = 0;
  // Upper bound of the next contraction's expanded row length (twice the
  // largest degree): the contraction skips the kernels of row classes that
  // cannot occur.
  int64_t row_bound = 0;
  if (input_on_device) {
    L0.g = *g;
    L0.owns_graph = false;
    // match + cmap for level 0 from the pool
    char *p = nullptr;
    const size_t bv = align256(std::max<int64_t>(n0, 1) * 4);
    if ((rc = cuda_status(cudaMallocFromPoolAsync((void **)&p, 2 * bv, ctx->pool, s), "level alloc"))) return fail(rc);
    L0.block = p;
    L0.match = (int32_t *)p;
    L0.cmap = (int32_t *)(p + bv);
    unsigned long long *d_stats = (unsigned long long *)ws_take(ctx, 16);
    cudaMemsetAsync(d_stats, 0, 16, s);
    k_input_stats<<<std::max(1, ctx->num_sms * 4), 256, 0, s>>>(g->vwgt, g->xadj, n0, d_stats);
    ctx->launches++;
    unsigned long long *hs = reinterpret_cast<unsigned long long *>(ctx->h_small);
    if ((rc = cuda_status(cudaMemcpyAsync(hs, d_stats, 16, cudaMemcpyDeviceToHost, s), "input stats readback")) ||
        (rc = stream_wait(ctx, s, "input stats sync")))
      return fail(rc);
    tvwgt = (int64_t)hs[0];
    row_bound = 2 * (int64_t)hs[1];
  } else {
    if ((rc = alloc_level(L0, n0, m0, ctx->pool, s))) return fail(rc);
    L0.g.nvtxs = (int32_t)n0;
    L0.g.nedges = (int32_t)m0;
    cudaMemcpyAsync(L0.g.xadj, g->xadj, (n0 + 1) * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(L0.g.vwgt, g->vwgt, n0 * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(L0.g.adjncy, g->adjncy, m0 * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(L0.g.adjwgt, g->adjwgt, m0 * 4, cudaMemcpyHostToDevice, s);
    if ((rc = cuda_status(cudaGetLastError(), "input upload"))) return fail(rc);
    int64_t maxdeg = 0;
    for (int64_t i = 0; i < n0; ++i) {
      tvwgt += g->vwgt[i];
      maxdeg = std::max<int64_t>(maxdeg, (int64_t)g->xadj[i + 1] - g->xadj[i]);
    }
    row_bound = 2 * maxdeg;
  }
  h->levels.push_back(L0);
  // maxvwgt = (int)(1.5 * tvwgt / Coarsen_threshold), cuMetis.cu:1828
  h->maxvwgt = params->maxvwgt > 0 ? params->maxvwgt : (int32_t)(1.5 * (double)tvwgt / params->coarsen_to);
  int32_t *sizes = (int32_t *)ws_take(ctx, 64);
  const size_t level_ws_off = ctx->ws_used;

  for (int level = 0;; ++level) {
    cm_level &F = h->levels.back();
    const int64_t n = F.g.nvtxs, m = F.g.nedges;
    cm_level C;
    if ((rc = alloc_level(C, n, m, ctx->pool, s))) return fail(rc);
    ctx->ws_used = level_ws_off;
    if ((rc = launch_match(ctx, &F.g, h->maxvwgt, params->match_mode, F.match, s))) {
      cudaFreeAsync(C.block, s);
      return fail(rc);
    }
    ctx->ws_used = level_ws_off;
    if ((rc = launch_contract(ctx, &F.g, F.match, F.cmap, &C.g, sizes, s, row_bound))) {
      cudaFreeAsync(C.block, s);
      return fail(rc);
    }
    // one small readback per level: (n', m') and the device status
    cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
    int32_t *hsz = ctx->h_small;
    cudaMemcpyAsync(hsz, sizes, 8, cudaMemcpyDeviceToHost, s);
    if ((rc = stream_wait(ctx, s, "level sync"))) { cudaFreeAsync(C.block, s); return fail(rc); }
    if (ctx->h_status->error) {
      cudaFreeAsync(C.block, s);
      rc = take_device_error(ctx, s);  // also resets the status block
      return fail(rc ? rc : CM_ERR_CUDA);
    }
    h->rounds.push_back(ctx->h_status->rounds);
    // a coarse row holds at most its expanded length: the next level's
    // degrees are at most this level's longest expanded row
    row_bound = 2 * (int64_t)ctx->h_status->max_row;
    C.g.nvtxs = hsz[0];
    C.g.nedges = hsz[1];
    h->levels.push_back(C);
    const int64_t cn = hsz[0], cm_ = hsz[1];
    const bool go_on = cn > params->coarsen_to && (double)cn < params->shrink * (double)n && cm_ > cn / 2 &&
                       (int)h->levels.size() - 1 < params->max_levels;
    if (!go_on) break;
  }
  *out = h;
  return CM_OK;
}

extern "C" int32_t cm_hierarchy_levels(const cm_hierarchy *h) { return h ? (int32_t)h->levels.size() : 0; }

extern "C" int cm_hierarchy_level(const cm_hierarchy *h, int32_t level, cm_graph *g_dev, const int32_t **d_cmap,
                                  const int32_t **d_match) {
  if (!h || level < 0 || level >= (int32_t)h->levels.size()) return cm_fail(CM_ERR_INVALID, "hierarchy level out of range");
  const cm_level &L = h->levels[level];
  const bool last = level == (int32_t)h->levels.size() - 1;
  if (g_dev) *g_dev = L.g;
  if (d_cmap) *d_cmap = last ? nullptr : L.cmap;
  if (d_match) *d_match = last ? nullptr : L.match;
  return CM_OK;
}

extern "C" int cm_hierarchy_copy_level(const cm_hierarchy *h, int32_t level, cm_graph *out, int32_t *cmap_host,
                                       int32_t *match_host) {
  if (!h || !out || level < 0 || level >= (int32_t)h->levels.size())
    return cm_fail(CM_ERR_INVALID, "cm_hierarchy_copy_level: bad arguments");
  const cm_level &L = h->levels[level];
  int rc = cm_graph_alloc(L.g.nvtxs, L.g.nedges, out);
  if (rc) return rc;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  const int64_t n = L.g.nvtxs, m = L.g.nedges;
  cudaMemcpyAsync(out->xadj, L.g.xadj, (n + 1) * 4, cudaMemcpyDeviceToHost, s);
  if (n) cudaMemcpyAsync(out->vwgt, L.g.vwgt, n * 4, cudaMemcpyDeviceToHost, s);
  if (m) cudaMemcpyAsync(out->adjncy, L.g.adjncy, m * 4, cudaMemcpyDeviceToHost, s);
  if (m) cudaMemcpyAsync(out->adjwgt, L.g.adjwgt, m * 4, cudaMemcpyDeviceToHost, s);
  if (cmap_host && n && level < (int32_t)h->levels.size() - 1)
    cudaMemcpyAsync(cmap_host, L.cmap, n * 4, cudaMemcpyDeviceToHost, s);
  if (match_host && n && level < (int32_t)h->levels.size() - 1)
    cudaMemcpyAsync(match_host, L.match, n * 4, cudaMemcpyDeviceToHost, s);
  rc = cuda_status(cudaStreamSynchronize(s), "copy level");
  if (rc) cm_graph_free(out);
  return rc;
}

extern "C" int cm_hierarchy_read_level(const cm_hierarchy *h, int32_t level, int32_t *xadj, int32_t *adjncy,
                                       int32_t *adjwgt, int32_t *vwgt) {
  if (!h || level < 0 || level >= (int32_t)h->levels.size() || !xadj)
    return cm_fail(CM_ERR_INVALID, "cm_hierarchy_read_level: bad arguments");
  const cm_level &L = h->levels[level];
  const int64_t n = L.g.nvtxs, m = L.g.nedges;
  if ((n && !vwgt) || (m && (!adjncy || !adjwgt))) return cm_fail(CM_ERR_INVALID, "cm_hierarchy_read_level: null buffer");
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  cudaMemcpyAsync(xadj, L.g.xadj, (n + 1) * 4, cudaMemcpyDeviceToHost, s);
  if (n) cudaMemcpyAsync(vwgt, L.g.vwgt, n * 4, cudaMemcpyDeviceToHost, s);
  if (m) cudaMemcpyAsync(adjncy, L.g.adjncy, m * 4, cudaMemcpyDeviceToHost, s);
  if (m) cudaMemcpyAsync(adjwgt, L.g.adjwgt, m * 4, cudaMemcpyDeviceToHost, s);
  return cuda_status(cudaStreamSynchronize(s), "read level");
}
