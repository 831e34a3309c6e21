/*
 * cm.h -- C ABI of libcm, the GB300 (sm_103a) multilevel-coarsening library.
 *
 * The library rebuilds the coarsening hot path of cuMetis (lancunes/cuMetis):
 * heavy-edge matching, coarse-vertex map (cmap) construction and graph
 * contraction (sort of each coarse adjacency row, merge of duplicate edges,
 * summing of edge weights, coarse CSR emit).  Every entry point is plain C:
 * int32 CSR arrays, sizes, a status return and an optional CUDA stream passed
 * as `void *` (a cudaStream_t; NULL = the legacy default stream).
 *
 * Reference interfaces replaced (paths inside the cuMetis project):
 *   cuMetis.cu:1699  int  cuMetis_gpu_match(admin, graph, level)      -> cm_match + cm_build_cmap
 *   cuMetis.cu:1291  void cuMetis_gpu_create_cgraph(admin, graph, ..)  -> cm_contract
 *   cuMetis.cu:1824  cuMetis_graph_t *cuMetis_coarsen(admin, graph)    -> cm_coarsen
 *   include/cuMetis.h:18, cuMetis.cu:3622  cuMetis_PartGraph(...)      -> cm_part_graph / cuMetis_PartGraph
 *   cuMetis.cu:3712  cuMetis_readgraph(filename)                       -> cm_read_graph
 *   cuMetis.cu:3856  cuMetis_writetofile(fname, part, n, nparts)       -> cm_write_partition
 *   cuMetis.cu:356   cuMetis_computecut(graph, where)                  -> cm_edge_cut
 *   mtx_to_graph.c   main (MatrixMarket -> .graph)                     -> cm_read_mtx + cm_write_graph
 *
 * Conventions
 *   - Every function returns CM_OK (0) or a CM_ERR_* code; none calls exit().
 *     cm_last_error() returns a message for the calling thread's last failure.
 *   - Arrays named d_* are device pointers on the context's device; the
 *     caller owns them.  Host graphs filled by cm_gen_* / cm_read_graph are
 *     owned by the library and released with cm_graph_free().
 *   - No global mutable state: all device workspace lives in a cm_ctx.  A
 *     context is used by one host thread at a time.
 */
#ifndef CM_H_
#define CM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  CM_OK = 0,
  CM_ERR_INVALID = 1,     /* bad argument or malformed CSR                    */
  CM_ERR_NOMEM = 2,       /* host/device allocation failed or budget exceeded */
  CM_ERR_CUDA = 3,        /* CUDA runtime error (see cm_last_error)           */
  CM_ERR_LIMIT = 4,       /* a device-side wait or round limit ran out        */
  CM_ERR_IO = 5,          /* file open / parse error                          */
  CM_ERR_UNSUPPORTED = 6  /* sizes beyond int32 CSR limits, no GPU, ...       */
};

/* ---- matching modes ---------------------------------------------------- */
enum {
  /* Heavy-edge matching, deterministic: every vertex prefers its heaviest
   * eligible neighbour, ties to the lower vertex id; conflicts resolved by
   * mutual-proposal handshakes iterated to a fixed point.  The result equals
   * the sequential greedy matching over eligible edges sorted by
   * (weight desc, min endpoint asc, max endpoint asc). */
  CM_MATCH_HEM = 0,
  /* Same, but equal weights are ordered by a fixed hash of the edge's
   * endpoints (fewer handshake rounds on unit-weight meshes). */
  CM_MATCH_HEM_HASH = 1,
  /* One unsynchronised proposal pass plus cleanup, like cuMetis.cu:1563-1630
   * (cuda_shem2, cuda_cleanv, findc1): a light vertex that nobody claimed
   * takes its heaviest neighbour that points at it or is unmatched within
   * the cap, with plain stores; vertices whose partner does not point back
   * become singletons.  Nondeterministic, always a legal matching, not
   * necessarily maximal. */
  CM_MATCH_RACY = 2
};

/* ---- graphs ------------------------------------------------------------ */
typedef struct cm_graph {
  int32_t nvtxs;    /* n                                              */
  int32_t nedges;   /* m = xadj[n], directed adjacency entries (2x undirected) */
  int32_t *xadj;    /* n+1                                            */
  int32_t *adjncy;  /* m                                              */
  int32_t *adjwgt;  /* m                                              */
  int32_t *vwgt;    /* n                                              */
} cm_graph;

/* Host graphs (library-allocated; free with cm_graph_free). */
int  cm_graph_alloc(int32_t nvtxs, int32_t nedges, cm_graph *out);
void cm_graph_free(cm_graph *g);
/* Structural check of a host CSR: monotone xadj, ids in range, no self loops
 * (allowed if allow_self_loops), symmetric adjacency with equal weights. */
int  cm_graph_validate(const cm_graph *g, int check_symmetry, int allow_self_loops);

/* Synthetic inputs, all int32 CSR with rows sorted by neighbour id. */
int cm_gen_tri_grid(int32_t nx, int32_t ny, cm_graph *out);  /* right, down, down-right diagonal */
int cm_gen_grid2d(int32_t nx, int32_t ny, cm_graph *out);    /* 5-point */
int cm_gen_grid3d(int32_t nx, int32_t ny, int32_t nz, cm_graph *out); /* 7-point */
/* R-MAT: edge_factor * 2^scale generated pairs, quadrant probabilities a,b,c
 * (d = 1-a-b-c); self loops and duplicates dropped, symmetrised; edge weights
 * uniform in [wmin, wmax] (same for both directions); vertex weights 1. */
int cm_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                uint64_t seed, int32_t wmin, int32_t wmax, cm_graph *out);
/* Random geometric graph in the unit square, radius sqrt(mean_degree/(pi n)),
 * vertices numbered in cell order; unit weights. */
int cm_gen_rgg(int32_t n, double mean_degree, uint64_t seed, cm_graph *out);

/* METIS .graph IO (formats 0/1/10/11 and the 100s digit, as cuMetis.cu:3712). */
int cm_read_graph(const char *path, cm_graph *out);
int cm_write_graph(const char *path, const cm_graph *g);
/* MatrixMarket coordinate file (square) -> graph with the pattern of A + A^T
 * without the diagonal, unit weights (the reference's mtx_to_graph.c). */
int cm_read_mtx(const char *path, cm_graph *out);
/* Writes "<graph_path>.part.<nparts>", one part id per line (cuMetis.cu:3856). */
int cm_write_partition(const char *graph_path, int32_t nparts, int32_t nvtxs, const int32_t *part);
/* Edge cut (sum of cut edge weights / 2) and max part weight * nparts / total. */
int64_t cm_edge_cut(const cm_graph *g, const int32_t *part);
double  cm_imbalance(const cm_graph *g, int32_t nparts, const int32_t *part);

/* ---- device context ---------------------------------------------------- */
typedef struct cm_ctx cm_ctx;

int  cm_ctx_create(int device, cm_ctx **out);
void cm_ctx_destroy(cm_ctx *ctx);
/* Pre-sizes the context's device workspace for graphs up to n vertices and
 * m entries, so later calls on such graphs do not allocate. */
int  cm_ctx_reserve(cm_ctx *ctx, int64_t nvtxs, int64_t nedges);
const char *cm_last_error(void);
/* Waits for `stream` and returns the first error a kernel of this context
 * recorded since the last check (CM_ERR_LIMIT for a timed-out device wait,
 * CM_ERR_INVALID for an invalid matching), clearing it. */
int cm_ctx_sync(cm_ctx *ctx, void *stream);
/* The context's own non-blocking stream (a cudaStream_t), used by entry
 * points without a stream argument (cm_part_graph). */
void *cm_ctx_stream(const cm_ctx *ctx);
/* Failure-path check without a fault: runs the library's bounded device wait
 * (the decoupled look-back) on a predecessor that never publishes.  Returns
 * CM_ERR_LIMIT after the wait's time limit (about 2 s); the context stays
 * usable. */
int cm_ctx_selftest_wait(cm_ctx *ctx, void *stream);
/* Number of kernels this context has launched since creation. */
int64_t cm_ctx_launch_count(const cm_ctx *ctx);

/* Per-stage timing with CUDA events recorded around each kernel on the
 * caller's stream (replaces the reference's cudaDeviceSynchronize +
 * gettimeofday phase timers, cuMetis.cu:4-144).  cm_ctx_stage_times waits for
 * the recorded events and writes the accumulated milliseconds of up to `cap`
 * stages (CM_STAGE_* order); reset != 0 clears the accumulators. */
enum {
  CM_STAGE_MATCH = 0, /* heavy-edge matching */
  CM_STAGE_CMAP = 1,  /* coarse-vertex map, row bounds, row classes */
  CM_STAGE_ROWS = 2,  /* every coarse row sorted and merged into a stage */
  CM_STAGE_SCAN = 3,  /* cxadj */
  CM_STAGE_COPY = 4,  /* rows from the stage to their final place */
  CM_STAGE_COUNT = 5
};
int cm_ctx_set_stage_timing(cm_ctx *ctx, int enable);
/* Host waits inside the library's calls (per-level size readbacks, the
 * refinement's counters, the partition readback): 0 (default) spins on the
 * stream, lowest latency; 1 sleeps on a blocking-sync event, which frees the
 * core for other host work at the cost of a wake-up per wait.  The engine's
 * workers spin: with one worker per core the batch workload is bound by the
 * GPU, and sleeping measured 8% slower there. */
int cm_ctx_set_blocking_waits(cm_ctx *ctx, int enable);
/* Matching trace: with max_rounds > 0 the next cm_match / cm_coarsen levels
 * record, per handshake round, device timestamps (ns) of the phase starts and
 * the round's work sizes.  cm_ctx_match_trace copies rows of 8 int64 of the
 * last matching: row 0 = {kernel start, init done, round-0 start, end,
 * rounds, 0, 0, 0}; row r+1 = {phase A, phase B, phase C, round end,
 * lane-sized rows, chunked rows, row chunks, wake chunks}.  0 disables. */
int cm_ctx_set_match_trace(cm_ctx *ctx, int32_t max_rounds);
int cm_ctx_match_trace(cm_ctx *ctx, int64_t *out, int32_t cap_rows, int32_t *rows_out);
int cm_ctx_stage_times(cm_ctx *ctx, double *ms, int32_t cap, int reset);
const char *cm_stage_name(int32_t stage);

/* ---- one coarsening level (device arrays) ------------------------------ */
/* Heavy-edge matching (replaces cuMetis.cu:1709-1750: initcuda_match,
 * bb_segsort of each row by weight, cuda_shem2, cuda_cleanv, findc1).
 * Eligible pair (v,k): v != k, vwgt[v]+vwgt[k] <= maxvwgt and
 * 3*vwgt[v] < maxvwgt or 3*vwgt[k] < maxvwgt (cuMetis.cu:1570, 1583).
 * On return d_match[v] = partner, or v for a singleton (match is an
 * involution).  *rounds_out (optional host pointer) receives the number of
 * handshake rounds. The fine graph is not modified. */
int cm_match(cm_ctx *ctx, const cm_graph *g_dev, int32_t maxvwgt, int32_t mode,
             int32_t *d_match, int32_t *rounds_out, void *stream);

/* Coarse-vertex map (replaces findc2, thrust::inclusive_scan, findc2_5, findc3,
 * findc4 at cuMetis.cu:1634-1694,1755-1789 and the host exclusive scan at
 * cuMetis.cu:1304).  Leader = min(v, match[v]); coarse ids are assigned to
 * leaders in increasing order; d_cmap[v] for all v; d_leader[c] = leader of c;
 * d_cvwgt[c] = pair weight sum; d_eoff[c] = exclusive prefix of
 * deg(leader)+deg(follower) (d_eoff[n'] = m); d_cnvtxs[0] = n'.
 * d_leader, d_cvwgt need n entries, d_eoff n+1. */
int cm_build_cmap(cm_ctx *ctx, int32_t nvtxs, const int32_t *d_xadj, const int32_t *d_vwgt,
                  const int32_t *d_match, int32_t *d_cmap, int32_t *d_leader,
                  int32_t *d_cvwgt, int32_t *d_eoff, int32_t *d_cnvtxs, void *stream);

/* cm_build_cmap without any device allocation.  No counterpart in the
 * reference: it exists for callers that must not allocate device memory after
 * start-up (a host whose memory planner owns every device allocation, or a
 * latency-critical loop that cannot absorb the device-wide synchronisation a
 * cudaMalloc may cause).  Same arguments and outputs as cm_build_cmap, minus
 * the context; runs on the current device.  Its scratch is a fixed 64 KB
 * array inside the library, held by every GPU that loads it until exit, so
 * nvtxs is limited to 16,777,216 (larger inputs: CM_ERR_INVALID).  The first
 * call on a device looks up that array's device address; make that first call
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU (other streams, other threads) race and must be serialised by the
 * caller.  Problems the kernels detect are reported in band, once the call's
 * work has run on the stream: d_cnvtxs[0] then holds -CM_ERR_INVALID (an
 * out-of-range or non-involutive matching) or -CM_ERR_LIMIT (a look-back wait
 * past its time limit) instead of n', and the other outputs are not
 * meaningful.  The next call starts clean. */
int cm_build_cmap_noalloc(int32_t nvtxs, const int32_t *d_xadj, const int32_t *d_vwgt,
                          const int32_t *d_match, int32_t *d_cmap, int32_t *d_leader,
                          int32_t *d_cvwgt, int32_t *d_eoff, int32_t *d_cnvtxs, void *stream);

/* Contraction given a matching (replaces cuMetis_gpu_create_cgraph,
 * cuMetis.cu:1291-1406, with its bb_segsort and Sort_cnedges2_part1..3).
 * Output contract: coarse vertex c <-> leader c in increasing leader order;
 * cvwgt[c] = vwgt[leader] + vwgt[follower]; row c = the entries
 * (cmap[x], w) of the leader's and the follower's rows, self loops removed,
 * sorted by coarse id, duplicates merged with weights summed.
 * `coarse` holds device buffers with capacity n+1 (xadj), n (vwgt) and m
 * (adjncy, adjwgt); d_cmap receives n entries; d_sizes (device, 2 ints)
 * receives {n', m'}.  Nothing is read back to the host. */
int cm_contract(cm_ctx *ctx, const cm_graph *fine_dev, const int32_t *d_match,
                int32_t *d_cmap, cm_graph *coarse_dev, int32_t *d_sizes, void *stream);

/* ---- multilevel coarsening --------------------------------------------- */
typedef struct cm_coarsen_params {
  int32_t coarsen_to;      /* stop when n' <= coarsen_to (Coarsen_threshold)   */
  int32_t maxvwgt;         /* <= 0: (int)(1.5 * tvwgt / coarsen_to) (cu:1828)   */
  int32_t match_mode;      /* CM_MATCH_*                                       */
  int32_t max_levels;      /* safety cap, e.g. 64                              */
  double  shrink;          /* continue while n' < shrink * n (0.75, cu:1844)   */
} cm_coarsen_params;

void cm_coarsen_default_params(int32_t nvtxs, int32_t nparts, cm_coarsen_params *p);

typedef struct cm_hierarchy cm_hierarchy;

/* Coarsens a host graph (copied to the device inside the call) or, with
 * input_on_device != 0, a graph whose arrays are already device pointers.
 * The hierarchy keeps every level and each level's cmap on the device. */
int cm_coarsen(cm_ctx *ctx, const cm_graph *g, int input_on_device,
               const cm_coarsen_params *params, cm_hierarchy **out, void *stream);
void    cm_hierarchy_free(cm_hierarchy *h);
int32_t cm_hierarchy_levels(const cm_hierarchy *h);   /* graphs incl. the input */
/* Device view of level l (0 = input); cmap is NULL for the coarsest level. */
int cm_hierarchy_level(const cm_hierarchy *h, int32_t level, cm_graph *g_dev,
                       const int32_t **d_cmap, const int32_t **d_match);
/* Copies level l to a library-allocated host graph, and optionally its cmap
 * and matching (n of level l each; not for the coarsest level). */
int cm_hierarchy_copy_level(const cm_hierarchy *h, int32_t level, cm_graph *out,
                            int32_t *cmap_host, int32_t *match_host);

/* Copies level l into caller-owned host buffers (n+1, m, m, n entries; sizes
 * from cm_hierarchy_level), e.g. pinned memory, on the hierarchy's stream. */
int cm_hierarchy_read_level(const cm_hierarchy *h, int32_t level, int32_t *xadj, int32_t *adjncy,
                            int32_t *adjwgt, int32_t *vwgt);

/* Coarsens ngraphs host graphs together.  No counterpart in the reference
 * (one graph per process).  Every level of all the graphs still coarsening
 * is one graph of their disjoint union -- one matching launch and one
 * contraction for all of them -- after which each graph's coarse level is
 * split back into its own storage and each graph applies the stop rule
 * (params[i]: its threshold, cap, tie order, level limit) on its own sizes.
 * out[i] gets graph i's hierarchy, level for level the same as cm_coarsen
 * of that graph alone.  Levels of different graphs share device
 * allocations, which are released with their last hierarchy. */
int cm_coarsen_batch(cm_ctx *ctx, int32_t ngraphs, const cm_graph *graphs_host,
                     const cm_coarsen_params *params, cm_hierarchy **out, void *stream);

/* ---- partitioning: the tail of cuMetis_PartGraph ------------------------ */

/* Initial partition of a host graph (normally the coarsest level) by
 * multilevel recursive bisection, restating cuMetis_initialpartition
 * (cuMetis.cu:3091) -> cuMetis_rbbisection (3046): per bisection a random
 * heavy-edge coarsening to 200 vertices, 5 region-growing tries, 2-way
 * balancing and Fiduccia-Mattheyses refinement (10 passes) projected back,
 * then the split into two subgraphs.  `seed` seeds the C-library-compatible
 * rand() stream the reference draws from (the reference never seeds it, which
 * is seed 1).  part[nvtxs] gets part ids in [0, nparts); *objval the sum of
 * the bisection cuts.  Host only; g's arrays are host pointers (vwgt/adjwgt
 * may be NULL for unit weights). */
int cm_initial_partition(const cm_graph *g, int32_t nparts, uint32_t seed, int32_t *part, int32_t *objval);

/* One k-way refinement pass of partition d_where (device, n entries) on the
 * device graph g_dev (cuMetis_uncoarsen, cuMetis.cu:3494-3514): boundary
 * vertices move to their best-connected part, group by group per target part,
 * within a 1.03 balance window.  *moves (may be NULL) = vertices moved. */
int cm_refine_kway(cm_ctx *ctx, const cm_graph *g_dev, int32_t nparts, int32_t *d_where, int64_t *moves,
                   void *stream);

/* Projection d_where[v] = d_cwhere[d_cmap[v]] for v < n (cuMetis_kway_project,
 * cuMetis.cu:3079). */
int cm_project(cm_ctx *ctx, int32_t n, const int32_t *d_cmap, const int32_t *d_cwhere, int32_t *d_where,
               void *stream);

typedef struct cm_part_params {
  int32_t seed;          /* initial-partition rand() seed (1 = the reference's stream) */
  int32_t match_mode;    /* CM_MATCH_* for the coarsening (default CM_MATCH_HEM_HASH) */
  int32_t refine_passes; /* refinement passes per level (the reference: 1)        */
  int32_t coarsen_to;    /* 0: max(n / (20 log2 k), 30 k) (cuMetis.cu:3634)         */
} cm_part_params;
void cm_part_default_params(cm_part_params *p);

typedef struct cm_part_stats {
  double coarsen_ms, init_ms, uncoarsen_ms, total_ms;
  int32_t levels;         /* graphs in the hierarchy, input included */
  int32_t coarsest_nvtxs;
  int32_t initial_cut;    /* objective of the initial partition      */
  int64_t edge_cut;       /* final edge cut                          */
  int64_t moves;          /* vertices moved by the refinement        */
} cm_part_stats;

/* k-way partition of a host graph: coarsen on the device, initial partition on
 * the host, refinement and projection per level on the device; part[nvtxs]
 * (caller-allocated) gets ids in [0, nparts).  Host arrays are read, never
 * modified; vwgt/adjwgt may be NULL (unit weights).  tpwgts and ubvec are
 * accepted and ignored, as in the reference (cuMetis.cu:370-394).  Unlike
 * the reference, which leaves *objval = 0 (cu:3615), *objval is the final
 * edge cut.  params/stats may be NULL. */
int cm_part_graph(cm_ctx *ctx, int32_t nvtxs, const int32_t *xadj, const int32_t *adjncy, const int32_t *vwgt,
                  const int32_t *adjwgt, int32_t nparts, const float *tpwgts, const float *ubvec, int32_t *objval,
                  int32_t *part, const cm_part_params *params, cm_part_stats *stats);

/* Drop-in for the reference's entry point, same parameter list
 * (include/cuMetis.h:18-19, cuMetis.cu:3622): a context on the current device
 * for the call.  Returns 1 on success (as the reference), 0 on failure with
 * the message in cm_last_error() where the reference would exit. */
int cuMetis_PartGraph(int *nvtxs, int *xadj, int *adjncy, int *vwgt, int *adjwgt, int *nparts, float *tpwgts,
                      float *ubvec, int *objval, int *part);

/* ---- many graphs: batched and served partitioning ----------------------- */
/* No counterpart in the reference (one graph per process).  An engine is a
 * pool of worker threads on one device, each with its own context and
 * stream; a worker runs cm_part_graph for one job at a time, so jobs overlap
 * on the GPU and their host steps run in parallel.  A job is admitted while
 * the estimated device memory of running jobs stays within hbm_budget_bytes
 * (<= 0: no limit; a job larger than the budget runs alone).  reserve_* size
 * every worker's workspace up front (0: grow on demand, which synchronises
 * the device).  Host arrays of a submitted graph and its part buffer must
 * stay valid until cm_engine_wait returns for the job (or the engine is
 * destroyed). */
typedef struct cm_engine cm_engine;
typedef struct cm_job_info {
  double queue_ms;     /* submit -> start  */
  double run_ms;       /* start -> end     */
  double latency_ms;   /* submit -> end    */
  cm_part_stats stats;
  int32_t status;      /* CM_OK or the job's error code */
} cm_job_info;
/* max_queue > 0 bounds the jobs waiting to start: cm_engine_submit then
 * returns CM_ERR_LIMIT when it is full. */
int  cm_engine_create(int device, int32_t nworkers, int64_t hbm_budget_bytes, int32_t max_queue,
                      int64_t reserve_nvtxs, int64_t reserve_nedges, cm_engine **out);
/* Lets running jobs finish, drops jobs not started (their waiters return
 * CM_ERR_INVALID), waits until every thread has left cm_engine_wait, and
 * frees the engine. */
void cm_engine_destroy(cm_engine *e);
int  cm_engine_submit(cm_engine *e, const cm_graph *g_host, int32_t nparts, const cm_part_params *params,
                      int32_t *part, int64_t *job_id);
/* *done = 1 once the job has finished (non-blocking). */
int  cm_engine_poll(cm_engine *e, int64_t job_id, int32_t *done);
/* Blocks until the job is done; returns its status (the job is forgotten).
 * One waiter per job: a second thread waiting for the same job at the same
 * time gets CM_ERR_INVALID. */
int  cm_engine_wait(cm_engine *e, int64_t job_id, int32_t *objval, cm_job_info *info);
/* Jobs completed and latency percentiles (submit -> end) since the last reset. */
int  cm_engine_stats(cm_engine *e, int64_t *completed, double *p50_ms, double *p99_ms, int reset);

typedef struct cm_batch_stats {
  double setup_ms;     /* engine and workspace creation */
  double run_ms;       /* first submit -> last result   */
  int32_t graphs;
  int64_t sum_nedges;
  int64_t sum_cut;
  double sum_coarsen_ms, sum_init_ms, sum_uncoarsen_ms;  /* per-job phase times, summed */
} cm_batch_stats;
/* Partitions nbatch host graphs (graph i into nparts[i] parts, result in
 * parts[i]) with nworkers workers; objvals[i] (may be NULL) = edge cuts. */
int cm_part_batch(int device, int32_t nworkers, int32_t nbatch, const cm_graph *graphs, const int32_t *nparts,
                  int32_t *const *parts, int32_t *objvals, const cm_part_params *params, cm_batch_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* CM_H_ */
