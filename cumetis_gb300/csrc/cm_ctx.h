// cm_ctx.h -- the device context behind the opaque cm_ctx handle (internal).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "cm_device.cuh"

struct cm_ctx {
  int device = 0;
  int num_sms = 0;
  int max_smem_optin = 0;       // bytes of dynamic shared memory a block may opt into
  cm::DevStatus *d_status = nullptr;   // device status block
  cm::DevStatus *h_status = nullptr;   // pinned host mirror for readbacks
  int32_t *h_small = nullptr;          // pinned 64-byte readback buffer
  char *ws = nullptr;           // device workspace (grown on demand)
  size_t ws_bytes = 0;
  size_t ws_used = 0;           // bump pointer of the current call
  int64_t launches = 0;         // kernels launched by this context
  // stage timing (CUDA events around kernels)
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  struct Pending { int stage; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  double stage_ms[CM_STAGE_COUNT] = {0};
  cudaEvent_t ev_open = nullptr;
  // the context's own stream (non-blocking), used by calls without a stream
  // argument (cm_part_graph)
  cudaStream_t stream = nullptr;
  // the context's own stream-ordered memory pool for level graphs and
  // partitions: blocks freed by one context are reused only by that context,
  // so contexts running side by side never wait on each other's streams
  cudaMemPool_t pool = nullptr;
  // internal streams/events for concurrent contraction stages
  static constexpr int kAux = 4;
  cudaStream_t aux[kAux] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork_ev = nullptr, join_ev[kAux] = {nullptr, nullptr, nullptr, nullptr};
  // matching trace (optional): 8 x uint64 per row, row 0 = header
  unsigned long long *d_trace = nullptr;
  int trace_rows = 0;
  // host waits: spin (default) or sleep on a blocking-sync event, which
  // frees the core for other host work (the engine's workers)
  bool blocking_waits = false;
  cudaEvent_t wait_ev = nullptr;
  // launch set-up done once: the contraction kernels' shared-memory limits,
  // the matching kernel's resident blocks per SM (per tie order)
  bool contract_attrs_set = false;
  int match_blocks_per_sm[2] = {0, 0};
  // resident blocks per SM of the contraction's tiny-unit kernel (32- and
  // 64-bit keys) and of its row-class kernels
  int unit_blocks_per_sm[2] = {1, 1};
  int class_blocks_per_sm[16] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
};

// One coarsening level on the device.
struct cm_level {
  cm_graph g{};              // device arrays
  int32_t *match = nullptr;  // device, n (absent on the coarsest level)
  int32_t *cmap = nullptr;   // device, n (absent on the coarsest level)
  void *block = nullptr;     // allocation backing the arrays (freed with the hierarchy), or
  bool owns_graph = true;    // false for a caller-owned input on the device
};

// Device memory shared by the levels of several hierarchies (a batch carves
// every graph's level out of one allocation): freed, stream-ordered, when its
// last user lets go.
struct cm_slab {
  void *ptr = nullptr;
  int device = 0;
  cudaStream_t stream = nullptr;
  ~cm_slab() {
    if (ptr) {
      cudaSetDevice(device);
      cudaFreeAsync(ptr, stream);
    }
  }
};

struct cm_hierarchy {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<cm_level> levels;
  int32_t maxvwgt = 0;
  std::vector<int32_t> rounds;
  std::vector<std::shared_ptr<cm_slab>> slabs;  // shared backing of levels carved from a batch
};

namespace cm {

// Bump-allocates `bytes` (256-byte aligned) from the context workspace for the
// duration of one entry point.  Returns nullptr if it does not fit.
void *ws_take(cm_ctx *ctx, size_t bytes);
// Makes the workspace at least `bytes` large (synchronising the device before
// replacing a smaller buffer).  Returns a CM status.
int ws_ensure(cm_ctx *ctx, size_t bytes);
inline void ws_reset(cm_ctx *ctx) { ctx->ws_used = 0; }

// Stage timing: events recorded on the launch stream around one kernel.
void stage_begin(cm_ctx *ctx, cudaStream_t s);
void stage_end(cm_ctx *ctx, int stage, cudaStream_t s);

// Makes the context's device current.
int set_device(cm_ctx *ctx);
// Waits until the work queued on s so far is done: a stream synchronisation,
// or with ctx->blocking_waits a blocking-sync event (the thread sleeps).
int stream_wait(cm_ctx *ctx, cudaStream_t s, const char *what);
// Reads the device status block on stream s, clears a recorded error and
// returns it as a CM status (CM_OK when none).
int take_device_error(cm_ctx *ctx, cudaStream_t s);

// Records the CUDA error (if any) as the thread's last error; returns a status.
int cuda_status(cudaError_t e, const char *what);
int check_launch(cm_ctx *ctx, const char *what);

// Row classes of the contraction, two per octave: class 2j lists the coarse
// rows of base 2^j < L <= 1.5 base 2^j expanded entries, class 2j+1 those of
// 1.5 base 2^j < L <= base 2^(j+1) (L <= the chunk size; base a power of two
// >= 16), at class_offset(m, base, k) of one list array, at most class_cap
// entries.
constexpr int kRowClasses = 16;
__host__ __device__ inline int64_t class_lo(int base, int k) {  // rows of class k have more entries than this
  return (k & 1) ? (3 * ((int64_t)base << (k >> 1))) / 2 : ((int64_t)base << (k >> 1));
}
__host__ __device__ inline int64_t class_hi(int base, int k) {  // ... and at most this many
  return (k & 1) ? ((int64_t)base << ((k >> 1) + 1)) : (3 * ((int64_t)base << (k >> 1))) / 2;
}
__host__ __device__ inline int64_t class_cap(int64_t m, int base, int k) { return m / class_lo(base, k) + 2; }
__host__ __device__ inline int64_t class_offset(int64_t m, int base, int k) {
  int64_t o = 0;
  for (int i = 0; i < k; ++i) o += class_cap(m, base, i);
  return o;
}

// Workspace bytes each stage needs for a graph of n vertices, m entries.
size_t match_ws_bytes(int64_t n, int64_t m);
size_t cmap_ws_bytes(int64_t n);
size_t contract_ws_bytes(int64_t n, int64_t m);

// Stage launchers shared between entry points (no argument checking).
// vgid/gbase/gcap (optional): several graphs side by side -- vertex v belongs
// to graph vgid[v], whose first vertex is gbase[g] and whose weight cap is
// gcap[g]; maxvwgt is then the smallest cap.
int launch_match(cm_ctx *ctx, const cm_graph *g, int32_t maxvwgt, int32_t mode, int32_t *d_match,
                 cudaStream_t s, const int32_t *vgid = nullptr, const int32_t *gbase = nullptr,
                 const int32_t *gcap = nullptr);
// Rows of more than long_threshold expanded entries are listed: up to
// long_chunk entries by size class (class_offset(m, long_threshold, k) of
// class_list, counts in class_ctr[k]), longer ones as chunked rows.
int launch_cmap(cm_ctx *ctx, int32_t n, const int32_t *xadj, const int32_t *vwgt, const int32_t *match,
                int32_t *cmap, int32_t *leader, int32_t *cvwgt, int32_t *eoff, int32_t *d_cnvtxs,
                int32_t *long_list, int32_t long_threshold, int32_t long_chunk, unsigned long long *d_long_ctr,
                int32_t *chunk_row, int32_t *class_list, int32_t *class_ctr, int64_t m, void *row_meta,
                cudaStream_t s);
// row_bound: an upper bound of the longest expanded coarse row (INT64_MAX
// when unknown); kernels of row classes above it are not launched.
int launch_contract(cm_ctx *ctx, const cm_graph *fine, const int32_t *match, int32_t *cmap, cm_graph *coarse,
                    int32_t *d_sizes, cudaStream_t s, int64_t row_bound);

}  // namespace cm

// Partition of a coarsened graph (cm_refine.cu): the initial partition of the
// hierarchy's coarsest level on the host, then projection and refinement
// level by level on the context's stream.  Frees the hierarchy.
int part_hierarchy(cm_ctx *ctx, cm_hierarchy *h, int32_t nparts, const cm_part_params &P, int32_t *part,
                   int32_t *objval, cm_part_stats *stats);
