// cm_cmap.cu -- coarse-vertex map in one pass with a decoupled look-back scan.
//
// Replaces (cuMetis.cu) findc1/findc2 (1621-1646), thrust::inclusive_scan over
// the leader flags (1758), findc2_5 + the blocking D2H of cnvtxs (1651, 1770),
// findc3/findc4 (1660-1694), the D2H of the degree bounds (1789) and the host
// thrust::exclusive_scan + H2D of the expanded row offsets (1304-1309).
//
// One tile = 2048 fine vertices (8 warps x 8 steps x 32 lanes, coalesced).
// Each vertex contributes the packed pair (leader ? 1 : 0, leader ? L : 0),
// L = deg(v) + deg(match[v]) the expanded coarse-row length, as
// (count << 31 | L); one 64-bit look-back scan yields both the coarse id and
// the expanded offset of every leader.  HBM traffic per vertex: match (4 B),
// xadj (4 B), vwgt (4 B) read; cmap (4 B) written; leader/cvwgt/eoff
// (12 B per coarse vertex) written.
#include "cm_ctx.h"

namespace cm {
namespace {

constexpr int kCmapThreads = 256;
constexpr int kCmapSteps = 8;
constexpr int kCmapTile = kCmapThreads * kCmapSteps;  // 2048 vertices
constexpr unsigned long long kMask31 = (1ull << 31) - 1;

__global__ void __launch_bounds__(kCmapThreads)
k_cmap(int n, const int *__restrict__ xadj, const int *__restrict__ vwgt, const int *__restrict__ match,
       int *__restrict__ cmap, int *__restrict__ leader, int *__restrict__ cvwgt, int *__restrict__ eoff,
       int *__restrict__ d_cnvtxs, int *__restrict__ long_list, int long_thr, unsigned long long *long_ctr,
       int long_chunk, int *__restrict__ chunk_row, int *__restrict__ class_list, int *__restrict__ class_ctr,
       long long m_fine, int4 *__restrict__ row_meta, unsigned long long *__restrict__ lb, DevStatus *st) {
  __shared__ int s_tile;
  __shared__ unsigned long long s_warp[kCmapThreads / 32];
  __shared__ unsigned long long s_excl;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd((unsigned long long *)lb, 1ull);
  __syncthreads();
  const int tile = s_tile;
  const long long wbase = (long long)tile * kCmapTile + wid * (32 * kCmapSteps);

  unsigned long long pre[kCmapSteps];
  unsigned long long carry = 0;
#pragma unroll
  for (int it = 0; it < kCmapSteps; ++it) {
    const long long v = wbase + it * 32 + lane;
    unsigned long long val = 0;
    if (v < n) {
      int u = match[v];
      if (u < 0 || u >= n) {  // not a matching: treat as singleton, report
        record_error(st, CM_ERR_INVALID, ERR_SITE_MATCH_INVALID);
        u = (int)v;
      }
      if (v <= u) {
        int L = xadj[v + 1] - xadj[v];
        if (u != v) L += xadj[u + 1] - xadj[u];
        val = (1ull << 31) | (unsigned long long)L;
      }
    }
    unsigned long long x = warp_inclusive_scan_u64(val);
    pre[it] = carry + x - val;  // exclusive within the warp slice
    carry += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) s_warp[wid] = carry;
  __syncthreads();
  if (wid == 0) {
    unsigned long long w = lane < kCmapThreads / 32 ? s_warp[lane] : 0ull;
    unsigned long long wi = warp_inclusive_scan_u64(w);
    unsigned long long agg = __shfl_sync(0xffffffffu, wi, kCmapThreads / 32 - 1);
    if (lane < kCmapThreads / 32) s_warp[lane] = wi - w;
    unsigned long long ex = lookback_exclusive(lb, tile, agg, st);
    if (lane == 0) s_excl = ex;
  }
  __syncthreads();
  const unsigned long long tbase = s_excl + s_warp[wid];
  int row_max = 0;
#pragma unroll
  for (int it = 0; it < kCmapSteps; ++it) {
    const long long v = wbase + it * 32 + lane;
    int kind = -1, crow = 0;  // a leader's size class (its row goes to that class's list), and its coarse id
    if (v < n) {
      int u = match[v];
      if (u < 0 || u >= n) u = (int)v;
      const unsigned long long P = tbase + pre[it];
      if (v <= u) {
        const int c = (int)(P >> 31);
        const int e = (int)(P & kMask31);
        const int xv = xadj[v], dv = xadj[v + 1] - xv;
        const int xu = u != v ? xadj[u] : 0;
        const int L = dv + (u != v ? xadj[u + 1] - xu : 0);
        cmap[v] = c;
        leader[c] = (int)v;
        // contraction row metadata: leader's row start and length, follower's row start
        if (row_meta) row_meta[c] = make_int4(xv, dv, xu, L);
        cvwgt[c] = (int)((unsigned)vwgt[v] + (u != v ? (unsigned)vwgt[u] : 0u));
        eoff[c] = e;
        if (L > long_thr) {
          if (L > long_chunk) {  // sorted in chunks and merged
            const int nch = (L + long_chunk - 1) / long_chunk;
            unsigned long long old = atomicAdd(long_ctr, (1ull << 32) | (unsigned long long)nch);
            const int idx = (int)(old >> 32);
            const int cbase = (int)(old & 0xffffffffu);
            long_list[2 * idx] = c;
            long_list[2 * idx + 1] = cbase;  // first chunk index of this row
            for (int j = 0; j < nch; ++j) chunk_row[cbase + j] = idx;
          } else {  // sorted whole by one block of the row's size class
            const unsigned q = (unsigned)(L - 1) / (unsigned)(long_thr / 2);  // >= 2
            const int b = 31 - __clz(q);
            kind = min(kRowClasses - 1, 2 * (b - 1) + (int)((q >> (b - 1)) & 1u));
            crow = c;
          }
        }
        row_max = L > row_max ? L : row_max;
      }
      if (v == n - 1) {  // the last vertex closes the scan
        const unsigned long long inc =
            P + ((v <= u) ? ((1ull << 31) |
                             (unsigned long long)((xadj[v + 1] - xadj[v]) + (u != v ? xadj[u + 1] - xadj[u] : 0)))
                          : 0ull);
        const int cn = (int)(inc >> 31);
        *d_cnvtxs = cn;
        eoff[cn] = (int)(inc & kMask31);
      }
    }
    // class-list appends aggregated over the lanes of equal class: one
    // atomicAdd per class present in the warp
    const unsigned peers = __match_any_sync(0xffffffffu, kind);
    if (kind >= 0) {
      const int first = __ffs(peers) - 1;
      int base = 0;
      if (lane == first) base = atomicAdd(class_ctr + kind, __popc(peers));
      base = __shfl_sync(peers, base, first);
      class_list[class_offset(m_fine, long_thr, kind) + base + __popc(peers & ((1u << lane) - 1u))] = crow;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) row_max = max(row_max, __shfl_xor_sync(0xffffffffu, row_max, o));
  if (lane == 0 && row_max > 0) atomicMax(&st->max_row, row_max);
}

// Followers take their leader's id; also checks that match is an involution.
__global__ void k_cmap_followers(int n, const int *__restrict__ match, int *__restrict__ cmap, DevStatus *st) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    int u = match[v];
    if (u < 0 || u >= n) continue;  // already reported by k_cmap
    if (u != v && match[u] != v) record_error(st, CM_ERR_INVALID, ERR_SITE_MATCH_INVALID);
    if (u < v) cmap[v] = cmap[u];
  }
}

}  // namespace

size_t cmap_ws_bytes(int64_t n) { return (size_t)((n + kCmapTile - 1) / kCmapTile + 2) * 8 + 256; }

int launch_cmap(cm_ctx *ctx, int32_t n, const int32_t *xadj, const int32_t *vwgt, const int32_t *match,
                int32_t *cmap, int32_t *leader, int32_t *cvwgt, int32_t *eoff, int32_t *d_cnvtxs,
                int32_t *long_list, int32_t long_threshold, int32_t long_chunk, unsigned long long *d_long_ctr,
                int32_t *chunk_row, int32_t *class_list, int32_t *class_ctr, int64_t m, void *row_meta,
                cudaStream_t s) {
  if (n == 0) {
    cudaMemsetAsync(d_cnvtxs, 0, sizeof(int32_t), s);
    cudaMemsetAsync(eoff, 0, sizeof(int32_t), s);
    return cuda_status(cudaGetLastError(), "cmap(empty)");
  }
  const int ntiles = (n + kCmapTile - 1) / kCmapTile;
  unsigned long long *lb = (unsigned long long *)ws_take(ctx, (size_t)(ntiles + 1) * 8);
  if (!lb) return cm_fail(CM_ERR_NOMEM, "cmap: workspace too small");
  cudaMemsetAsync(lb, 0, (size_t)(ntiles + 1) * 8, s);
  stage_begin(ctx, s);
  k_cmap<<<ntiles, kCmapThreads, 0, s>>>(n, xadj, vwgt, match, cmap, leader, cvwgt, eoff, d_cnvtxs, long_list,
                                          long_list ? long_threshold : INT32_MAX, d_long_ctr,
                                          long_chunk > 0 ? long_chunk : 1, chunk_row, class_list, class_ctr,
                                          (long long)m, (int4 *)row_meta, lb, ctx->d_status);
  ctx->launches++;
  int blocks = ctx->num_sms * 8;
  k_cmap_followers<<<blocks, 256, 0, s>>>(n, match, cmap, ctx->d_status);
  stage_end(ctx, CM_STAGE_CMAP, s);
  ctx->launches++;
  return check_launch(ctx, "cmap");
}

}  // namespace cm

// ---------------------------------------------------------------------------
// cm_build_cmap_noalloc: the same coarse-vertex map for callers that must not
// allocate device memory after start-up -- hosts whose memory planner owns
// every device allocation, or latency-critical loops that cannot absorb the
// device-wide synchronisation a cudaMalloc may cause.  Its only scratch (the
// look-back status words and a status block) is the file-scope array below,
// which every GPU that loads this library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace cm {
namespace {

constexpr int kNoAllocMaxVertices = 1 << 24;                     // 16,777,216
constexpr int kNoAllocTiles = kNoAllocMaxVertices / kCmapTile;   // 8,192
constexpr int kNoAllocStatusWords = (int)((sizeof(DevStatus) + 7) / 8);
constexpr int kNoAllocWords = kNoAllocStatusWords + kNoAllocTiles + 2;  // 65,584 bytes

// [status block][look-back ticket][one status word per tile]
static __device__ __align__(256) unsigned long long g_cmap_noalloc_scratch[kNoAllocWords];

// In host code the array's name is only a stand-in; the device address comes
// from cudaGetSymbolAddress, looked up with that device current on the first
// call that succeeds in doing so (a failed look-up is retried by the next
// call instead of being remembered).
constexpr int kNoAllocMaxDevices = 64;
struct NoAllocDevice {
  std::mutex mu;
  bool ready = false;
  unsigned long long *scratch = nullptr;
  int num_sms = 0;
};
NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];

// Reports, in band, what the kernels recorded in the array's status block:
// *d_cnvtxs becomes -(error code) when an error was recorded.
__global__ void k_noalloc_report(const DevStatus *st, int *d_cnvtxs) {
  const int e = st->error;
  if (e != 0) *d_cnvtxs = -e;
}

}  // namespace
}  // namespace cm

extern "C" int cm_build_cmap_noalloc(int32_t nvtxs, const int32_t *d_xadj, const int32_t *d_vwgt,
                                     const int32_t *d_match, int32_t *d_cmap, int32_t *d_leader,
                                     int32_t *d_cvwgt, int32_t *d_eoff, int32_t *d_cnvtxs, void *stream) {
  using namespace cm;
  if (nvtxs < 0 || (nvtxs > 0 && (!d_xadj || !d_vwgt || !d_match || !d_cmap || !d_leader || !d_cvwgt)) ||
      !d_eoff || !d_cnvtxs)
    return cm_fail(CM_ERR_INVALID, "cm_build_cmap_noalloc: bad arguments");
  if (nvtxs > kNoAllocMaxVertices)
    return cm_fail(CM_ERR_INVALID,
                   "cm_build_cmap_noalloc: %d vertices exceed its fixed scratch (at most %d); use cm_build_cmap",
                   nvtxs, kNoAllocMaxVertices);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cm_build_cmap_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cm_fail(CM_ERR_UNSUPPORTED, "cm_build_cmap_noalloc: device %d", dev);
  NoAllocDevice &D = g_noalloc_devices[dev];
  {
    std::lock_guard<std::mutex> lock(D.mu);
    if (!D.ready) {
      unsigned long long *p = nullptr;
      int sms = 0;
      e = cudaGetSymbolAddress((void **)&p, g_cmap_noalloc_scratch);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess || !p) return cuda_status(e, "cm_build_cmap_noalloc: scratch set-up");
      D.scratch = p;
      D.num_sms = sms;
      D.ready = true;
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (nvtxs == 0) {
    cudaMemsetAsync(d_cnvtxs, 0, sizeof(int32_t), s);
    cudaMemsetAsync(d_eoff, 0, sizeof(int32_t), s);
    return cuda_status(cudaGetLastError(), "cm_build_cmap_noalloc(empty)");
  }
  DevStatus *st = reinterpret_cast<DevStatus *>(D.scratch);
  unsigned long long *lb = D.scratch + kNoAllocStatusWords;
  const int ntiles = (nvtxs + kCmapTile - 1) / kCmapTile;
  // The array keeps the previous call's contents: clear the status block, the
  // ticket and this call's tile words.
  cudaMemsetAsync(D.scratch, 0, (size_t)(kNoAllocStatusWords + ntiles + 1) * 8, s);
  k_cmap<<<ntiles, kCmapThreads, 0, s>>>(nvtxs, d_xadj, d_vwgt, d_match, d_cmap, d_leader, d_cvwgt, d_eoff, d_cnvtxs,
                                          nullptr, INT32_MAX, nullptr, 1, nullptr, nullptr, nullptr, 0, nullptr, lb,
                                          st);
  k_cmap_followers<<<D.num_sms * 8, 256, 0, s>>>(nvtxs, d_match, d_cmap, st);
  k_noalloc_report<<<1, 1, 0, s>>>(st, d_cnvtxs);
  return cuda_status(cudaGetLastError(), "cm_build_cmap_noalloc launch");
}
