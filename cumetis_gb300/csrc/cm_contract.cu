// cm_contract.cu -- graph contraction given a matching.
//
// Replaces cuMetis_gpu_create_cgraph (cuMetis.cu:1291-1406): the host scan of
// row bounds (1304), find_cnvtxsedge_original (1006-1068), the segmented sort
// bb_segsort of every expanded coarse row (1332; include/bb_segsort.h), the
// head flags + thrust scan (Sort_cnedges2_part1, 1072-1156, 1351), the cxadj
// emit and its blocking D2H (part2, 1160-1179, 1367) and the atomicAdd merge
// (part2_5/part3, 1183-1271).
//
// Output contract (fixed by the reference's kernels): coarse row c collects
// (cmap[x], w) over the leader's row then the follower's row, drops the self
// loop cmap[x] == c, is sorted ascending by coarse id, and equal ids are merged
// with their weights summed (int32, wrapping).
//
// Every sort is a shared-memory LSD radix sort with private per-thread digit
// counters (cm_sort.cuh), sized to the row: no comparison network, no hash,
// no atomics in the ranking.  Work split by expanded coarse-row length
// L = deg(leader) + deg(follower):
//   L <= kTinyMax     : tiny units, one warp each.  Unit k owns the rows
//                       whose diagonal (rows before + tiny entries before)
//                       lies in [kD, (k+1)D) (D = kTinyDiag), so it holds
//                       < D + kTinyMax entries of <= D/2 rows; their
//                       (row, coarse id) keys are sorted together.
//   kTinyMax < L <= kChunk : one block per row, sized to the row's class
//                       (two classes per octave, capacities 1.5 and 2 times
//                       a power of two, from 96 to kChunk entries; one warp
//                       up to 512 entries), coarse-id keys only.
//   L > kChunk        : huge rows.  Chunks of kChunk entries are sorted,
//                       merged pairwise (merge path, one launch per pass) and
//                       deduplicated.
// Every row leaves its unique entries in a stage at its expanded offset
// eoff[c] and their number in ucount[c]; a scan of ucount gives cxadj, and
// one warp per row moves the entries to their final place.
#include <algorithm>

#include "cm_ctx.h"
#include "cm_sort.cuh"

namespace cm {
namespace {

__host__ __device__ constexpr int ilog2(int v) { return v <= 1 ? 0 : 1 + ilog2(v >> 1); }

// Tiny units: rows of at most kTinyMax entries, D = kTinyDiag diagonals per
// unit, one warp per unit (fewer than D + kTinyMax entries, at most D/2
// non-empty rows).
#ifndef CM_TINY_MAX
#define CM_TINY_MAX 64
#endif
constexpr int kTinyMax = CM_TINY_MAX;
// Diagonals per unit (a multiple of 32).  A unit's entries stay below
// kTinyDiag + kTinyMax (its last row may run past the unit's diagonals by at
// most one row), which sets the capacity.
#ifndef CM_TINY_DIAG
#define CM_TINY_DIAG (2 * CM_TINY_MAX)
#endif
constexpr int kTinyDiag = CM_TINY_DIAG;
constexpr int kTinyCap = (kTinyDiag + kTinyMax + 31) / 32 * 32;
static_assert(kTinyDiag % 32 == 0 && kTinyDiag >= 2 * kTinyMax && kTinyCap <= 512, "CM_TINY_DIAG");
constexpr int kTinyItems = kTinyCap / 32;
constexpr int kTinyRowsPerLane = kTinyDiag / 32;
constexpr int kTinyMaxNz = kTinyDiag / 2;
constexpr int kTinyRowBits = ilog2(kTinyMaxNz - 1) + 1;
static_assert(kTinyMax == 16 || kTinyMax == 32 || kTinyMax == 64, "CM_TINY_MAX: 16, 32 or 64");
// Rows longer than kChunk are sorted in kChunk-entry chunks and merged.
#ifndef CM_CHUNK
#define CM_CHUNK 16384
#endif
#ifndef CM_CHUNK_THREADS
#define CM_CHUNK_THREADS 1024
#endif
constexpr int kChunk = CM_CHUNK;
constexpr int kChunkThreads = CM_CHUNK_THREADS;
constexpr int kChunkItems = kChunk / kChunkThreads;
static_assert(kChunk == 4096 || kChunk == 8192 || kChunk == 16384, "CM_CHUNK: 4096, 8192 or 16384");
static_assert(kChunkItems >= 1 && kChunkItems <= 16 && kChunkItems * kChunkThreads == kChunk, "CM_CHUNK_THREADS");
// Row classes, two per octave up to kChunk (class_lo / class_hi): class 2j
// holds the rows of kTinyMax 2^j < L <= 1.5 kTinyMax 2^j entries, class 2j+1
// those up to kTinyMax 2^(j+1).  A class's block has max(32, cap / items)
// threads, items = kClassItems for the power-of-two capacities and 3/4 of it
// for the others.
#ifndef CM_CLASS_ITEMS
#define CM_CLASS_ITEMS 16
#endif
constexpr int kClassItems = CM_CLASS_ITEMS;
static_assert(kClassItems == 4 || kClassItems == 8 || kClassItems == 16, "CM_CLASS_ITEMS: 4, 8 or 16");
constexpr int kClasses = 2 * ilog2(kChunk / kTinyMax);
static_assert(kClasses <= kRowClasses, "row classes");
constexpr int class_cap_entries(int k) {
  return (k & 1) ? (kTinyMax << ((k >> 1) + 1)) : (3 * (kTinyMax << (k >> 1))) / 2;
}
constexpr int class_item_target(int k) { return (k & 1) ? kClassItems : (3 * kClassItems) / 4; }
constexpr int class_threads(int k) {
  return class_cap_entries(k) / class_item_target(k) < 32 ? 32 : class_cap_entries(k) / class_item_target(k);
}
// Rows above kCopySplit expanded entries are copied one warp per row, the
// others 32 rows per warp.
constexpr int kCopySplit = 256;
constexpr int class_items(int k) { return class_cap_entries(k) / class_threads(k); }
constexpr bool class_shapes_exact(int k) {
  return k >= kClasses || (class_items(k) * class_threads(k) == class_cap_entries(k) && class_items(k) <= 16 &&
                           class_threads(k) <= 1024 && class_shapes_exact(k + 1));
}
static_assert(class_shapes_exact(0), "size-class block shapes");
constexpr int kCopyBatch = 4;  // stage loads in flight per thread before their stores

// Expanded entry o (0 <= o < L) of a coarse row: the leader's entries first
// (as find_cnvtxsedge_original places them, cuMetis.cu:1014-1020).
__device__ __forceinline__ int expanded_src(int o, int xl, int dl, int xf) { return o < dl ? xl + o : xf + (o - dl); }

// Bits of a coarse id (ids < nc).
__device__ __forceinline__ int id_bits(int nc) { return nc > 1 ? 32 - __clz(nc - 1) : 0; }

// Appends (key, w) for the lanes with keep set to a padded sort buffer at a
// shared counter (warp-aggregated; the order within the buffer is arbitrary).
template <typename K>
__device__ __forceinline__ void append_pair(SortPair<K> *buf, int *ctr, bool keep, K key, int w) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(ctr, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (keep) buf[rslot(base + __popc(m & lanemask_lt()))] = make_pair_kv<K>(key, w);
}

// ---------------------------------------------------------------------------
// One block sorts a segment of one row (class rows and chunks)
// ---------------------------------------------------------------------------
template <int NT, int ITEMS>
struct SegSmem {
  SortPair<unsigned> work[rslots(NT * ITEMS)];
  SortScratch<NT> sc;
  int ctr;
};

// Writes the unique entries (coarse id, summed weight) of entries
// [cs, cs + cnt) of coarse row c's expanded row (metadata md), ascending by
// id, self loops dropped, to dst[0..U).  Returns U.  cnt <= NT * ITEMS; all
// NT threads call it; it ends with a block barrier.
template <int NT, int ITEMS>
__device__ __forceinline__ int segment_sorted_unique(SegSmem<NT, ITEMS> &S, int c, const int4 &md, int cs, int cnt,
                                                     int idbits, const int *__restrict__ adjncy,
                                                     const int *__restrict__ adjwgt, const int *__restrict__ cmap,
                                                     int2 *__restrict__ dst) {
  constexpr int kBatch = ITEMS < 4 ? ITEMS : 4;
  if (threadIdx.x == 0) S.ctr = 0;
  __syncthreads();
  for (int b = 0; b < cnt; b += kBatch * NT) {
    int src[kBatch], x[kBatch], w[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int t = b + u * NT + (int)threadIdx.x;
      src[u] = t < cnt ? expanded_src(cs + t, md.x, md.y, md.z) : -1;
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      x[u] = src[u] >= 0 ? __ldcs(adjncy + src[u]) : 0;
      w[u] = src[u] >= 0 ? __ldcs(adjwgt + src[u]) : 0;
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) x[u] = src[u] >= 0 ? cmap[x[u]] : c;
#pragma unroll
    for (int u = 0; u < kBatch; ++u) append_pair<unsigned>(S.work, &S.ctr, x[u] != c, (unsigned)x[u], w[u]);
  }
  __syncthreads();
  const int n = S.ctr;
  block_radix_sort<unsigned, NT, ITEMS>(S.work, S.sc, n, idbits);
  return block_unique_emit<unsigned, NT, ITEMS>(S.work, n, S.sc, [&](unsigned key, int sum, int q) {
    dst[q] = make_int2((int)key, sum);
  });
}

// Rows of one size class: one block per row writes the row's unique entries
// to stage[eoff[c] ...) and their number to ucount[c].
// Resident blocks per SM asked of the compiler for a class shape (0: no
// bound).  Left to itself the compiler gives these shapes 71-117 registers,
// so that registers, not shared memory, cap their blocks per SM; the bounds
// bring them to 56-72 registers without spills (nvcc 13.0, sm_103a), e.g.
// <256,16> from 2 to 3 blocks and <64,16> from 10 to 14.  <512,16> at 2
// blocks (64 registers, 28 bytes spilled) still gains a little; <64,12> and
// <256,12> spill under any bound that would add a block and gain nothing.
#ifndef CM_MB_32_12
#define CM_MB_32_12 32
#endif
#ifndef CM_MB_32_16
#define CM_MB_32_16 22
#endif
#ifndef CM_MB_64_16
#define CM_MB_64_16 13
#endif
#ifndef CM_MB_128_12
#define CM_MB_128_12 9
#endif
#ifndef CM_MB_128_16
#define CM_MB_128_16 6
#endif
#ifndef CM_MB_256_16
#define CM_MB_256_16 3
#endif
#ifndef CM_MB_64_12
#define CM_MB_64_12 0
#endif
#ifndef CM_MB_256_12
#define CM_MB_256_12 0
#endif
#ifndef CM_MB_512_16
#define CM_MB_512_16 2
#endif
template <int NT, int ITEMS>
constexpr int class_min_blocks() {
  return (NT == 32 && ITEMS == 12)    ? CM_MB_32_12
         : (NT == 32 && ITEMS == 16)  ? CM_MB_32_16
         : (NT == 64 && ITEMS == 12)  ? CM_MB_64_12
         : (NT == 64 && ITEMS == 16)  ? CM_MB_64_16
         : (NT == 128 && ITEMS == 12) ? CM_MB_128_12
         : (NT == 128 && ITEMS == 16) ? CM_MB_128_16
         : (NT == 256 && ITEMS == 12) ? CM_MB_256_12
         : (NT == 256 && ITEMS == 16) ? CM_MB_256_16
         : (NT == 512 && ITEMS == 16) ? CM_MB_512_16
                                      : 0;
}
template <int NT, int ITEMS>
__global__ void __launch_bounds__(NT, class_min_blocks<NT, ITEMS>())
k_class_rows(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
             const int *__restrict__ eoff, const int4 *__restrict__ row_meta, const int *__restrict__ list,
             const int *__restrict__ count, const int *d_cn, int2 *__restrict__ stage, int *__restrict__ ucount) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SegSmem<NT, ITEMS> &S = *reinterpret_cast<SegSmem<NT, ITEMS> *>(smem_raw);
  const int nrows = *count;
  const int idbits = id_bits(*d_cn);
  for (int i = blockIdx.x; i < nrows; i += gridDim.x) {
    const int c = list[i];
    const int4 md = row_meta[c];
    const int U = segment_sorted_unique<NT, ITEMS>(S, c, md, 0, min(md.w, NT * ITEMS), idbits, adjncy, adjwgt, cmap,
                                                   stage + eoff[c]);
    if (threadIdx.x == 0) ucount[c] = U;
  }
}

// Passes a row of length L needs before its chunks form one sorted run.
__host__ __device__ __forceinline__ int merge_passes(int L) {
  int p = 0;
  long long w = kChunk;
  while (w < L) { w <<= 1; ++p; }
  return p;
}

// Chunked rows carry packed entries (coarse id << 32 | weight) through the
// merge passes.  Pad entries have the id kPadId, above every coarse id
// (< 2^31 - 1), so they sort to the end of every merged run.
constexpr unsigned kPadId = 0x7fffffffu;
__device__ __forceinline__ unsigned long long pack_entry(int2 e) {
  return ((unsigned long long)(unsigned)e.x << 32) | (unsigned)e.y;
}
__device__ __forceinline__ int2 unpack_entry(unsigned long long v) {
  return make_int2((int)(unsigned)(v >> 32), (int)(unsigned)v);
}

// Rows longer than kChunk: each chunk of kChunk entries becomes one sorted run
// in stage0 for the merge passes -- its unique entries (duplicates within the
// chunk already merged, self loops dropped), then pad entries up to the
// chunk's length, which sort after every coarse id and are skipped by the
// dedup.  chunk_np[q] = the merge passes the chunk's row needs.
__global__ void __launch_bounds__(kChunkThreads, 1)
k_long_sort(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
            const int *__restrict__ eoff, const int4 *__restrict__ row_meta, const int *__restrict__ long_list,
            const int *__restrict__ chunk_row, const unsigned long long *long_ctr, const int *d_cn,
            int2 *__restrict__ stage, int *__restrict__ ucount, int *__restrict__ chunk_np) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SegSmem<kChunkThreads, kChunkItems> &S = *reinterpret_cast<SegSmem<kChunkThreads, kChunkItems> *>(smem_raw);
  const int nchunks = (int)(*long_ctr & 0xffffffffu);
  const int idbits = id_bits(*d_cn);
  for (int q = blockIdx.x; q < nchunks; q += gridDim.x) {
    const int idx = chunk_row[q];
    const int c = long_list[2 * idx];
    const int4 md = row_meta[c];
    const int j = q - long_list[2 * idx + 1];
    const int cs = j * kChunk;
    const int cnt = min(kChunk, md.w - cs);
    if (j == 0 && threadIdx.x == 0) ucount[c] = 0;  // the dedup adds the chunks' counts
    if (threadIdx.x == 0) chunk_np[q] = merge_passes(md.w);
    int2 *dst = stage + eoff[c] + cs;
    const int U = segment_sorted_unique<kChunkThreads, kChunkItems>(S, c, md, cs, cnt, idbits, adjncy, adjwgt, cmap,
                                                                    dst);
    for (int t = U + threadIdx.x; t < cnt; t += kChunkThreads) dst[t] = make_int2((int)kPadId, 0);
  }
}

// ---------------------------------------------------------------------------
// Unit map: first row of every tiny unit
// ---------------------------------------------------------------------------
constexpr int kMapThreads = 256, kMapItems = 8, kMapTile = kMapThreads * kMapItems;

// Row c costs 1 + (L <= kTinyMax ? L : 0) diagonals; unit k starts at the
// first row whose diagonal (the cost of the rows before it) is >= kD.  A
// single-pass scan over the coarse rows (2048 per tile, decoupled
// look-back).  *unit_last = the unit of the last row.
__global__ void __launch_bounds__(kMapThreads)
k_unit_map(const int *d_cn, const int *__restrict__ eoff, int *__restrict__ first_row, int *unit_last,
           unsigned long long *lb, DevStatus *st) {
  __shared__ int s_tile;
  __shared__ unsigned long long s_warp[kMapThreads / 32];
  __shared__ unsigned long long s_excl;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nc = *d_cn;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(lb, 1ull);
  __syncthreads();
  const int tile = s_tile;
  if ((long long)tile * kMapTile >= nc) return;  // past the last row: nobody looks back at it
  const long long base = (long long)tile * kMapTile + (long long)threadIdx.x * kMapItems;
  int cost[kMapItems];
  unsigned long long sum = 0;
#pragma unroll
  for (int i = 0; i < kMapItems; ++i) {
    const long long c = base + i;
    cost[i] = 0;
    if (c < nc) {
      const int L = eoff[c + 1] - eoff[c];
      cost[i] = 1 + (L <= kTinyMax ? L : 0);
    }
    sum += (unsigned)cost[i];
  }
  const unsigned long long inc = warp_inclusive_scan_u64(sum);
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const unsigned long long x = lane < kMapThreads / 32 ? s_warp[lane] : 0ull;
    const unsigned long long xi = warp_inclusive_scan_u64(x);
    const unsigned long long agg = __shfl_sync(0xffffffffu, xi, kMapThreads / 32 - 1);
    if (lane < kMapThreads / 32) s_warp[lane] = xi - x;
    const unsigned long long ex = lookback_exclusive(lb, tile, agg, st);
    if (lane == 0) s_excl = ex;
  }
  __syncthreads();
  long long d0 = (long long)(s_excl + s_warp[wid] + inc - sum);
#pragma unroll
  for (int i = 0; i < kMapItems; ++i) {
    const long long c = base + i;
    if (c >= nc) break;
    const long long d1 = d0 + cost[i];
    for (long long k = d0 / kTinyDiag + 1; k <= d1 / kTinyDiag; ++k) first_row[k] = (int)c + 1;
    if (c == 0) first_row[0] = 0;
    if (c == nc - 1) *unit_last = (int)(d0 / kTinyDiag);
    d0 = d1;
  }
}

// ---------------------------------------------------------------------------
// Tiny units: one warp each
// ---------------------------------------------------------------------------
template <typename K>
struct TinySmem {
  SortPair<K> work[rslots(kTinyCap)];
  SortScratch<32> sc;
  int4 rmeta[kTinyMaxNz];  // per non-empty row: first entry in the unit, leader row start and length, follower row start
  int rcount[kTinyMaxNz], rfirst[kTinyMaxNz], rdst[kTinyMaxNz];
  unsigned char rowid[kTinyCap];  // sorted row of every gathered entry
  unsigned char nz_row[kTinyMaxNz];
  int ctr;
};
static_assert(kTinyMaxNz <= 256 && kTinyDiag <= 256, "tiny unit row ids are 8-bit");

// One warp per unit (grid-stride over the units).  Per unit: the rows'
// metadata, every entry's row (a max-scan of the rows' first entries), the
// gather of (row << idbits | coarse id, weight) pairs without self loops, a
// radix sort of the keys, and every run of equal keys written once, weights
// summed, to stage[eoff[c] ...) of its row; ucount[c] = the row's unique
// entries (0 for empty rows; rows above kTinyMax are counted by their class).
template <typename K>
__global__ void __launch_bounds__(32)
k_tiny_units(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
             const int *d_sizes, const int *__restrict__ first_row, const int *unit_last,
             const int4 *__restrict__ row_meta, const int *__restrict__ eoff, int2 *__restrict__ stage,
             int *__restrict__ ucount, DevStatus *st) {
  constexpr int RPL = kTinyRowsPerLane;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TinySmem<K> &S = *reinterpret_cast<TinySmem<K> *>(smem_raw);
  const int lane = threadIdx.x;
  const unsigned below = lanemask_lt();
  const int nc = d_sizes[0];
  const int last = *unit_last;
  const int idbits = id_bits(nc);
  const unsigned idmask = idbits >= 32 ? 0xffffffffu : ((1u << idbits) - 1u);
  for (int u = blockIdx.x; u <= last; u += gridDim.x) {
    const int clo = first_row[u];
    const int chi = u < last ? first_row[u + 1] : nc;
    int R = chi - clo;
    if (R < 0 || R > kTinyDiag) {  // inconsistent unit map: report, touch nothing
      if (lane == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
      R = 0;
    }
    // ---- rows: metadata, sorted-row index, entry layout (lane l: rows RPL*l ..)
    int len[RPL], jr[RPL], packed = 0;
    int4 md[RPL];
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
      const int r = lane * RPL + i;
      md[i] = make_int4(0, 0, 0, 0);
      if (r < R) md[i] = row_meta[clo + r];
      const bool tiny = r < R && md[i].w <= kTinyMax;
      len[i] = tiny ? md[i].w : 0;
      if (tiny && len[i] == 0) ucount[clo + r] = 0;
      packed += (len[i] > 0 ? (1 << 16) : 0) + len[i];
    }
    const int incl = warp_inclusive_scan_i32(packed);
    const int tot = __shfl_sync(0xffffffffu, incl, 31);
    int ex = incl - packed;
    int ntot = tot & 0xffff, nnz = tot >> 16;
    if (ntot >= kTinyCap || nnz > kTinyMaxNz) {  // inconsistent row metadata: report, touch nothing
      if (lane == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
      ntot = 0;
      nnz = 0;
#pragma unroll
      for (int i = 0; i < RPL; ++i) len[i] = 0;
    }
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
      jr[i] = -1;
      if (len[i] > 0) {
        const int j = ex >> 16, e0 = ex & 0xffff;
        jr[i] = j;
        S.rmeta[j] = make_int4(e0, md[i].x, md[i].y, md[i].z);
        S.nz_row[j] = (unsigned char)(lane * RPL + i);
        S.rcount[j] = 0;
        ex += (1 << 16) + len[i];
      }
    }
    for (int e = lane; e < kTinyCap; e += 32) S.rowid[e] = 0;
    if (lane == 0) S.ctr = 0;
    __syncwarp();
#pragma unroll
    for (int i = 0; i < RPL; ++i)
      if (jr[i] > 0) S.rowid[S.rmeta[jr[i]].x] = (unsigned char)jr[i];
    __syncwarp();
    {  // every entry's row: inclusive max-scan of the first-entry marks
      unsigned v[kTinyItems], run = 0;
#pragma unroll
      for (int i = 0; i < kTinyItems; ++i) {
        v[i] = S.rowid[lane * kTinyItems + i];
        run = max(run, v[i]);
      }
      unsigned wmax = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, wmax, o);
        if (lane >= o) wmax = max(wmax, y);
      }
      unsigned cur = __shfl_up_sync(0xffffffffu, wmax, 1);
      if (lane == 0) cur = 0;
      __syncwarp();
#pragma unroll
      for (int i = 0; i < kTinyItems; ++i) {
        cur = max(cur, v[i]);
        S.rowid[lane * kTinyItems + i] = (unsigned char)cur;
      }
    }
    __syncwarp();
    // ---- gather (row << idbits | coarse id, weight), self loops dropped
    {
      int src[kTinyItems], x[kTinyItems], w[kTinyItems], jj[kTinyItems];
#pragma unroll
      for (int q = 0; q < kTinyItems; ++q) {
        const int e = q * 32 + lane;
        src[q] = -1;
        jj[q] = 0;
        if (e < ntot) {
          const int j = S.rowid[e];
          jj[q] = j;
          const int4 r = S.rmeta[j];
          src[q] = expanded_src(e - r.x, r.y, r.z, r.w);
        }
      }
#pragma unroll
      for (int q = 0; q < kTinyItems; ++q) {
        x[q] = src[q] >= 0 ? __ldcs(adjncy + src[q]) : 0;
        w[q] = src[q] >= 0 ? __ldcs(adjwgt + src[q]) : 0;
      }
#pragma unroll
      for (int q = 0; q < kTinyItems; ++q) x[q] = src[q] >= 0 ? cmap[x[q]] : -1;
#pragma unroll
      for (int q = 0; q < kTinyItems; ++q) {
        const bool keep = src[q] >= 0 && x[q] != clo + (int)S.nz_row[jj[q]];
        append_pair<K>(S.work, &S.ctr, keep, ((K)jj[q] << idbits) | (K)(unsigned)x[q], w[q]);
      }
    }
    __syncwarp();
    const int n = S.ctr;
    const int rowbits = nnz > 1 ? 32 - __clz(nnz - 1) : 0;
    block_radix_sort<K, 32, kTinyItems>(S.work, S.sc, n, rowbits + idbits);
    // ---- runs of equal keys: per sorted row, its first run's index and its
    // number of runs; then every run to the row's stage
    unsigned hm[kTinyItems];
    int qbase = 0;
#pragma unroll
    for (int r = 0; r < kTinyItems; ++r) {
      const int i = r * 32 + lane;
      const K key = i < n ? S.work[i].k : (K)0;
      const bool head = i < n && (i == 0 || S.work[i - 1].k != key);
      hm[r] = __ballot_sync(0xffffffffu, head);
      if (head) {
        const int j = (int)(key >> idbits);
        const int q = qbase + __popc(hm[r] & below);
        if (i == 0 || (int)(S.work[i - 1].k >> idbits) != j) S.rfirst[j] = q;
        atomicAdd(&S.rcount[j], 1);
      }
      qbase += __popc(hm[r]);
    }
    __syncwarp();
    for (int j = lane; j < nnz; j += 32) {
      const int c = clo + (int)S.nz_row[j];
      S.rdst[j] = eoff[c];
      ucount[c] = S.rcount[j];
    }
    __syncwarp();
    qbase = 0;
#pragma unroll
    for (int r = 0; r < kTinyItems; ++r) {
      const int i = r * 32 + lane;
      if (hm[r] >> lane & 1u) {
        const K key = S.work[i].k;
        unsigned sum = (unsigned)S.work[i].v;
        for (int j2 = i + 1; j2 < n && S.work[j2].k == key; ++j2) sum += (unsigned)S.work[j2].v;
        const int j = (int)(key >> idbits);
        const int q = qbase + __popc(hm[r] & below);
        stage[S.rdst[j] + (q - S.rfirst[j])] = make_int2((int)((unsigned)key & idmask), (int)sum);
      }
      qbase += __popc(hm[r]);
    }
    __syncwarp();
  }
}

// Exclusive scan of the per-row unique counts into cxadj (decoupled look-back
// over 2048-row tiles); d_sizes[1] = m'.
constexpr int kScanThreads = 256, kScanItems = 8;
__global__ void __launch_bounds__(kScanThreads)
k_count_scan(const int *__restrict__ ucount, const int *d_cn, int *__restrict__ cxadj, int *d_sizes,
             unsigned long long *lb, DevStatus *st) {
  __shared__ int s_tile;
  __shared__ unsigned long long s_warp[kScanThreads / 32];
  __shared__ unsigned long long s_excl;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nc = *d_cn;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(lb, 1ull);
  __syncthreads();
  const int tile = s_tile;
  const long long base = (long long)tile * kScanThreads * kScanItems + (long long)threadIdx.x * kScanItems;
  int v[kScanItems];
  unsigned long long sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < nc ? ucount[base + i] : 0;
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
  if (tile == 0 && threadIdx.x == 0) cxadj[0] = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i >= nc) break;
    run += (unsigned)v[i];
    cxadj[base + i + 1] = (int)run;
    if (base + i == nc - 1) d_sizes[1] = (int)run;
  }
}

// Moves every row of at most kCopySplit expanded entries from the stage
// (stage[eoff[c] ..], ucount[c] entries) to its final place cxadj[c].  A warp
// takes 32 consecutive rows: lane l loads row l's offsets and count, a warp
// scan lays the rows' entries out back to back, and the warp then walks them
// 32 at a time (kCopyBatch steps in flight), each lane finding its entry's
// row by a five-step search over the prefixes held in the lanes.
constexpr int kCopyThreads = 256;
__global__ void __launch_bounds__(kCopyThreads)
k_copy_rows(const int *d_cn, const int *__restrict__ eoff, const int *__restrict__ ucount,
            const int *__restrict__ cxadj, const int2 *__restrict__ stage, int *__restrict__ cadjncy,
            int *__restrict__ cadjwgt) {
  const int lane = threadIdx.x & 31;
  const int nc = *d_cn;
  const long long warps = (long long)gridDim.x * (kCopyThreads / 32);
  for (long long base = ((long long)blockIdx.x * (kCopyThreads / 32) + (threadIdx.x >> 5)) * 32; base < nc;
       base += warps * 32) {
    const long long c = base + lane;
    int src = 0, cnt = 0, dst = 0;
    if (c < nc) {
      const int e0 = eoff[c];
      if (eoff[c + 1] - e0 <= kCopySplit) {  // longer rows: one block each
        src = e0;
        cnt = ucount[c];
        dst = cxadj[c];
      }
    }
    const int incl = warp_inclusive_scan_i32(cnt);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - cnt;
    for (int k0 = 0; k0 < total; k0 += 32 * kCopyBatch) {
      int2 e[kCopyBatch];
      int d[kCopyBatch];
#pragma unroll
      for (int q = 0; q < kCopyBatch; ++q) {
        const int k = k0 + 32 * q + lane;
        int r = 0;  // the last row whose first entry is at or before k
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int v = __shfl_sync(0xffffffffu, excl, r + step);
          if (v <= k) r += step;
        }
        const int off = k - __shfl_sync(0xffffffffu, excl, r);
        const int s0 = __shfl_sync(0xffffffffu, src, r), d0 = __shfl_sync(0xffffffffu, dst, r);
        d[q] = k < total ? d0 + off : -1;
        e[q] = k < total ? __ldcs(stage + s0 + off) : make_int2(0, 0);
      }
#pragma unroll
      for (int q = 0; q < kCopyBatch; ++q)
        if (d[q] >= 0) {
          cadjncy[d[q]] = e[q].x;
          cadjwgt[d[q]] = e[q].y;
        }
    }
  }
}

// Items of merge(A[0..alen), B[0..blen)) taken from A among the first diag
// outputs (A wins ties), on packed entries in global memory: the first i in
// [max(0, diag - blen), min(diag, alen)) with A[i] > B[diag - 1 - i], else the
// upper end.  The predicate A[i] <= B[diag - 1 - i] holds on a prefix of the
// range, so one warp probes 32 evenly spaced points per step and keeps the
// gap between the last true and the first false probe: about log32 of the
// range in dependent loads instead of log2.  All 32 lanes call it and get the
// same result.
__device__ __forceinline__ int merge_path_warp(const int2 *A, int alen, const int2 *B, int blen, int diag) {
  const int lane = threadIdx.x & 31;
  int lo = diag > blen ? diag - blen : 0;
  int hi = diag < alen ? diag : alen;
  while (lo < hi) {
    const int stride = (hi - lo + 31) >> 5;  // >= 1; lane 31's probe may lie past hi
    const int pos = lo + lane * stride;
    const bool pred = pos < hi && pack_entry(__ldcg(&A[pos])) <= pack_entry(__ldcg(&B[diag - 1 - pos]));
    const int t = __popc(__ballot_sync(0xffffffffu, pred));  // true probes: lanes 0 .. t-1
    if (t == 0) {
      hi = lo;  // false at lo
    } else {
      hi = min(hi, lo + t * stride);  // first false probe (or the end)
      lo = lo + (t - 1) * stride + 1;  // one past the last true probe
    }
  }
  return lo;
}

// One merge pass per launch: pass p merges run pairs of width kChunk << p
// (launches beyond the longest row's last pass return at once; the host
// launches the most passes a graph of m entries can need).  Work items are
// kMergeOut-sized pieces of output (kMergeSub per chunk).  A block first keeps
// those of its items whose row still needs pass p (one load of chunk_np per
// item, all at once), then per item: two warps find where it starts and ends
// in the two runs (merge path over global memory, 32 probes per step), the
// block loads both windows into shared memory, every thread merges kMergePer
// outputs from there into registers, which then overwrite the window, and the
// block stores the result coalesced.  Small blocks (several per SM) overlap
// one another's load latencies.
#ifndef CM_MERGE_THREADS
#define CM_MERGE_THREADS 256
#endif
#ifndef CM_MERGE_OUT
#define CM_MERGE_OUT 2048
#endif
constexpr int kMergeThreads = CM_MERGE_THREADS;
constexpr int kMergeOut = CM_MERGE_OUT;                 // outputs per work item
constexpr int kMergePer = kMergeOut / kMergeThreads;    // outputs per thread
constexpr int kMergeSub = kChunk / kMergeOut;           // work items per chunk
constexpr int kMergeBlocksPerSm = 65536 / (64 * kMergeThreads);
static_assert(kMergePer * kMergeThreads == kMergeOut && kMergeSub * kMergeOut == kChunk, "merge tiling");
struct MergeSmem {
  unsigned long long win[padded_k<unsigned long long>(kMergeOut)];  // the two input windows, then the output
  int items[kMergeThreads];
  int scan[kMergeThreads / 32 + 1];
  int cut[2];
};

__global__ void __launch_bounds__(kMergeThreads, kMergeBlocksPerSm)
k_long_merge(int p, const int *__restrict__ long_list, const int *__restrict__ chunk_row, const int *__restrict__ eoff,
             const unsigned long long *long_ctr, const int *__restrict__ chunk_np, int2 *stage0, int2 *stage1,
             DevStatus *st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MergeSmem &S = *reinterpret_cast<MergeSmem *>(smem_raw);
  if (p >= merge_passes(st->max_row)) return;
  const long long nitems = (long long)(int)(*long_ctr & 0xffffffffu) * kMergeSub;
  const long long width = (long long)kChunk << p;
  const int2 *src = (p & 1) ? stage1 : stage0;
  int2 *dst = (p & 1) ? stage0 : stage1;
  // the block's items are blockIdx.x + k * gridDim.x, k = 0, 1, ...
  for (long long k0 = 0; blockIdx.x + k0 * gridDim.x < nitems; k0 += kMergeThreads) {
    const long long it = blockIdx.x + (k0 + threadIdx.x) * gridDim.x;
    const int act = it < nitems && chunk_np[it / kMergeSub] > p;
    int nact;
    const int ex = block_exclusive_scan<kMergeThreads>(act, S.scan, &nact);
    if (act) S.items[ex] = (int)it;
    __syncthreads();
    for (int a = 0; a < nact; ++a) {
      const int item = S.items[a];
      const int q = item / kMergeSub;
      const int idx = chunk_row[q];
      const int c = long_list[2 * idx];
      const long long base = eoff[c];
      const int L = eoff[c + 1] - (int)base;
      const int o0 = (q - long_list[2 * idx + 1]) * kChunk + (item % kMergeSub) * kMergeOut;
      if (o0 >= L) continue;  // past the end of the row's last (partial) chunk; uniform per block
      const int ps = (int)((o0 / (2 * width)) * (2 * width));
      const int alen = (int)min(width, (long long)(L - ps));
      const int blen = (int)min(width, (long long)(L - ps - alen));
      const int2 *A = src + base + ps;
      const int2 *B = A + alen;
      const int d0 = o0 - ps, d1 = min(o0 + kMergeOut, ps + alen + blen) - ps;
      const int nout = d1 - d0;
      const int warp = threadIdx.x >> 5;
      if (warp < 2) {
        const int d = warp == 0 ? d0 : d1;
        const int cut = blen == 0 ? min(d, alen) : merge_path_warp(A, alen, B, blen, d);
        if ((threadIdx.x & 31) == 0) S.cut[warp] = cut;
      }
      __syncthreads();
      const int i0 = S.cut[0], i1 = S.cut[1];
      const int na = i1 - i0, nb = nout - na;
      const int j0 = d0 - i0;
      if (na < 0 || nb < 0 || i1 > alen || j0 + nb > blen) {
        // cuts of runs that are not sorted: report, read nothing
        if (threadIdx.x == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
        __syncthreads();
        continue;
      }
      // window: A[i0 .. i1) then B[j0 .. j0 + nb)
      {
        int2 e[kMergePer];
#pragma unroll
        for (int u = 0; u < kMergePer; ++u) {
          const int t = threadIdx.x + u * kMergeThreads;
          e[u] = t < na ? __ldcg(A + i0 + t) : (t < nout ? __ldcg(B + j0 + (t - na)) : make_int2(0, 0));
        }
#pragma unroll
        for (int u = 0; u < kMergePer; ++u) {
          const int t = threadIdx.x + u * kMergeThreads;
          if (t < nout) S.win[padk<unsigned long long>(t)] = pack_entry(e[u]);
        }
      }
      __syncthreads();
      const int od = threadIdx.x * kMergePer;
      const int cnt = max(0, min(kMergePer, nout - od));
      unsigned long long out[kMergePer];
      if (cnt > 0) {
        int lo = od > nb ? od - nb : 0, hi = od < na ? od : na;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (S.win[padk<unsigned long long>(mid)] <= S.win[padk<unsigned long long>(na + od - 1 - mid)]) lo = mid + 1;
          else hi = mid;
        }
        int ia = lo, ib = od - lo;
        const unsigned long long kMax = ~0ull;
        unsigned long long ka = ia < na ? S.win[padk<unsigned long long>(ia)] : kMax;
        unsigned long long kb = ib < nb ? S.win[padk<unsigned long long>(na + ib)] : kMax;
#pragma unroll
        for (int t = 0; t < kMergePer; ++t) {
          const bool takeA = (ib >= nb) || (ia < na && ka <= kb);
          out[t] = takeA ? ka : kb;
          if (t + 1 < cnt) {
            if (takeA) { ++ia; ka = ia < na ? S.win[padk<unsigned long long>(ia)] : kMax; }
            else { ++ib; kb = ib < nb ? S.win[padk<unsigned long long>(na + ib)] : kMax; }
          }
        }
      }
      __syncthreads();
#pragma unroll
      for (int t = 0; t < kMergePer; ++t)
        if (t < cnt) S.win[padk<unsigned long long>(od + t)] = out[t];
      __syncthreads();
      int2 *o = dst + base + ps + d0;
      for (int t = threadIdx.x; t < nout; t += kMergeThreads) o[t] = unpack_entry(S.win[padk<unsigned long long>(t)]);
      __syncthreads();
    }
  }
}

// Merges duplicates of the chunked rows, one block per chunk of the sorted row
// (in stage[merge_passes(L) & 1]): a head is the first entry of a run of equal
// ids that is not a pad; each head's run (which may reach into the next
// chunk) is summed and written, compacted within the chunk, to the other stage
// at eoff[c] + j*kChunk.  chunk_cnt[q] = the chunk's unique entries, also added
// to ucount[c].
constexpr int kDedupThreads = 512, kDedupPer = 4;
__global__ void __launch_bounds__(kDedupThreads)
k_long_dedup(const int *__restrict__ long_list, const int *__restrict__ chunk_row, const int *__restrict__ eoff,
             const unsigned long long *long_ctr, const int2 *stage0, const int2 *stage1, int2 *out0, int2 *out1,
             int *__restrict__ chunk_cnt, int *__restrict__ ucount) {
  __shared__ int scan[kDedupThreads / 32 + 1];
  const int nchunks = (int)(*long_ctr & 0xffffffffu);
  for (int q = blockIdx.x; q < nchunks; q += gridDim.x) {
    const int idx = chunk_row[q];
    const int c = long_list[2 * idx];
    const int L = eoff[c + 1] - eoff[c];
    const int j = q - long_list[2 * idx + 1];
    const int fb = merge_passes(L) & 1;
    const int2 *src = (fb ? stage1 : stage0) + eoff[c];
    int2 *dst = (fb ? out0 : out1) + eoff[c] + (long long)j * kChunk;
    const int lo = j * kChunk, hi = min(L, lo + kChunk);
    int carry = 0;
    // Each thread takes kDedupPer consecutive entries (loaded together with
    // the entry before them); a head's run is summed from the thread's own
    // entries and, past them, from global memory.
    for (int b = lo; b < hi; b += kDedupThreads * kDedupPer) {
      const int i0 = b + threadIdx.x * kDedupPer;
      int2 e[kDedupPer];
      const int prev = i0 > 0 && i0 < hi ? src[i0 - 1].x : (int)kPadId;
#pragma unroll
      for (int u = 0; u < kDedupPer; ++u) e[u] = i0 + u < L ? src[i0 + u] : make_int2((int)kPadId, 0);  // runs may cross hi
      bool h[kDedupPer];
      int nh = 0;
#pragma unroll
      for (int u = 0; u < kDedupPer; ++u) {
        const int before = u == 0 ? prev : e[u - 1].x;
        h[u] = i0 + u < hi && (unsigned)e[u].x < kPadId && (i0 + u == 0 || before != e[u].x);
        nh += h[u];
      }
      int tot;
      int o = carry + block_exclusive_scan<kDedupThreads>(nh, scan, &tot);
#pragma unroll
      for (int u = 0; u < kDedupPer; ++u) {
        if (!h[u]) continue;
        unsigned sum = (unsigned)e[u].y;
        bool open = true;  // the run still reaches the next entry
#pragma unroll
        for (int v = u + 1; v < kDedupPer; ++v) {
          open = open && e[v].x == e[u].x;
          if (open) sum += (unsigned)e[v].y;
        }
        if (open)
          for (int k = i0 + kDedupPer; k < L && src[k].x == e[u].x; ++k) sum += (unsigned)src[k].y;
        dst[o++] = make_int2(e[u].x, (int)sum);
      }
      carry += tot;
    }
    if (threadIdx.x == 0) {
      chunk_cnt[q] = carry;
      atomicAdd(&ucount[c], carry);
    }
  }
}

// Moves the class rows above kCopySplit expanded entries from the stage to
// their final place: one warp per row, 2 kCopyBatch loads in flight per
// lane.
__global__ void __launch_bounds__(256)
k_copy_class_rows(const int *__restrict__ class_list, const int *__restrict__ class_ctr, long long m,
                  const int *__restrict__ eoff, const int *__restrict__ ucount, const int *__restrict__ cxadj,
                  const int2 *__restrict__ stage, int *__restrict__ cadjncy, int *__restrict__ cadjwgt) {
  constexpr int k0 = 2 * ilog2(kCopySplit / kTinyMax);  // first class copied here (rows above kCopySplit)
  constexpr int kBatch = 2 * kCopyBatch;             // stage loads in flight per lane
  const int lane = threadIdx.x & 31;
  // per class: its first row in this kernel's numbering and its list's offset
  __shared__ int s_first[kClasses + 1];
  __shared__ long long s_off[kClasses];
  if (threadIdx.x == 0) {
    int t = 0;
    for (int k = 0; k < kClasses; ++k) {
      s_first[k] = t;
      s_off[k] = class_offset(m, kTinyMax, k);
      t += k >= k0 ? class_ctr[k] : 0;
    }
    s_first[kClasses] = t;
  }
  __syncthreads();
  const int total = s_first[kClasses];
  // one warp per row: many rows' metadata loads in flight per SM
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < total; i += nw) {
    int k = k0;
    while (i >= s_first[k + 1]) ++k;
    const int c = class_list[s_off[k] + (i - s_first[k])];
    const int n = ucount[c];
    const int2 *src = stage + eoff[c];
    const long long dst = cxadj[c];
    for (int t0 = lane; t0 < n; t0 += kBatch * 32) {
      int2 e[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int t = t0 + u * 32;
        e[u] = t < n ? __ldcs(src + t) : make_int2(0, 0);
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int t = t0 + u * 32;
        if (t < n) {
          cadjncy[dst + t] = e[u].x;
          cadjwgt[dst + t] = e[u].y;
        }
      }
    }
  }
}

// Copies the chunked rows' unique entries to their final place once cxadj is
// known: each chunk at cxadj[c] + the unique entries of the row's earlier
// chunks.
__global__ void k_long_copy(const int *__restrict__ long_list, const int *__restrict__ chunk_row,
                            const int *__restrict__ eoff, const unsigned long long *long_ctr, const int2 *stage0,
                            const int2 *stage1, const int *__restrict__ chunk_cnt, const int *__restrict__ cxadj,
                            int *__restrict__ cadjncy, int *__restrict__ cadjwgt) {
  __shared__ int s_pre[32];
  const int nchunks = (int)(*long_ctr & 0xffffffffu);
  for (int q = blockIdx.x; q < nchunks; q += gridDim.x) {
    const int idx = chunk_row[q];
    const int c = long_list[2 * idx];
    const int first = long_list[2 * idx + 1];
    const int L = eoff[c + 1] - eoff[c];
    const int2 *src = ((merge_passes(L) & 1) ? stage0 : stage1) + eoff[c] + (long long)(q - first) * kChunk;
    const int cnt = chunk_cnt[q];
    int pre = 0;
    for (int k = first + threadIdx.x; k < q; k += blockDim.x) pre += chunk_cnt[k];
    pre = __reduce_add_sync(0xffffffffu, pre);
    if ((threadIdx.x & 31) == 0) s_pre[threadIdx.x >> 5] = pre;
    __syncthreads();
    pre = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) pre += s_pre[w];
    __syncthreads();
    const long long dst = (long long)cxadj[c] + pre;
    for (int t0 = threadIdx.x; t0 < cnt; t0 += kCopyBatch * blockDim.x) {
      int2 e[kCopyBatch];
#pragma unroll
      for (int u = 0; u < kCopyBatch; ++u) {
        const int t = t0 + u * blockDim.x;
        e[u] = t < cnt ? __ldcs(src + t) : make_int2(0, 0);
      }
#pragma unroll
      for (int u = 0; u < kCopyBatch; ++u) {
        const int t = t0 + u * blockDim.x;
        if (t < cnt) {
          cadjncy[dst + t] = e[u].x;
          cadjwgt[dst + t] = e[u].y;
        }
      }
    }
  }
}

}  // namespace

// Grid of a kernel that loops over at most `items` work items: no more blocks
// than items (at least one), at most `cap`.
static unsigned grid_for(int64_t cap, int64_t items) { return (unsigned)std::max<int64_t>(1, std::min(cap, items)); }

namespace {
// Tiny units of a graph of n vertices and m entries: at most (n + m) / D + 1.
int64_t units_max(int64_t n, int64_t m) { return (n + m) / kTinyDiag + 2; }
int64_t class_list_size(int64_t m) { return class_offset(m, kTinyMax, kRowClasses); }

template <int K>
void class_attrs(cm_ctx *ctx) {
  constexpr int NT = class_threads(K), IT = class_items(K);
  cudaFuncSetAttribute(k_class_rows<NT, IT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SegSmem<NT, IT>));
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_class_rows<NT, IT>, NT, sizeof(SegSmem<NT, IT>));
  ctx->class_blocks_per_sm[K] = std::max(1, b);
  if constexpr (K + 1 < kClasses) class_attrs<K + 1>(ctx);
}

// Launches the class kernels of the classes a row of at most row_bound
// entries can fall in, round-robin on the auxiliary streams.
template <int K>
void launch_classes(cm_ctx *ctx, const cm_graph *fine, const int *cmap, const int *eoff, const int4 *row_meta,
                    const int *class_list, const int *class_ctr, const int *d_sizes, int2 *stage, int *ucount,
                    int64_t row_bound) {
  constexpr int NT = class_threads(K), IT = class_items(K);
  const int64_t m = fine->nedges;
  if (row_bound > class_lo(kTinyMax, K)) {
    const unsigned grid = grid_for((int64_t)ctx->num_sms * ctx->class_blocks_per_sm[K], class_cap(m, kTinyMax, K));
    k_class_rows<NT, IT><<<grid, NT, sizeof(SegSmem<NT, IT>), ctx->aux[K % cm_ctx::kAux]>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, row_meta, class_list + class_offset(m, kTinyMax, K), class_ctr + K,
        d_sizes, stage, ucount);
    ctx->launches++;
  }
  if constexpr (K + 1 < kClasses)
    launch_classes<K + 1>(ctx, fine, cmap, eoff, row_meta, class_list, class_ctr, d_sizes, stage, ucount, row_bound);
}
}  // namespace

size_t contract_ws_bytes(int64_t n, int64_t m) {
  const int64_t nunits = units_max(n, m);
  const int64_t nchunks = m / kChunk + 2;
  size_t b = 0;
  b += (size_t)n * 4 * 3 + 4 * 256;                    // leader, ucount, eoff(+1)
  b += (size_t)(nunits + 2) * 4 + 256;                 // first row of every tiny unit
  b += (size_t)(m / kChunk + 2) * 8 + 256;             // long_list
  b += (size_t)class_list_size(m) * 4 + 256;           // class lists
  b += (size_t)nchunks * 4 * 3 + 768;                  // chunk_row, chunk_cnt, chunk_np
  b += 256;                                            // counters
  b += (size_t)(n / kMapTile + 3) * 8 + 256;           // unit-map look-back
  b += (size_t)(n / (kScanThreads * kScanItems) + 3) * 8 + 256;  // count-scan look-back
  b += (size_t)n * 16 + 256;                           // row metadata
  b += (size_t)m * 8 * 2 + 512;                        // stages
  b += cmap_ws_bytes(n);
  return b + 4096;
}

int launch_contract(cm_ctx *ctx, const cm_graph *fine, const int32_t *match, int32_t *cmap, cm_graph *coarse,
                    int32_t *d_sizes, cudaStream_t s, int64_t row_bound) {
  const int64_t n = fine->nvtxs, m = fine->nedges;
  if (n == 0) {
    cudaMemsetAsync(d_sizes, 0, 2 * sizeof(int32_t), s);
    cudaMemsetAsync(coarse->xadj, 0, sizeof(int32_t), s);
    return cuda_status(cudaGetLastError(), "contract(empty)");
  }
  if (!ctx->contract_attrs_set) {  // once per context (the attributes last for the process)
    cudaFuncSetAttribute(k_tiny_units<unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(TinySmem<unsigned>));
    cudaFuncSetAttribute(k_tiny_units<unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(TinySmem<unsigned long long>));
    cudaFuncSetAttribute(k_long_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(SegSmem<kChunkThreads, kChunkItems>));
    cudaFuncSetAttribute(k_long_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MergeSmem));
    class_attrs<0>(ctx);
    int b32 = 0, b64 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b32, k_tiny_units<unsigned>, 32, sizeof(TinySmem<unsigned>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b64, k_tiny_units<unsigned long long>, 32,
                                                  sizeof(TinySmem<unsigned long long>));
    ctx->unit_blocks_per_sm[0] = std::max(1, b32);
    ctx->unit_blocks_per_sm[1] = std::max(1, b64);
    if (int rc2 = check_launch(ctx, "contract: kernel attributes")) return rc2;
    ctx->contract_attrs_set = true;
  }
  const int64_t nunits = units_max(n, m);
  const int64_t nchunks_max = m / kChunk + 2;
  const int64_t map_tiles = (n + kMapTile - 1) / kMapTile;
  const int64_t scan_tiles = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  int *leader = (int *)ws_take(ctx, (size_t)n * 4);
  int *ucount = (int *)ws_take(ctx, (size_t)n * 4);
  int *eoff = (int *)ws_take(ctx, (size_t)(n + 1) * 4);
  int *first_row = (int *)ws_take(ctx, (size_t)(nunits + 2) * 4);
  int *long_list = (int *)ws_take(ctx, (size_t)(m / kChunk + 2) * 8);
  int *class_list = (int *)ws_take(ctx, (size_t)class_list_size(m) * 4);
  int *chunk_row = (int *)ws_take(ctx, (size_t)nchunks_max * 4);
  int *chunk_cnt = (int *)ws_take(ctx, (size_t)nchunks_max * 4);
  int *chunk_np = (int *)ws_take(ctx, (size_t)nchunks_max * 4);
  int4 *row_meta = (int4 *)ws_take(ctx, (size_t)n * 16);
  // [0] chunked rows (rows << 32 | chunks); ints 2 .. 2 + kRowClasses - 1 the
  // class counters; int 2 + kRowClasses the last tiny unit's index
  static_assert(2 + kRowClasses + 1 <= 32, "contraction counter block");
  unsigned long long *ctr = (unsigned long long *)ws_take(ctx, 128);
  unsigned long long *map_lb = (unsigned long long *)ws_take(ctx, (size_t)(map_tiles + 3) * 8);
  unsigned long long *scan_lb = (unsigned long long *)ws_take(ctx, (size_t)(scan_tiles + 3) * 8);
  int2 *stage0 = (int2 *)ws_take(ctx, (size_t)m * 8 + 8);
  int2 *stage1 = (int2 *)ws_take(ctx, (size_t)m * 8 + 8);
  if (!leader || !ucount || !eoff || !first_row || !long_list || !class_list || !chunk_row || !chunk_cnt ||
      !chunk_np || !row_meta || !ctr || !map_lb || !scan_lb || !stage0 || !stage1)
    return cm_fail(CM_ERR_NOMEM, "contract: workspace too small");
  int *class_ctr = reinterpret_cast<int *>(ctr) + 2;
  int *unit_last = reinterpret_cast<int *>(ctr) + 2 + kRowClasses;
  DevStatus *st = ctx->d_status;
  cudaMemsetAsync(ctr, 0, 128, s);
  cudaMemsetAsync(&st->max_row, 0, sizeof(int), s);
  cudaMemsetAsync(map_lb, 0, (size_t)(map_tiles + 3) * 8, s);
  cudaMemsetAsync(scan_lb, 0, (size_t)(scan_tiles + 3) * 8, s);
  int rc = launch_cmap(ctx, (int32_t)n, fine->xadj, fine->vwgt, match, cmap, leader, coarse->vwgt, eoff,
                       d_sizes /* n' lands in d_sizes[0] */, long_list, kTinyMax, kChunk, ctr, chunk_row, class_list,
                       class_ctr, m, row_meta, s);
  if (rc) return rc;
  const int sms = ctx->num_sms;
  const bool small_ids = n <= (1ll << (32 - kTinyRowBits));

  // Rows above kTinyMax on the auxiliary streams (one kernel per size class;
  // the chunked rows' sort, merge passes and dedup on the last stream), the
  // tiny units on the caller's stream; every row's unique entries land in
  // stage1 at eoff[c] (the chunked rows in the stage their merge parity
  // picks) and their number in ucount[c].  Classes above row_bound (an upper
  // bound of the expanded row length known to the caller) cannot have rows
  // and are not launched.
  const bool any_big = row_bound > kTinyMax;
  const bool chunked = row_bound > kChunk;
  stage_begin(ctx, s);
  if (any_big) {
    cudaEventRecord(ctx->fork_ev, s);
    for (int i = 0; i < cm_ctx::kAux; ++i) cudaStreamWaitEvent(ctx->aux[i], ctx->fork_ev, 0);
    launch_classes<0>(ctx, fine, cmap, eoff, row_meta, class_list, class_ctr, d_sizes, stage1, ucount, row_bound);
    if (chunked) {
      cudaStream_t cs = ctx->aux[cm_ctx::kAux - 1];
      // Grids of the chunked-row kernels scale with the most chunks the graph
      // can have (m / kChunk), so small graphs do not claim every SM.
      const int long_grid = (int)std::min<int64_t>(sms, m / kChunk / 4 + 1);
      k_long_sort<<<long_grid, kChunkThreads, sizeof(SegSmem<kChunkThreads, kChunkItems>), cs>>>(
          fine->adjncy, fine->adjwgt, cmap, eoff, row_meta, long_list, chunk_row, ctr, d_sizes, stage0, ucount,
          chunk_np);
      ctx->launches++;
      // Passes a row of at most min(m, row_bound) entries can need; each is a
      // plain launch.
      int max_pass = 0;
      for (int64_t w = kChunk; w < std::min<int64_t>(m, row_bound); w <<= 1) ++max_pass;
      const int merge_grid = (int)std::min<int64_t>((int64_t)sms * kMergeBlocksPerSm, m / kMergeOut + 1);
      for (int p = 0; p < max_pass; ++p) {
        k_long_merge<<<merge_grid, kMergeThreads, sizeof(MergeSmem), cs>>>(p, long_list, chunk_row, eoff, ctr,
                                                                          chunk_np, stage0, stage1, st);
        ctx->launches++;
      }
      k_long_dedup<<<long_grid * 4, kDedupThreads, 0, cs>>>(long_list, chunk_row, eoff, ctr, stage0, stage1, stage0,
                                                            stage1, chunk_cnt, ucount);
      ctx->launches++;
    }
  }
  k_unit_map<<<(unsigned)std::max<int64_t>(1, map_tiles), kMapThreads, 0, s>>>(d_sizes, eoff, first_row, unit_last,
                                                                                map_lb, st);
  ctx->launches++;
  const unsigned tiny_grid = grid_for((int64_t)sms * ctx->unit_blocks_per_sm[small_ids ? 0 : 1], nunits);
  if (small_ids)
    k_tiny_units<unsigned><<<tiny_grid, 32, sizeof(TinySmem<unsigned>), s>>>(
        fine->adjncy, fine->adjwgt, cmap, d_sizes, first_row, unit_last, row_meta, eoff, stage1, ucount, st);
  else
    k_tiny_units<unsigned long long><<<tiny_grid, 32, sizeof(TinySmem<unsigned long long>), s>>>(
        fine->adjncy, fine->adjwgt, cmap, d_sizes, first_row, unit_last, row_meta, eoff, stage1, ucount, st);
  ctx->launches++;
  if (any_big)
    for (int i = 0; i < cm_ctx::kAux; ++i) {
      cudaEventRecord(ctx->join_ev[i], ctx->aux[i]);
      cudaStreamWaitEvent(s, ctx->join_ev[i], 0);
    }
  stage_end(ctx, CM_STAGE_ROWS, s);

  // cxadj = exclusive scan of ucount; d_sizes[1] = m'.
  stage_begin(ctx, s);
  k_count_scan<<<(unsigned)std::max<int64_t>(1, scan_tiles), kScanThreads, 0, s>>>(ucount, d_sizes, coarse->xadj,
                                                                                     d_sizes, scan_lb, st);
  ctx->launches++;
  stage_end(ctx, CM_STAGE_SCAN, s);

  // Every row's unique entries to their final place.
  stage_begin(ctx, s);
  const bool big_copy = row_bound > kCopySplit;
  if (big_copy) {
    cudaEventRecord(ctx->fork_ev, s);
    cudaStreamWaitEvent(ctx->aux[0], ctx->fork_ev, 0);
    k_copy_class_rows<<<grid_for(sms * 8, m / kCopySplit + 1), 256, 0, ctx->aux[0]>>>(
        class_list, class_ctr, (long long)m, eoff, ucount, coarse->xadj, stage1, coarse->adjncy, coarse->adjwgt);
    ctx->launches++;
    if (chunked) {
      k_long_copy<<<grid_for(sms * 4, m / kChunk + 1), 256, 0, ctx->aux[0]>>>(
          long_list, chunk_row, eoff, ctr, stage0, stage1, chunk_cnt, coarse->xadj, coarse->adjncy, coarse->adjwgt);
      ctx->launches++;
    }
    cudaEventRecord(ctx->join_ev[0], ctx->aux[0]);
  }
  k_copy_rows<<<grid_for((int64_t)sms * 8, n / kCopyThreads + 1), kCopyThreads, 0, s>>>(
      d_sizes, eoff, ucount, coarse->xadj, stage1, coarse->adjncy, coarse->adjwgt);
  ctx->launches++;
  if (big_copy) cudaStreamWaitEvent(s, ctx->join_ev[0], 0);
  stage_end(ctx, CM_STAGE_COPY, s);
  return check_launch(ctx, "contract");
}

}  // namespace cm
