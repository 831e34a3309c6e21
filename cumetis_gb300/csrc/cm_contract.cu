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
// Work split by expanded coarse-row length L = deg(leader) + deg(follower):
//   L <= kLongThr : contraction tiles.  Tile k owns the rows whose diagonal
//                   c + eoff[c] lies in [kD, (k+1)D) (D = kTileDiag), so a tile
//                   holds <= D rows and < D + kLongThr entries.  One pass per
//                   tile: gather, merge duplicates in a shared-memory hash set,
//                   sort the unique (row, coarse id) keys, and write each row's
//                   unique entries to a stage at its expanded offset eoff[c].
//   L >  kLongThr : long rows, beside the tiles on auxiliary streams.  Rows up
//                   to kChunk entries: one block merges and sorts a row (three
//                   size classes).  Longer rows: chunks of kChunk entries are
//                   sorted in shared memory into a global stage, merged pairwise
//                   (merge path, one launch per pass) and deduplicated.
// A scan of the rows' unique counts gives cxadj; two copy kernels then move
// every row from the stage to its final place.
#include <algorithm>

#include "cm_ctx.h"
#include "cm_sort.cuh"

namespace cm {
namespace {

#ifndef CM_TILE_THREADS
#define CM_TILE_THREADS 256
#endif
constexpr int kTileThreads = CM_TILE_THREADS;     // threads per contraction tile
#ifndef CM_TILE_E
#define CM_TILE_E 4
#endif
constexpr int kTileE = CM_TILE_E;                 // keys per lane in the tile sort's register runs
// D, diagonals per tile (a tuning parameter).  A tile holds at most D rows,
// so its row index needs kTileRowBits bits.
#ifndef CM_TILE_DIAG
#define CM_TILE_DIAG 512
#endif
constexpr int kTileDiag = CM_TILE_DIAG;
// Rows longer than kLongThr take the long path; rows longer than kChunk are
// sorted in kChunk-entry chunks and merged.  Both are tuning parameters (the
// autotuner's choice lands here through the build).
#ifndef CM_LONG_THR
#define CM_LONG_THR 1024
#endif
#ifndef CM_CHUNK
#define CM_CHUNK 8192
#endif
constexpr int kLongThr = CM_LONG_THR;
constexpr int kTileCap = kTileDiag + kLongThr;    // a tile holds fewer entries than this
constexpr int kChunk = CM_CHUNK;                  // long-row chunk (entries sorted per block)
constexpr int kChunkThreads = 1024;
static_assert(kLongThr == 512 || kLongThr == 1024 || kLongThr == 2048, "CM_LONG_THR: 512, 1024 or 2048");
static_assert(kChunk == 4096 || kChunk == 8192, "CM_CHUNK: 4096 or 8192 (one block's shared memory)");
static_assert(4 * kLongThr <= kChunk, "the size classes 2x and 4x CM_LONG_THR must fit a chunk");
// Threads per block of the three size classes of rows between kLongThr and
// kChunk entries ((T, 2T], (2T, 4T], (4T, kChunk] for T = kLongThr; with the
// defaults 1025-2048, 2049-4096, 4097-8192).
#ifndef CM_MID_THREADS0
#define CM_MID_THREADS0 256
#endif
#ifndef CM_MID_THREADS1
#define CM_MID_THREADS1 512
#endif
constexpr int kMidThreads0 = CM_MID_THREADS0, kMidThreads1 = CM_MID_THREADS1;

// Composite key (tile-local row, coarse id).  32-bit when the coarse ids fit
// the bits the row index leaves (kTileIdBits), else 64-bit.  All-ones is the
// empty hash slot and the sort pad; no key reaches it: with D < 2^rowbits the
// row field never reaches all-ones, with D = 2^rowbits the id field must not
// (n < 2^idbits).
__host__ __device__ constexpr int ilog2(int v) { return v <= 1 ? 0 : 1 + ilog2(v >> 1); }
constexpr int kTileRowBits = ilog2(kTileDiag - 1) + 1;  // rows 0 .. D-1
constexpr int kTileIdBits = 32 - kTileRowBits;
constexpr long long kSmallIdMaxN =                       // largest n with 32-bit keys
    kTileDiag < (1 << kTileRowBits) ? (1ll << kTileIdBits) : (1ll << kTileIdBits) - 1;
static_assert(kTileDiag >= 256 && kTileDiag <= 1024, "CM_TILE_DIAG: 256 .. 1024");
template <typename K> struct KeyT;
template <> struct KeyT<unsigned> {
  static constexpr int kShift = kTileIdBits;
  static constexpr unsigned kIdMask = (1u << kTileIdBits) - 1;
  static __device__ __forceinline__ unsigned make(int r, unsigned id) { return ((unsigned)r << kShift) | id; }
  static __device__ __forceinline__ int row(unsigned k) { return (int)(k >> kShift); }
  static __device__ __forceinline__ unsigned id(unsigned k) { return k & kIdMask; }
};
template <> struct KeyT<unsigned long long> {
  static __device__ __forceinline__ unsigned long long make(int r, unsigned id) {
    return ((unsigned long long)r << 32) | id;
  }
  static __device__ __forceinline__ int row(unsigned long long k) { return (int)(k >> 32); }
  static __device__ __forceinline__ unsigned id(unsigned long long k) { return (unsigned)k; }
};

__device__ __forceinline__ int upper_bound_smem(const int *a, int n, int x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Gathers entry o (0 <= o < L) of the expanded row: the leader's entries first
// (as find_cnvtxsedge_original places them, cuMetis.cu:1014-1020).
__device__ __forceinline__ int expanded_src(int o, int xl, int dl, int xf) { return o < dl ? xl + o : xf + (o - dl); }

// ---------------------------------------------------------------------------
// Shared-memory hash set with weight sums (one per tile or per row).  Keys are
// inserted with atomicCAS into open-addressed slots (linear probing, Fibonacci
// hashing); the weight of every copy of a key is added to its slot.  A slot,
// once set, never changes, so a plain read that finds the key is final.
// ---------------------------------------------------------------------------
template <typename K>
__device__ __forceinline__ unsigned hash_home(K key, int shift) {
  return (unsigned)(((unsigned long long)key * 0x9E3779B97F4A7C15ull) >> shift);
}

template <typename K>
__device__ __forceinline__ void hash_add(K *hk, int *hw, unsigned hmask, int shift, K key, int w) {
  const K empty = ~(K)0;
  unsigned h = hash_home(key, shift);
  for (unsigned p = 0; p <= hmask; ++p) {
    K old = hk[h];
    if (old == empty) old = atomicCAS(&hk[h], empty, key);
    if (old == empty || old == key) {
      atomicAdd(&hw[h], w);
      return;
    }
    h = (h + 1) & hmask;
  }
}

// Weight sum of a key known to be in the set.
template <typename K>
__device__ __forceinline__ int hash_get(const K *hk, const int *hw, unsigned hmask, int shift, K key) {
  unsigned h = hash_home(key, shift);
  for (unsigned p = 0; p <= hmask; ++p) {
    if (hk[h] == key) return hw[h];
    h = (h + 1) & hmask;
  }
  return 0;
}

// Table size for n keys: the power of two >= kHashSlack2 * n / 2 (load at
// most 2 / kHashSlack2; at least 64 slots, at most the cap); returns log2.
#ifndef CM_HASH_SLACK2
#define CM_HASH_SLACK2 4
#endif
constexpr int kHashSlack2 = CM_HASH_SLACK2;
__device__ __forceinline__ int hash_log2(int n, int cap_log2) {
  int lg = 6;
  while (lg < cap_log2 && 2 * (1 << lg) < kHashSlack2 * n) ++lg;
  return lg;
}

// Appends the set's keys to dst (arbitrary order, warp-aggregated); returns
// their number.  All NT threads call it; *ctr is a shared counter set to 0.
template <typename K, int NT>
__device__ __forceinline__ int hash_compact(const K *hk, int hsize, K *dst, int *ctr) {
  const K empty = ~(K)0;
  const int lane = threadIdx.x & 31;
  for (int i0 = threadIdx.x - lane; i0 < hsize; i0 += NT) {
    const int i = i0 + lane;
    const K k = i < hsize ? hk[i] : empty;
    const unsigned m = __ballot_sync(0xffffffffu, k != empty);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(ctr, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (k != empty) dst[padk<K>(base + __popc(m & ((1u << lane) - 1)))] = k;
  }
  __syncthreads();
  const int n = *ctr;
  __syncthreads();
  return n;
}

// ---------------------------------------------------------------------------
// Contraction tiles
// ---------------------------------------------------------------------------
// Table slots: the power of two of at least 4/3 kTileCap (load <= 3/4; 2048
// for the default kTileCap of 1536).
constexpr int kTileHashLog2 = ilog2((4 * kTileCap + 2) / 3 - 1) + 1;
constexpr int kTileHash = 1 << kTileHashLog2;
static_assert(kTileHash > kTileCap, "tile hash must have a free slot for every entry");

struct TileRows {
  int r_xl[kTileDiag], r_dl[kTileDiag], r_xf[kTileDiag], r_start[kTileDiag];
};

template <typename K>
struct TileSmem {
  union {
    TileRows T;                                   // gather
    K keys[2][padded_k<K>(((kTileCap + 32 * kTileE - 1) / (32 * kTileE)) * 32 * kTileE)];  // sort of the unique keys
  } u;
  K hk[kTileHash];
  int hw[kTileHash];
  int r_out[kTileDiag];                           // staging offset eoff[c] of a short row, -1 for a long row
  int ustart[kTileDiag + 1];                      // first sorted unique key of each row
  int scan[kTileThreads / 32 + 1];
  int ctr;
};

// Rows [clo, clo+R) of tile t (rows whose diagonal c + eoff[c] lies in
// [tD, (t+1)D)); loads their metadata and lays the short rows' entries out
// back to back (long rows take no space).  Returns the number of entries.
template <typename K>
__device__ __forceinline__ int tile_rows(TileSmem<K> &S, int tile, int nc, long long dend,
                                         const int *__restrict__ first_row, const int4 *__restrict__ row_meta,
                                         const int *__restrict__ eoff, int &clo, int &R, DevStatus *st) {
  const int tid = threadIdx.x;
  const long long last = dend / kTileDiag;
  clo = tile <= last ? first_row[tile] : nc;
  const int chi = tile + 1 <= last ? first_row[tile + 1] : nc;
  R = chi - clo;
  if (R < 0 || R > kTileDiag) {  // inconsistent tile map: report, touch nothing
    if (tid == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
    R = 0;
  }
  if (R == 0) return 0;  // a tile inside a long row's diagonal span holds no row
  constexpr int kRowsPerThread = (kTileDiag + kTileThreads - 1) / kTileThreads;
  int lens[kRowsPerThread];
  int mysum = 0;
#pragma unroll
  for (int i = 0; i < kRowsPerThread; ++i) {
    const int r = tid * kRowsPerThread + i;
    int len = 0;
    if (r < R) {
      const int4 md = row_meta[clo + r];  // (leader start, leader length, follower start, length)
      S.u.T.r_xl[r] = md.x;
      S.u.T.r_dl[r] = md.y;
      S.u.T.r_xf[r] = md.z;
      const bool lng = md.w > kLongThr;
      S.r_out[r] = lng ? -1 : eoff[clo + r];
      len = lng ? 0 : md.w;
    }
    lens[i] = len;
    mysum += len;
  }
  int ntot;
  int ex = block_exclusive_scan<kTileThreads>(mysum, S.scan, &ntot);
  const bool overflow = ntot > kTileCap;
  if (overflow) {
    if (tid == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
    ntot = 0;
  }
#pragma unroll
  for (int i = 0; i < kRowsPerThread; ++i) {
    const int r = tid * kRowsPerThread + i;
    if (r < R) {
      S.u.T.r_start[r] = overflow ? 0 : ex;
      if (overflow) S.r_out[r] = -1;
    }
    ex += lens[i];
  }
  __syncthreads();
  return ntot;
}

// One pass per tile: gathers the short rows' expanded entries (row, coarse
// id, weight), merges duplicates in a shared-memory hash set (self loops are
// dropped), sorts the unique (row, id) keys, and writes each row's unique
// entries, ascending by id with summed weights, to stage[eoff[c] ...) and
// their number to ucount[c].
template <typename K>
__global__ void __launch_bounds__(kTileThreads)
k_contract_tiles(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
                 const int *__restrict__ eoff, const int *d_cn, const int *__restrict__ first_row,
                 const int4 *__restrict__ row_meta, int2 *__restrict__ stage, int *__restrict__ ucount,
                 DevStatus *st) {
  using KT = KeyT<K>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem<K> &S = *reinterpret_cast<TileSmem<K> *>(smem_raw);
  const int tid = threadIdx.x;
  const int nc = *d_cn;
  const long long dend = (long long)nc + eoff[nc];
  int clo, R;
  if (tid == 0) S.ctr = 0;
  const int ntot = tile_rows(S, blockIdx.x, nc, dend, first_row, row_meta, eoff, clo, R, st);
  if (ntot == 0) {  // no short-row entries (uniform): short rows here are empty
    for (int r = tid; r < R; r += kTileThreads)
      if (S.r_out[r] >= 0) ucount[clo + r] = 0;
    return;
  }
  const int lg = hash_log2(ntot, kTileHashLog2);
  const int hsize = 1 << lg, shift = 64 - lg;
  const unsigned hmask = hsize - 1;
  for (int i = tid; i < hsize; i += kTileThreads) {
    S.hk[i] = ~(K)0;
    S.hw[i] = 0;
  }
  __syncthreads();
  for (int e0 = tid; e0 < ntot; e0 += 4 * kTileThreads) {
    int src[4], rr[4], id[4], w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * kTileThreads;
      rr[u] = 0;
      src[u] = -1;
      if (e < ntot) {
        const int r = upper_bound_smem(S.u.T.r_start, R, e) - 1;
        rr[u] = r;
        src[u] = expanded_src(e - S.u.T.r_start[r], S.u.T.r_xl[r], S.u.T.r_dl[r], S.u.T.r_xf[r]);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      id[u] = src[u] >= 0 ? adjncy[src[u]] : 0;
      w[u] = src[u] >= 0 ? adjwgt[src[u]] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) id[u] = src[u] >= 0 ? cmap[id[u]] : 0;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (src[u] >= 0 && id[u] != clo + rr[u])
        hash_add<K>(S.hk, S.hw, hmask, shift, KT::make(rr[u], (unsigned)id[u]), w[u]);
  }
  __syncthreads();  // gather done: the row table is dead, its space holds the keys
  const int U = hash_compact<K, kTileThreads>(S.hk, hsize, S.u.keys[0], &S.ctr);
  const int b = block_sort_keys<K, kTileThreads, kTileE>(S.u.keys[0], S.u.keys[1], U);
  const K *sk = S.u.keys[b];
  // first sorted key of each row: lower bound of (r, 0)
  for (int r = tid; r <= R; r += kTileThreads) {
    const K key = r < R ? KT::make(r, 0u) : ~(K)0;
    int lo = 0, hi = U;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (sk[padk<K>(mid)] < key) lo = mid + 1;
      else hi = mid;
    }
    S.ustart[r] = r < R ? lo : U;
  }
  __syncthreads();
  for (int r = tid; r < R; r += kTileThreads)
    if (S.r_out[r] >= 0) ucount[clo + r] = S.ustart[r + 1] - S.ustart[r];
  for (int i = tid; i < U; i += kTileThreads) {
    const K k = sk[padk<K>(i)];
    const int r = KT::row(k);
    const int w = hash_get<K>(S.hk, S.hw, hmask, shift, k);
    stage[S.r_out[r] + (i - S.ustart[r])] = make_int2((int)KT::id(k), w);
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

// Copies the short rows' unique entries from the stage to their final place
// cxadj[c]: one block per group of kCopyGroup consecutive tiles, one thread
// per entry.
#ifndef CM_COPY_GROUP
#define CM_COPY_GROUP 1
#endif
#ifndef CM_COPY_THREADS
#define CM_COPY_THREADS 128
#endif
constexpr int kCopyThreads = CM_COPY_THREADS, kCopyGroup = CM_COPY_GROUP;
constexpr int kCopyBatch = 4;  // stage loads in flight per thread before their stores
constexpr int kCopyRows = kTileDiag * kCopyGroup;
__global__ void __launch_bounds__(kCopyThreads)
k_copy_tiles(const int *__restrict__ eoff, const int *d_cn, const int *__restrict__ first_row,
             const int *__restrict__ ucount, const int *__restrict__ cxadj, const int2 *__restrict__ stage,
             int *__restrict__ cadjncy, int *__restrict__ cadjwgt) {
  __shared__ int s_pre[kCopyRows + 1], s_src[kCopyRows], s_dst[kCopyRows], s_scan[kCopyThreads / 32 + 1];
  const int tid = threadIdx.x;
  const int nc = *d_cn;
  const long long dend = (long long)nc + eoff[nc];
  const long long last = dend / kTileDiag;
  const long long t0 = (long long)blockIdx.x * kCopyGroup, t1 = t0 + kCopyGroup;
  const int clo = t0 <= last ? first_row[t0] : nc;
  const int chi = t1 <= last ? first_row[t1] : nc;
  const int R = max(0, min(kCopyRows, chi - clo));
  if (R == 0) return;  // tiles inside a long row's diagonal span
  constexpr int kRowsPerThread = (kCopyRows + kCopyThreads - 1) / kCopyThreads;
  int cnt[kRowsPerThread];
  int mysum = 0;
#pragma unroll
  for (int i = 0; i < kRowsPerThread; ++i) {
    const int r = tid * kRowsPerThread + i;
    cnt[i] = 0;
    if (r < R) {
      const int c = clo + r;
      const int e0 = eoff[c];
      if (eoff[c + 1] - e0 <= kLongThr) cnt[i] = ucount[c];
      s_src[r] = e0;
      s_dst[r] = cxadj[c];
    }
    mysum += cnt[i];
  }
  int U;
  int ex = block_exclusive_scan<kCopyThreads>(mysum, s_scan, &U);
#pragma unroll
  for (int i = 0; i < kRowsPerThread; ++i) {
    const int r = tid * kRowsPerThread + i;
    if (r < R) s_pre[r] = ex;
    ex += cnt[i];
  }
  __syncthreads();
  for (int o0 = tid; o0 < U; o0 += kCopyBatch * kCopyThreads) {
    int2 e[kCopyBatch];
    int d[kCopyBatch];
#pragma unroll
    for (int u = 0; u < kCopyBatch; ++u) {
      const int o = o0 + u * kCopyThreads;
      d[u] = -1;
      e[u] = make_int2(0, 0);
      if (o < U) {
        const int r = upper_bound_smem(s_pre, R, o) - 1;
        const int k = o - s_pre[r];
        e[u] = __ldcs(stage + s_src[r] + k);
        d[u] = s_dst[r] + k;
      }
    }
#pragma unroll
    for (int u = 0; u < kCopyBatch; ++u)
      if (d[u] >= 0) {
        cadjncy[d[u]] = e[u].x;
        cadjwgt[d[u]] = e[u].y;
      }
  }
}

// ---------------------------------------------------------------------------
// Long rows
// ---------------------------------------------------------------------------
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

// Shared memory of one block that merges and sorts up to CAP entries.
template <int CAP>
struct MidSmem {
  unsigned keys[2][padded_k<unsigned>(CAP + 8)];
  unsigned hk[2 * CAP];
  int hw[2 * CAP];
  int ctr;
};

// Gathers entries [cs, cs + cnt) of coarse row c's expanded row (metadata
// md), merges duplicates in a shared-memory hash set that sums the weights
// (self loops dropped), sorts the unique coarse ids (register runs, then
// merge passes) and writes them with their weights to dst[0 .. U).  Returns U.
// All NT threads call it; cnt <= CAP.
template <int NT, int CAP>
__device__ int unique_sorted_segment(MidSmem<CAP> &S, int c, const int4 &md, int cs, int cnt,
                                     const int *__restrict__ adjncy, const int *__restrict__ adjwgt,
                                     const int *__restrict__ cmap, int2 *__restrict__ dst) {
  constexpr int kLg = ilog2(2 * CAP);
  const int lg = hash_log2(cnt, kLg);
  const int hsize = 1 << lg, shift = 64 - lg;
  const unsigned hmask = hsize - 1;
  if (threadIdx.x == 0) S.ctr = 0;
  for (int t = threadIdx.x; t < hsize; t += NT) {
    S.hk[t] = ~0u;
    S.hw[t] = 0;
  }
  __syncthreads();
  for (int t0 = threadIdx.x; t0 < cnt; t0 += 4 * NT) {
    int src[4], x[4], w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int t = t0 + u * NT;
      src[u] = t < cnt ? expanded_src(cs + t, md.x, md.y, md.z) : -1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      x[u] = src[u] >= 0 ? adjncy[src[u]] : 0;
      w[u] = src[u] >= 0 ? adjwgt[src[u]] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = src[u] >= 0 ? cmap[x[u]] : 0;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (src[u] >= 0 && x[u] != c) hash_add<unsigned>(S.hk, S.hw, hmask, shift, (unsigned)x[u], w[u]);
  }
  __syncthreads();
  const int U = hash_compact<unsigned, NT>(S.hk, hsize, S.keys[0], &S.ctr);
  const int b = block_sort_keys<unsigned, NT, 8>(S.keys[0], S.keys[1], U);
  const unsigned *sk = S.keys[b];
  for (int t = threadIdx.x; t < U; t += NT) {
    const unsigned k = sk[padk<unsigned>(t)];
    dst[t] = make_int2((int)k, hash_get<unsigned>(S.hk, S.hw, hmask, shift, k));
  }
  return U;
}

// Rows too long for a tile but <= kChunk entries, one size class per launch:
// one block per row writes the row's unique entries to stage[eoff[c] ...) and
// their number to ucount[c].
template <int NT, int CAP>
__global__ void __launch_bounds__(NT)
k_mid_rows(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
           const int *__restrict__ eoff, const int4 *__restrict__ row_meta, const int *__restrict__ list,
           const int *__restrict__ count, int2 *__restrict__ stage, int *__restrict__ ucount) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MidSmem<CAP> &S = *reinterpret_cast<MidSmem<CAP> *>(smem_raw);
  const int nrows = *count;
  for (int i = blockIdx.x; i < nrows; i += gridDim.x) {
    const int c = list[i];
    const int4 md = row_meta[c];
    const int U = unique_sorted_segment<NT, CAP>(S, c, md, 0, min(md.w, CAP), adjncy, adjwgt, cmap, stage + eoff[c]);
    if (threadIdx.x == 0) ucount[c] = U;
    __syncthreads();
  }
}

// Rows longer than kChunk: each chunk of kChunk entries becomes one sorted run
// in stage0 for the merge passes -- its unique entries (duplicates within the
// chunk already merged, self loops dropped), then pad entries up to the
// chunk's length, which sort after every coarse id and are skipped by the
// dedup.  chunk_np[q] = the merge passes the chunk's row needs.
__global__ void __launch_bounds__(kChunkThreads, 1)
k_long_sort(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
            const int *__restrict__ eoff, const int4 *__restrict__ row_meta, const int *__restrict__ long_list,
            const int *__restrict__ chunk_row, const unsigned long long *long_ctr, int2 *__restrict__ stage,
            int *__restrict__ ucount, int *__restrict__ chunk_np) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MidSmem<kChunk> &S = *reinterpret_cast<MidSmem<kChunk> *>(smem_raw);
  const int nchunks = (int)(*long_ctr & 0xffffffffu);
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
    const int U = unique_sorted_segment<kChunkThreads, kChunk>(S, c, md, cs, cnt, adjncy, adjwgt, cmap, dst);
    for (int t = U + threadIdx.x; t < cnt; t += kChunkThreads) dst[t] = make_int2((int)kPadId, 0);
    __syncthreads();
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
             const DevStatus *st) {
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

// Copies every long row's unique entries to its final place once cxadj is
// known: first the size-class rows (stage1 at eoff[c]), then the chunks of the
// chunked rows (each at cxadj[c] + the unique entries of the row's earlier
// chunks).
__global__ void k_long_copy(const int *__restrict__ long_list, const int *__restrict__ chunk_row,
                            const int *__restrict__ eoff, const unsigned long long *long_ctr,
                            const int *__restrict__ mid_list, const int *__restrict__ mid_ctr, int mid_cap,
                            const int2 *stage0, const int2 *stage1, const int *__restrict__ chunk_cnt,
                            const int *__restrict__ ucount, const int *__restrict__ cxadj, int *__restrict__ cadjncy,
                            int *__restrict__ cadjwgt) {
  __shared__ int s_pre[32];
  const int n0 = mid_ctr[0], n1 = mid_ctr[1], n2 = mid_ctr[2];
  const int nmid = n0 + n1 + n2;
  const int nchunks = (int)(*long_ctr & 0xffffffffu);
  for (int q = blockIdx.x; q < nmid + nchunks; q += gridDim.x) {
    int cnt;
    long long dst;
    const int2 *src;
    if (q < nmid) {
      const int cls = q < n0 ? 0 : (q < n0 + n1 ? 1 : 2);
      const int i = q - (cls == 0 ? 0 : (cls == 1 ? n0 : n0 + n1));
      const int c = mid_list[(size_t)cls * mid_cap + i];
      src = stage1 + eoff[c];
      cnt = ucount[c];
      dst = cxadj[c];
    } else {
      const int qq = q - nmid;
      const int idx = chunk_row[qq];
      const int c = long_list[2 * idx];
      const int first = long_list[2 * idx + 1];
      const int L = eoff[c + 1] - eoff[c];
      src = ((merge_passes(L) & 1) ? stage0 : stage1) + eoff[c] + (long long)(qq - first) * kChunk;
      cnt = chunk_cnt[qq];
      int pre = 0;
      for (int k = first + threadIdx.x; k < qq; k += blockDim.x) pre += chunk_cnt[k];
      pre = __reduce_add_sync(0xffffffffu, pre);
      if ((threadIdx.x & 31) == 0) s_pre[threadIdx.x >> 5] = pre;
      __syncthreads();
      pre = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) pre += s_pre[w];
      __syncthreads();
      dst = (long long)cxadj[c] + pre;
    }
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

size_t contract_ws_bytes(int64_t n, int64_t m) {
  const int64_t ntiles = (n + m) / kTileDiag + 2;
  const int64_t nchunks = m / kChunk + m / kLongThr + 2;
  size_t b = 0;
  b += (size_t)n * 4 * 3 + 4 * 256;          // leader, ucount, eoff(+1)
  b += (size_t)(ntiles + 2) * 4 + 256;       // first_row
  b += (size_t)(m / kChunk + 2) * 8 + 256;   // long_list
  b += (size_t)(m / (kLongThr + 1) + 2) * 12 + 256;  // size-class lists
  b += (size_t)nchunks * 4 * 3 + 768;        // chunk_row, chunk_cnt, chunk_np
  b += 256;                                  // counters
  b += (size_t)(ntiles + 2) * 8 + 256;       // tile look-back
  b += (size_t)n * 16 + 256;                 // row metadata
  b += (size_t)m * 8 * 2 + 512;              // stages
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
  const int64_t ntiles = (n + m) / kTileDiag + 1;
  const int64_t nchunks_max = m / kChunk + m / kLongThr + 2;
  const int64_t mid_cap = m / (kLongThr + 1) + 2;
  int *leader = (int *)ws_take(ctx, (size_t)n * 4);
  int *ucount = (int *)ws_take(ctx, (size_t)n * 4);
  int *eoff = (int *)ws_take(ctx, (size_t)(n + 1) * 4);
  int *first_row = (int *)ws_take(ctx, (size_t)(ntiles + 2) * 4);
  int *long_list = (int *)ws_take(ctx, (size_t)(m / kChunk + 2) * 8);
  int *chunk_row = (int *)ws_take(ctx, (size_t)nchunks_max * 4);
  int *chunk_cnt = (int *)ws_take(ctx, (size_t)nchunks_max * 4);
  int *chunk_np = (int *)ws_take(ctx, (size_t)nchunks_max * 4);
  int *mid_list = (int *)ws_take(ctx, (size_t)mid_cap * 3 * 4);
  int4 *row_meta = (int4 *)ws_take(ctx, (size_t)n * 16);
  unsigned long long *ctr = (unsigned long long *)ws_take(ctx, 64);   // [0] chunked rows, [1] mid counters
  unsigned long long *lb = (unsigned long long *)ws_take(ctx, (size_t)(ntiles + 2) * 8);
  int2 *stage0 = (int2 *)ws_take(ctx, (size_t)m * 8 + 8);
  int2 *stage1 = (int2 *)ws_take(ctx, (size_t)m * 8 + 8);
  if (!leader || !ucount || !eoff || !first_row || !long_list || !chunk_row || !chunk_cnt || !chunk_np || !mid_list ||
      !row_meta || !ctr || !lb ||
      !stage0 || !stage1)
    return cm_fail(CM_ERR_NOMEM, "contract: workspace too small");
  int *mid_ctr = reinterpret_cast<int *>(ctr + 1);
  DevStatus *st = ctx->d_status;
  cudaMemsetAsync(ctr, 0, 64, s);
  cudaMemsetAsync(&st->max_row, 0, sizeof(int), s);
  cudaMemsetAsync(lb, 0, (size_t)(n / (kScanThreads * kScanItems) + 3) * 8, s);
  int rc = launch_cmap(ctx, (int32_t)n, fine->xadj, fine->vwgt, match, cmap, leader, coarse->vwgt, eoff,
                       d_sizes /* n' lands in d_sizes[0] */, long_list, kLongThr, kChunk, ctr, chunk_row, first_row,
                       kTileDiag, mid_list, mid_ctr, (int32_t)mid_cap, row_meta, s);
  if (rc) return rc;
  const int sms = ctx->num_sms;
  const bool small_ids = n <= kSmallIdMaxN;
  const size_t tile_smem = small_ids ? sizeof(TileSmem<unsigned>) : sizeof(TileSmem<unsigned long long>);
  if (!ctx->contract_attrs_set) {  // once per context (the attributes last for the process)
    cudaFuncSetAttribute(k_contract_tiles<unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(TileSmem<unsigned>));
    cudaFuncSetAttribute(k_contract_tiles<unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(TileSmem<unsigned long long>));
    cudaFuncSetAttribute(k_mid_rows<kMidThreads0, 2 * kLongThr>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(MidSmem<2 * kLongThr>));
    cudaFuncSetAttribute(k_mid_rows<kMidThreads1, 4 * kLongThr>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(MidSmem<4 * kLongThr>));
    cudaFuncSetAttribute(k_mid_rows<1024, kChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(MidSmem<kChunk>));
    cudaFuncSetAttribute(k_long_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MidSmem<kChunk>));
    cudaFuncSetAttribute(k_long_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MergeSmem));
    if (int rc2 = check_launch(ctx, "contract: kernel attributes")) return rc2;
    ctx->contract_attrs_set = true;
  }

  // Long rows on the auxiliary streams (three size classes; the chunked
  // rows' sort, merge passes and dedup after the largest class) while the
  // tiles do the short rows on the caller's stream.  All of them leave their
  // unique entries in stage1 at eoff[c] (the chunked rows in the stage their
  // merge parity picks) and their number in ucount[c].  Classes above
  // row_bound (an upper bound of the expanded row length known to the
  // caller) cannot have rows and are not launched.
  const bool any_long = row_bound > kLongThr;
  const bool class1 = row_bound > 2 * kLongThr, class2 = row_bound > 4 * kLongThr, chunked = row_bound > kChunk;
  stage_begin(ctx, s);
  if (any_long) {
    cudaEventRecord(ctx->fork_ev, s);
    for (int i = 0; i < 3; ++i) cudaStreamWaitEvent(ctx->aux[i], ctx->fork_ev, 0);
    k_mid_rows<kMidThreads0, 2 * kLongThr><<<grid_for(sms * 4, m / (kLongThr + 1)), kMidThreads0,
                                             sizeof(MidSmem<2 * kLongThr>), ctx->aux[0]>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, row_meta, mid_list, mid_ctr + 0, stage1, ucount);
    ctx->launches++;
    if (class1) {
      k_mid_rows<kMidThreads1, 4 * kLongThr><<<grid_for(sms * 2, m / (2 * kLongThr + 1)), kMidThreads1,
                                               sizeof(MidSmem<4 * kLongThr>), ctx->aux[1]>>>(
          fine->adjncy, fine->adjwgt, cmap, eoff, row_meta, mid_list + mid_cap, mid_ctr + 1, stage1, ucount);
      ctx->launches++;
    }
    if (class2) {
      k_mid_rows<1024, kChunk><<<grid_for(sms, m / (4 * kLongThr + 1)), 1024, sizeof(MidSmem<kChunk>), ctx->aux[2]>>>(
          fine->adjncy, fine->adjwgt, cmap, eoff, row_meta, mid_list + 2 * mid_cap, mid_ctr + 2, stage1, ucount);
      ctx->launches++;
    }
    if (chunked) {
      // Grids of the chunked-row kernels scale with the most chunks the graph
      // can have (m / kChunk), so small graphs do not claim every SM.
      const int long_grid = (int)std::min<int64_t>(sms, m / kChunk / 4 + 1);
      k_long_sort<<<long_grid, kChunkThreads, sizeof(MidSmem<kChunk>), ctx->aux[2]>>>(
          fine->adjncy, fine->adjwgt, cmap, eoff, row_meta, long_list, chunk_row, ctr, stage0, ucount, chunk_np);
      ctx->launches++;
      // Passes a row of at most min(m, row_bound) entries can need; each is a
      // plain launch.
      int max_pass = 0;
      for (int64_t w = kChunk; w < std::min<int64_t>(m, row_bound); w <<= 1) ++max_pass;
      const int merge_grid = (int)std::min<int64_t>((int64_t)sms * kMergeBlocksPerSm, m / kMergeOut + 1);
      for (int p = 0; p < max_pass; ++p) {
        k_long_merge<<<merge_grid, kMergeThreads, sizeof(MergeSmem), ctx->aux[2]>>>(p, long_list, chunk_row, eoff, ctr,
                                                                                    chunk_np, stage0, stage1, st);
        ctx->launches++;
      }
      k_long_dedup<<<long_grid * 4, kDedupThreads, 0, ctx->aux[2]>>>(long_list, chunk_row, eoff, ctr, stage0, stage1,
                                                                     stage0, stage1, chunk_cnt, ucount);
      ctx->launches++;
    }
    for (int i = 0; i < 3; ++i) cudaEventRecord(ctx->join_ev[i], ctx->aux[i]);
  }
  // d_sizes[0] holds n' (written by the cmap scan).
  if (small_ids)
    k_contract_tiles<unsigned><<<(unsigned)ntiles, kTileThreads, tile_smem, s>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, d_sizes, first_row, row_meta, stage1, ucount, st);
  else
    k_contract_tiles<unsigned long long><<<(unsigned)ntiles, kTileThreads, tile_smem, s>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, d_sizes, first_row, row_meta, stage1, ucount, st);
  ctx->launches++;
  if (any_long)
    for (int i = 0; i < 3; ++i) cudaStreamWaitEvent(s, ctx->join_ev[i], 0);
  stage_end(ctx, CM_STAGE_TILES, s);

  // cxadj = exclusive scan of ucount; d_sizes[1] = m'.
  stage_begin(ctx, s);
  const int64_t scan_tiles = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  k_count_scan<<<(unsigned)scan_tiles, kScanThreads, 0, s>>>(ucount, d_sizes, coarse->xadj, d_sizes, lb, st);
  ctx->launches++;
  stage_end(ctx, CM_STAGE_SCAN, s);

  // Every row's unique entries to their final place.
  stage_begin(ctx, s);
  if (any_long) {
    cudaEventRecord(ctx->fork_ev, s);
    cudaStreamWaitEvent(ctx->aux[0], ctx->fork_ev, 0);
    k_long_copy<<<grid_for(sms * 4, m / kLongThr), 256, 0, ctx->aux[0]>>>(
        long_list, chunk_row, eoff, ctr, mid_list, mid_ctr, (int)mid_cap, stage0, stage1, chunk_cnt, ucount,
        coarse->xadj, coarse->adjncy, coarse->adjwgt);
    cudaEventRecord(ctx->join_ev[0], ctx->aux[0]);
    ctx->launches++;
  }
  k_copy_tiles<<<(unsigned)((ntiles + kCopyGroup - 1) / kCopyGroup), kCopyThreads, 0, s>>>(
      eoff, d_sizes, first_row, ucount, coarse->xadj, stage1, coarse->adjncy, coarse->adjwgt);
  ctx->launches++;
  if (any_long) cudaStreamWaitEvent(s, ctx->join_ev[0], 0);
  stage_end(ctx, CM_STAGE_COPY, s);
  return check_launch(ctx, "contract");
}

}  // namespace cm
