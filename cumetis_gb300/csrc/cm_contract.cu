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
//                   holds <= D rows and < D + kLongThr entries.  Two passes:
//                   the count pass gathers the tile's entries and counts each
//                   row's distinct coarse ids with a shared-memory hash set; a
//                   scan of the counts gives cxadj (the "one more scan"); the
//                   emit pass gathers again, sorts by (row, coarse id) with a
//                   block merge sort, merges duplicates and writes each entry
//                   once to its final place.
//   L >  kLongThr : long rows, beside the count pass on auxiliary streams.
//                   Rows up to kChunk entries: one block sorts and merges a
//                   row (three size classes).  Longer rows: chunks of kChunk
//                   entries are sorted in shared memory into a global stage,
//                   merged pairwise (merge path, all blocks cooperating, one
//                   grid barrier per pass) and deduplicated.  Their unique
//                   entries are copied out beside the emit pass.
#include "cm_ctx.h"
#include "cm_sort.cuh"

namespace cm {
namespace {

constexpr int kTileThreads = 128;
constexpr int kTileE = 4;
constexpr int kTileDiag = 512;                    // D
constexpr int kLongThr = 1024;                    // rows longer than this take the long path
constexpr int kTileCap = kTileDiag + kLongThr;    // max entries in a tile (multiple of kTileE)
constexpr int kHashCap = 4096;                    // count-pass hash slots (power of two >= 2 kTileCap)
constexpr int kChunk = 8192;                      // long-row chunk (entries sorted per block)
constexpr int kChunkThreads = 1024;
constexpr unsigned kSelfKey = 0xffffffffu;        // self loops sort last in their row

// Composite sort key (tile-local row, coarse id).  32-bit when coarse ids fit
// in 23 bits (n < 2^23 - 1; rows need 9 bits for kTileDiag = 512), else 64-bit.  The self-loop id is the largest
// id value, so self loops sort last in their row; the pad sorts after all.
template <typename K> struct KeyT;
template <> struct KeyT<unsigned> {
  static constexpr int kShift = 23;
  static constexpr unsigned kIdMask = (1u << 23) - 1;
  static constexpr unsigned kSelf = kIdMask;
  static constexpr unsigned kPad = 0xffffffffu;
  static __device__ __forceinline__ unsigned make(int r, unsigned id) { return ((unsigned)r << kShift) | id; }
  static __device__ __forceinline__ int row(unsigned k) { return (int)(k >> kShift); }
  static __device__ __forceinline__ unsigned id(unsigned k) { return k & kIdMask; }
};
template <> struct KeyT<unsigned long long> {
  static constexpr unsigned kSelf = 0xffffffffu;
  static constexpr unsigned long long kPad = ~0ull;
  static __device__ __forceinline__ unsigned long long make(int r, unsigned id) {
    return ((unsigned long long)r << 32) | id;
  }
  static __device__ __forceinline__ int row(unsigned long long k) { return (int)(k >> 32); }
  static __device__ __forceinline__ unsigned id(unsigned long long k) { return (unsigned)k; }
};
constexpr int kSmallIdLimit = (1 << 23) - 1;   // n below this uses 32-bit keys
static_assert(kHashCap >= 2 * kTileCap && (kHashCap & (kHashCap - 1)) == 0, "count hash: power of two >= 2 cap");
static_assert(kTileDiag <= 512, "tile rows must fit in 9 bits");

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

// Per-tile row table shared by the count and emit passes.
struct TileRows {
  int r_xl[kTileDiag], r_dl[kTileDiag], r_xf[kTileDiag], r_start[kTileDiag], r_len[kTileDiag];
  int scan[kTileThreads / 32 + 1];
};

// Rows [clo, clo+R) of tile t (rows whose diagonal c + eoff[c] lies in
// [tD, (t+1)D)); loads their metadata and lays the short rows' entries out
// back to back (long rows take no space).  Returns the number of entries.
__device__ __forceinline__ int tile_rows(TileRows &T, int tile, int nc, long long dend, const int *first_row,
                                         const int4 *row_meta, int &clo, int &R, DevStatus *st) {
  const int tid = threadIdx.x;
  const long long last = dend / kTileDiag;
  clo = tile <= last ? first_row[tile] : nc;
  const int chi = tile + 1 <= last ? first_row[tile + 1] : nc;
  R = chi - clo;
  if (R < 0 || R > kTileDiag) {  // inconsistent tile map: report, touch nothing
    if (tid == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
    R = 0;
  }
  constexpr int kRowsPerThread = kTileDiag / kTileThreads;
  int lens[kRowsPerThread];
  int mysum = 0;
#pragma unroll
  for (int i = 0; i < kRowsPerThread; ++i) {
    const int r = tid * kRowsPerThread + i;
    int len = 0;
    if (r < R) {
      const int4 md = row_meta[clo + r];  // (leader start, leader length, follower start, length)
      T.r_xl[r] = md.x;
      T.r_dl[r] = md.y;
      T.r_xf[r] = md.z;
      T.r_len[r] = md.w > kLongThr ? -1 : md.w;
      len = md.w > kLongThr ? 0 : md.w;
    }
    lens[i] = len;
    mysum += len;
  }
  int ntot;
  int ex = block_exclusive_scan<kTileThreads>(mysum, T.scan, &ntot);
  const bool overflow = ntot > kTileCap;
  if (overflow) {
    if (tid == 0) record_error(st, CM_ERR_INVALID, ERR_SITE_BOUNDS);
    ntot = 0;
  }
#pragma unroll
  for (int i = 0; i < kRowsPerThread; ++i) {
    const int r = tid * kRowsPerThread + i;
    if (r < R) T.r_start[r] = overflow ? 0 : ex;
    if (r < R && overflow) T.r_len[r] = 0;
    ex += lens[i];
  }
  __syncthreads();
  return ntot;
}

// Gathers 4 entries per thread per step: row, coarse id (self loops marked)
// and weight of expanded entries e0 + u*kTileThreads; consecutive entries of a
// fine row go to consecutive lanes (coalesced adjncy/adjwgt reads).
__device__ __forceinline__ void tile_gather4(const TileRows &T, int R, int clo, int ntot, int e0,
                                             const int *__restrict__ adjncy, const int *__restrict__ adjwgt,
                                             const int *__restrict__ cmap, int (&rr)[4], int (&id)[4], int (&w)[4],
                                             unsigned selfkey) {
  int src[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int e = e0 + u * kTileThreads;
    rr[u] = 0;
    src[u] = -1;
    if (e < ntot) {
      const int r = upper_bound_smem(T.r_start, R, e) - 1;
      rr[u] = r;
      src[u] = expanded_src(e - T.r_start[r], T.r_xl[r], T.r_dl[r], T.r_xf[r]);
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
    if (src[u] >= 0 && id[u] == clo + rr[u]) id[u] = (int)selfkey;
}

// Pass 1: unique coarse ids per short row, counted with a shared-memory hash
// set of (row, id) keys; writes ucount[c].  No sort, no look-back.
template <typename K>
struct CountSmem {
  TileRows T;
  K tab[kHashCap];
  int cnt[kTileDiag];
};

template <typename K>
__global__ void __launch_bounds__(kTileThreads)
k_tile_count(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
             const int *__restrict__ eoff, const int *d_cn, const int *__restrict__ first_row,
             const int4 *__restrict__ row_meta, int *__restrict__ ucount, DevStatus *st) {
  using KT = KeyT<K>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CountSmem<K> &S = *reinterpret_cast<CountSmem<K> *>(smem_raw);
  const int tid = threadIdx.x;
  const int nc = *d_cn;
  const long long dend = (long long)nc + eoff[nc];
  int clo, R;
  const int ntot = tile_rows(S.T, blockIdx.x, nc, dend, first_row, row_meta, clo, R, st);
  unsigned hsize = 64;
  while (hsize < (unsigned)(2 * ntot)) hsize <<= 1;  // <= kHashCap since ntot <= kTileCap
  const unsigned hmask = hsize - 1;
  for (int i = tid; i < (int)hsize; i += kTileThreads) S.tab[i] = KT::kPad;
  for (int r = tid; r < R; r += kTileThreads) S.cnt[r] = 0;
  __syncthreads();
  for (int e0 = tid; e0 < ntot; e0 += 4 * kTileThreads) {
    int rr[4], id[4], w[4];
    tile_gather4(S.T, R, clo, ntot, e0, adjncy, adjwgt, cmap, rr, id, w, KT::kSelf);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (e0 + u * kTileThreads >= ntot || (unsigned)id[u] == KT::kSelf) continue;
      const K key = KT::make(rr[u], (unsigned)id[u]);
      unsigned h = (unsigned)(((unsigned long long)key * 0x9E3779B97F4A7C15ull) >> 40) & hmask;
      for (unsigned probe = 0; probe < hsize; ++probe) {
        const K old = atomicCAS(&S.tab[h], KT::kPad, key);
        if (old == KT::kPad) { atomicAdd(&S.cnt[rr[u]], 1); break; }
        if (old == key) break;
        h = (h + 1) & hmask;
      }
    }
  }
  __syncthreads();
  for (int r = tid; r < R; r += kTileThreads)
    if (S.T.r_len[r] >= 0) ucount[clo + r] = S.cnt[r];
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

// Pass 2: gathers each tile's entries again, sorts them by (row, coarse id),
// merges duplicates and writes every unique entry to its final place
// cxadj[row] + rank.
template <typename K>
struct EmitSmem;
template <>
struct EmitSmem<unsigned> {  // packed (row:9 | id:23) << 32 | weight, padded layout
  TileRows T;
  int r_out[kTileDiag];
  unsigned long long p[2][padded_size(kTileCap + 8)];
};
template <>
struct EmitSmem<unsigned long long> {  // 64-bit (row, id) keys with separate weights
  TileRows T;
  int r_out[kTileDiag];
  unsigned long long k[2][kTileCap];
  int w[2][kTileCap];
};

template <typename K>
__global__ void __launch_bounds__(kTileThreads)
k_tile_emit(const int *__restrict__ adjncy, const int *__restrict__ adjwgt, const int *__restrict__ cmap,
            const int *__restrict__ eoff, const int *d_cn, const int *__restrict__ first_row,
            const int4 *__restrict__ row_meta, const int *__restrict__ cxadj, int *__restrict__ cadjncy,
            int *__restrict__ cadjwgt, DevStatus *st) {
  using KT = KeyT<K>;
  constexpr bool kPacked = sizeof(K) == 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EmitSmem<K> &S = *reinterpret_cast<EmitSmem<K> *>(smem_raw);
  const int tid = threadIdx.x;
  const int nc = *d_cn;
  const long long dend = (long long)nc + eoff[nc];
  int clo, R;
  const int ntot = tile_rows(S.T, blockIdx.x, nc, dend, first_row, row_meta, clo, R, st);
  for (int r = tid; r < R; r += kTileThreads) S.r_out[r] = cxadj[clo + r];
  for (int e0 = tid; e0 < ntot; e0 += 4 * kTileThreads) {
    int rr[4], id[4], w[4];
    tile_gather4(S.T, R, clo, ntot, e0, adjncy, adjwgt, cmap, rr, id, w, KT::kSelf);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * kTileThreads;
      if (e >= ntot) continue;
      if constexpr (kPacked) {
        S.p[0][pad16(e)] = ((unsigned long long)KT::make(rr[u], (unsigned)id[u]) << 32) | (unsigned)w[u];
      } else {
        S.k[0][e] = KT::make(rr[u], (unsigned)id[u]);
        S.w[0][e] = w[u];
      }
    }
  }
  __syncthreads();
  int b;
  if constexpr (kPacked) b = block_merge_sort_packed<kTileThreads, kTileE>(S.p[0], S.p[1], ntot);
  else b = block_merge_sort<K, kTileThreads, kTileE>(S.k[0], S.w[0], S.k[1], S.w[1], ntot, KT::kPad);
  auto keyat = [&](int i) -> K {
    if constexpr (kPacked) return (K)(S.p[b][pad16(i)] >> 32);
    else return S.k[b][i];
  };
  auto wat = [&](int i) -> int {
    if constexpr (kPacked) return (int)(unsigned)S.p[b][pad16(i)];
    else return S.w[b][i];
  };
  int *hs;
  if constexpr (kPacked) hs = reinterpret_cast<int *>(S.p[b ^ 1]);
  else hs = reinterpret_cast<int *>(S.k[b ^ 1]);
  // heads (first of a run of equal (row, id), not a self loop), one block scan
  // over per-thread contiguous chunks
  const int ipt = (ntot + kTileThreads - 1) / kTileThreads;
  const int i0 = min(ntot, tid * ipt), i1 = min(ntot, i0 + ipt);
  int hcnt = 0;
  for (int i = i0; i < i1; ++i) {
    const K k = keyat(i);
    hcnt += (KT::id(k) != KT::kSelf) && (i == 0 || keyat(i - 1) != k);
  }
  int htot;
  int run = block_exclusive_scan<kTileThreads>(hcnt, S.T.scan, &htot);
  for (int i = i0; i < i1; ++i) {
    const K k = keyat(i);
    hs[i] = run;
    run += (KT::id(k) != KT::kSelf) && (i == 0 || keyat(i - 1) != k);
  }
  if (tid == 0) hs[ntot] = htot;
  __syncthreads();
  for (int i = tid; i < ntot; i += kTileThreads) {
    const int hb = hs[i];
    if (hs[i + 1] == hb) continue;  // not a head
    const K k = keyat(i);
    const int r = KT::row(k);
    unsigned sum = (unsigned)wat(i);
    for (int j = i + 1; j < ntot && keyat(j) == k; ++j) sum += (unsigned)wat(j);
    const long long pos = (long long)S.r_out[r] + (hb - hs[S.T.r_start[r]]);
    cadjncy[pos] = (int)KT::id(k);
    cadjwgt[pos] = (int)sum;
  }
}

// ---------------------------------------------------------------------------
// Long rows
// ---------------------------------------------------------------------------
template <int CAP>
struct RowSmem {
  unsigned long long v[2][padded_size(CAP + 8)];  // packed (coarse id << 32 | weight) at pad16(i); +8 for hs[cnt]
};
using ChunkSmem = RowSmem<kChunk>;

// Passes a row of length L needs before its chunks form one sorted run.
__host__ __device__ __forceinline__ int merge_passes(int L) {
  int p = 0;
  long long w = kChunk;
  while (w < L) { w <<= 1; ++p; }
  return p;
}

// Gathers entries [cs, cs+cnt) of coarse row c's expanded row into shared
// memory and sorts them.  If `whole` (the segment is the entire row), merges
// duplicates and writes the unique entries to dedup_dst and their count to
// *ucount_c; otherwise writes the sorted run to run_dst.
template <int NT, int CAP>
__device__ __forceinline__ void sort_row_segment(RowSmem<CAP> &S, int *scan, int c, int xl, int dl, int xf, int cs,
                                                 int cnt, bool whole, int2 *run_dst, int2 *dedup_dst, int *ucount_c,
                                                 const int *__restrict__ adjncy, const int *__restrict__ adjwgt,
                                                 const int *__restrict__ cmap) {
  for (int t0 = threadIdx.x; t0 < cnt; t0 += 4 * NT) {
    int src[4], x[4], w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int t = t0 + u * NT;
      src[u] = t < cnt ? expanded_src(cs + t, xl, dl, xf) : -1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      x[u] = src[u] >= 0 ? adjncy[src[u]] : 0;
      w[u] = src[u] >= 0 ? adjwgt[src[u]] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = src[u] >= 0 ? cmap[x[u]] : 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int t = t0 + u * NT;
      if (t < cnt) {
        const unsigned key = x[u] == c ? kSelfKey : (unsigned)x[u];
        S.v[0][pad16(t)] = ((unsigned long long)key << 32) | (unsigned)w[u];
      }
    }
  }
  __syncthreads();
  const int b = block_merge_sort_packed<NT, 8>(S.v[0], S.v[1], cnt);
  const unsigned long long *P = S.v[b];
  if (!whole) {
    for (int t = threadIdx.x; t < cnt; t += NT) {
      const unsigned long long e = P[pad16(t)];
      run_dst[t] = make_int2((int)(unsigned)(e >> 32), (int)(unsigned)e);
    }
  } else {
    int *hs = reinterpret_cast<int *>(S.v[b ^ 1]);
    const int ipt = (cnt + NT - 1) / NT;
    const int i0 = min(cnt, (int)threadIdx.x * ipt), i1 = min(cnt, i0 + ipt);
    auto head = [&](int i) {
      const unsigned k = (unsigned)(P[pad16(i)] >> 32);
      return k != kSelfKey && (i == 0 || (unsigned)(P[pad16(i - 1)] >> 32) != k);
    };
    int hc = 0;
    for (int i = i0; i < i1; ++i) hc += head(i);
    int tot;
    int run = block_exclusive_scan<NT>(hc, scan, &tot);
    for (int i = i0; i < i1; ++i) {
      hs[i] = run;
      run += head(i);
    }
    if (threadIdx.x == 0) { hs[cnt] = tot; *ucount_c = tot; }
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += NT) {
      if (hs[i + 1] == hs[i]) continue;
      const unsigned k = (unsigned)(P[pad16(i)] >> 32);
      unsigned sum = (unsigned)P[pad16(i)];
      for (int j = i + 1; j < cnt && (unsigned)(P[pad16(j)] >> 32) == k; ++j) sum += (unsigned)P[pad16(j)];
      dedup_dst[hs[i]] = make_int2((int)k, (int)sum);
    }
  }
  __syncthreads();
}

// Rows too long for a tile but <= kChunk entries, one size class per launch:
// one block sorts and deduplicates one whole row (unique entries to stage1).
template <int NT, int CAP>
__global__ void __launch_bounds__(NT)
k_mid_sort(const int *__restrict__ xadj, const int *__restrict__ adjncy, const int *__restrict__ adjwgt,
           const int *__restrict__ match, const int *__restrict__ cmap, const int *__restrict__ leader,
           const int *__restrict__ eoff, const int4 *__restrict__ row_meta, const int *__restrict__ list,
           const int *__restrict__ count, int2 *__restrict__ stage1, int *__restrict__ ucount) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RowSmem<CAP> &S = *reinterpret_cast<RowSmem<CAP> *>(smem_raw);
  __shared__ int scan[NT / 32 + 1];
  const int nrows = *count;
  for (int i = blockIdx.x; i < nrows; i += gridDim.x) {
    const int c = list[i];
    const int4 md = row_meta[c];
    sort_row_segment<NT, CAP>(S, scan, c, md.x, md.y, md.z, 0, md.w, true, nullptr, stage1 + eoff[c], ucount + c,
                              adjncy, adjwgt, cmap);
  }
}

// Rows longer than kChunk: each kChunk-entry chunk sorted into stage0 as one
// run for the merge passes.
__global__ void __launch_bounds__(kChunkThreads, 1)
k_long_sort(const int *__restrict__ xadj, const int *__restrict__ adjncy, const int *__restrict__ adjwgt,
            const int *__restrict__ match, const int *__restrict__ cmap, const int *__restrict__ leader,
            const int *__restrict__ eoff, const int4 *__restrict__ row_meta, const int *__restrict__ long_list,
            const int *__restrict__ chunk_row, const unsigned long long *long_ctr, int2 *__restrict__ stage) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem &S = *reinterpret_cast<ChunkSmem *>(smem_raw);
  __shared__ int scan[kChunkThreads / 32 + 1];
  const unsigned long long ctr = *long_ctr;
  const int nchunks = (int)(ctr & 0xffffffffu);
  for (int q = blockIdx.x; q < nchunks; q += gridDim.x) {
    const int idx = chunk_row[q];
    const int c = long_list[2 * idx];
    const int4 md = row_meta[c];
    const int j = q - long_list[2 * idx + 1];
    const int cs = j * kChunk;
    const int cnt = min(kChunk, md.w - cs);
    sort_row_segment<kChunkThreads, kChunk>(S, scan, c, md.x, md.y, md.z, cs, cnt, false, stage + eoff[c] + cs,
                                            nullptr, nullptr, adjncy, adjwgt, cmap);
  }
}

__device__ __forceinline__ int merge_path_g(const int2 *A, int alen, const int2 *B, int blen, int diag) {
  int lo = diag > blen ? diag - blen : 0;
  int hi = diag < alen ? diag : alen;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((unsigned)__ldcg(&A[mid].x) <= (unsigned)__ldcg(&B[diag - 1 - mid].x)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// All long rows' merge passes in one cooperative launch: pass p merges run
// pairs of width kChunk << p; blocks take kChunk-sized output blocks, threads
// 16 outputs each (merge path per thread).  Rows already a single run skip.
constexpr int kMergeThreads = 512;
constexpr int kMergePer = kChunk / kMergeThreads;  // 16

__global__ void __launch_bounds__(kMergeThreads)
k_long_merge(const int *__restrict__ long_list, const int *__restrict__ chunk_row, const int *__restrict__ eoff,
             const unsigned long long *long_ctr, int2 *stage0, int2 *stage1, DevStatus *st) {
  const unsigned long long ctr = *long_ctr;
  const int nchunks = (int)(ctr & 0xffffffffu);
  const int npass = merge_passes(st->max_row);
  for (int p = 0; p < npass; ++p) {
    const long long width = (long long)kChunk << p;
    const int2 *src = (p & 1) ? stage1 : stage0;
    int2 *dst = (p & 1) ? stage0 : stage1;
    for (int q = blockIdx.x; q < nchunks; q += gridDim.x) {
      const int idx = chunk_row[q];
      const int c = long_list[2 * idx];
      const int L = eoff[c + 1] - eoff[c];
      if (L <= width) continue;
      // Rows that finished earlier have their data in the other stage; a
      // row is merged in pass p only while it still has more than one run.
      if (merge_passes(L) <= p) continue;
      const int j = q - long_list[2 * idx + 1];
      const long long base = eoff[c];
      const int out0 = j * kChunk + threadIdx.x * kMergePer;
      if (out0 >= L) continue;
      const int ps = (int)((out0 / (2 * width)) * (2 * width));
      const int alen = (int)min(width, (long long)(L - ps));
      const int blen = (int)min(width, (long long)(L - ps - alen));
      const int2 *A = src + base + ps;
      const int2 *B = A + alen;
      const int diag = out0 - ps;
      int i = blen == 0 ? diag : merge_path_g(A, alen, B, blen, diag);
      int jj = diag - i;
      const int nout = min(kMergePer, L - out0);
      int2 a = i < alen ? __ldcg(A + i) : make_int2(0, 0);
      int2 bb = jj < blen ? __ldcg(B + jj) : make_int2(0, 0);
      for (int t = 0; t < nout; ++t) {
        const bool takeA = (jj >= blen) || (i < alen && (unsigned)a.x <= (unsigned)bb.x);
        if (takeA) {
          dst[base + out0 + t] = a;
          ++i;
          if (i < alen) a = __ldcg(A + i);
        } else {
          dst[base + out0 + t] = bb;
          ++jj;
          if (jj < blen) bb = __ldcg(B + jj);
        }
      }
    }
    if (p + 1 < npass && !grid_barrier(st, gridDim.x)) return;
  }
}

// Deduplicates each long row (sorted, in stage[merge_passes(L) & 1]) into the
// other stage, compacted at eoff[c]; ucount[c] = unique entries.
constexpr int kDedupThreads = 512;
__global__ void __launch_bounds__(kDedupThreads)
k_long_dedup(const int *__restrict__ long_list, const int *__restrict__ eoff, const unsigned long long *long_ctr,
             int2 *stage0, int2 *stage1, int *__restrict__ ucount) {
  __shared__ int scan[kDedupThreads / 32 + 1];
  const int nlong = (int)(*long_ctr >> 32);
  for (int idx = blockIdx.x; idx < nlong; idx += gridDim.x) {
    const int c = long_list[2 * idx];
    const int L = eoff[c + 1] - eoff[c];
    if (L <= kChunk) continue;  // (not in this list)
    const int fb = merge_passes(L) & 1;
    const int2 *src = (fb ? stage1 : stage0) + eoff[c];
    int2 *dst = (fb ? stage0 : stage1) + eoff[c];
    int carry = 0;
    for (int b = 0; b < L; b += kDedupThreads) {
      const int i = b + threadIdx.x;
      int h = 0;
      int2 e = make_int2(0, 0);
      if (i < L) {
        e = src[i];
        h = ((unsigned)e.x != kSelfKey) && (i == 0 || src[i - 1].x != e.x);
      }
      int tot;
      const int ex = block_exclusive_scan<kDedupThreads>(h, scan, &tot);
      if (h) {
        unsigned sum = (unsigned)e.y;
        for (int j = i + 1; j < L && src[j].x == e.x; ++j) sum += (unsigned)src[j].y;
        dst[carry + ex] = make_int2(e.x, (int)sum);
      }
      carry += tot;
    }
    if (threadIdx.x == 0) ucount[c] = carry;
  }
}

// Copies every long row's unique entries to its final place once the tiles
// have fixed cxadj: first the size-class rows (stage1), then the chunked rows.
__global__ void k_long_copy(const int *__restrict__ long_list, const int *__restrict__ chunk_row,
                            const int *__restrict__ eoff, const unsigned long long *long_ctr,
                            const int *__restrict__ mid_list, const int *__restrict__ mid_ctr, int mid_cap,
                            const int2 *stage0, const int2 *stage1, const int *__restrict__ ucount,
                            const int *__restrict__ cxadj, int *__restrict__ cadjncy, int *__restrict__ cadjwgt) {
  const int n0 = mid_ctr[0], n1 = mid_ctr[1], n2 = mid_ctr[2];
  const int nmid = n0 + n1 + n2;
  const int nchunks = (int)(*long_ctr & 0xffffffffu);
  for (int q = blockIdx.x; q < nmid + nchunks; q += gridDim.x) {
    int c, lo, hi;
    const int2 *src;
    if (q < nmid) {
      const int cls = q < n0 ? 0 : (q < n0 + n1 ? 1 : 2);
      const int i = q - (cls == 0 ? 0 : (cls == 1 ? n0 : n0 + n1));
      c = mid_list[(size_t)cls * mid_cap + i];
      src = stage1 + eoff[c];
      lo = 0;
      hi = ucount[c];
    } else {
      const int qq = q - nmid;
      const int idx = chunk_row[qq];
      c = long_list[2 * idx];
      const int L = eoff[c + 1] - eoff[c];
      src = ((merge_passes(L) & 1) ? stage0 : stage1) + eoff[c];
      const int j = qq - long_list[2 * idx + 1];
      lo = j * kChunk;
      hi = min(ucount[c], (j + 1) * kChunk);
    }
    const long long dst = cxadj[c];
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      const int2 e = src[t];
      cadjncy[dst + t] = e.x;
      cadjwgt[dst + t] = e.y;
    }
  }
}

}  // namespace

size_t contract_ws_bytes(int64_t n, int64_t m) {
  const int64_t ntiles = (n + m) / kTileDiag + 2;
  const int64_t nchunks = m / kChunk + m / kLongThr + 2;
  size_t b = 0;
  b += (size_t)n * 4 * 3 + 4 * 256;          // leader, ucount, eoff(+1)
  b += (size_t)(ntiles + 2) * 4 + 256;       // first_row
  b += (size_t)(m / kChunk + 2) * 8 + 256;   // long_list
  b += (size_t)(m / (kLongThr + 1) + 2) * 12 + 256;  // size-class lists
  b += (size_t)nchunks * 4 + 256;            // chunk_row
  b += 256;                                  // counters
  b += (size_t)(ntiles + 2) * 8 + 256;       // tile look-back
  b += (size_t)n * 16 + 256;                 // row metadata
  b += (size_t)m * 8 * 2 + 512;              // stages
  b += cmap_ws_bytes(n);
  return b + 4096;
}

int launch_contract(cm_ctx *ctx, const cm_graph *fine, const int32_t *match, int32_t *cmap, cm_graph *coarse,
                    int32_t *d_sizes, cudaStream_t s) {
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
  int *mid_list = (int *)ws_take(ctx, (size_t)mid_cap * 3 * 4);
  int4 *row_meta = (int4 *)ws_take(ctx, (size_t)n * 16);
  unsigned long long *ctr = (unsigned long long *)ws_take(ctx, 64);   // [0] chunked rows, [1] mid counters
  unsigned long long *lb = (unsigned long long *)ws_take(ctx, (size_t)(ntiles + 2) * 8);
  int2 *stage0 = (int2 *)ws_take(ctx, (size_t)m * 8 + 8);
  int2 *stage1 = (int2 *)ws_take(ctx, (size_t)m * 8 + 8);
  if (!leader || !ucount || !eoff || !first_row || !long_list || !chunk_row || !mid_list || !row_meta || !ctr || !lb ||
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
  const bool small_ids = n < kSmallIdLimit;
  const size_t count_smem = small_ids ? sizeof(CountSmem<unsigned>) : sizeof(CountSmem<unsigned long long>);
  const size_t emit_smem = small_ids ? sizeof(EmitSmem<unsigned>) : sizeof(EmitSmem<unsigned long long>);
  if (small_ids) {
    cudaFuncSetAttribute(k_tile_count<unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)count_smem);
    cudaFuncSetAttribute(k_tile_emit<unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)emit_smem);
  } else {
    cudaFuncSetAttribute(k_tile_count<unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)count_smem);
    cudaFuncSetAttribute(k_tile_emit<unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)emit_smem);
  }
  cudaFuncSetAttribute(k_mid_sort<256, 2 * kLongThr>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(RowSmem<2 * kLongThr>));
  cudaFuncSetAttribute(k_mid_sort<512, 4 * kLongThr>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(RowSmem<4 * kLongThr>));
  cudaFuncSetAttribute(k_mid_sort<1024, kChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(RowSmem<kChunk>));
  cudaFuncSetAttribute(k_long_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ChunkSmem));

  // Pass 1.  Long rows on the auxiliary streams (three size classes; the
  // chunked rows' sort, merge passes and dedup after the largest class) while
  // the tiles count the short rows' unique entries on the caller's stream.
  // Both write ucount; the scan waits for all of them.
  stage_begin(ctx, s);
  cudaEventRecord(ctx->fork_ev, s);
  for (int i = 0; i < 3; ++i) cudaStreamWaitEvent(ctx->aux[i], ctx->fork_ev, 0);
  k_mid_sort<256, 2 * kLongThr><<<sms * 4, 256, sizeof(RowSmem<2 * kLongThr>), ctx->aux[0]>>>(
      fine->xadj, fine->adjncy, fine->adjwgt, match, cmap, leader, eoff, row_meta, mid_list, mid_ctr + 0, stage1,
      ucount);
  k_mid_sort<512, 4 * kLongThr><<<sms * 2, 512, sizeof(RowSmem<4 * kLongThr>), ctx->aux[1]>>>(
      fine->xadj, fine->adjncy, fine->adjwgt, match, cmap, leader, eoff, row_meta, mid_list + mid_cap, mid_ctr + 1,
      stage1, ucount);
  k_mid_sort<1024, kChunk><<<sms, 1024, sizeof(RowSmem<kChunk>), ctx->aux[2]>>>(
      fine->xadj, fine->adjncy, fine->adjwgt, match, cmap, leader, eoff, row_meta, mid_list + 2 * mid_cap,
      mid_ctr + 2, stage1, ucount);
  k_long_sort<<<sms, kChunkThreads, sizeof(ChunkSmem), ctx->aux[2]>>>(
      fine->xadj, fine->adjncy, fine->adjwgt, match, cmap, leader, eoff, row_meta, long_list, chunk_row, ctr, stage0);
  ctx->launches += 4;
  {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_long_merge, kMergeThreads, 0);
    int grid = sms * (per_sm > 0 ? per_sm : 1);
    const int *a0 = long_list;
    const int *a1 = chunk_row;
    const int *a2 = eoff;
    const unsigned long long *a3 = ctr;
    int2 *a4 = stage0, *a5 = stage1;
    DevStatus *a6 = st;
    void *args[] = {(void *)&a0, (void *)&a1, (void *)&a2, (void *)&a3, (void *)&a4, (void *)&a5, (void *)&a6};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_long_merge, dim3(grid), dim3(kMergeThreads), args, 0,
                                                ctx->aux[2]);
    if (e != cudaSuccess) return cuda_status(e, "contract: long-row merge launch");
    ctx->launches++;
  }
  k_long_dedup<<<sms * 2, kDedupThreads, 0, ctx->aux[2]>>>(long_list, eoff, ctr, stage0, stage1, ucount);
  ctx->launches++;
  for (int i = 0; i < 3; ++i) cudaEventRecord(ctx->join_ev[i], ctx->aux[i]);
  // d_sizes[0] holds n' (written by the cmap scan).
  if (small_ids)
    k_tile_count<unsigned><<<(unsigned)ntiles, kTileThreads, count_smem, s>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, d_sizes, first_row, row_meta, ucount, st);
  else
    k_tile_count<unsigned long long><<<(unsigned)ntiles, kTileThreads, count_smem, s>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, d_sizes, first_row, row_meta, ucount, st);
  ctx->launches++;
  for (int i = 0; i < 3; ++i) cudaStreamWaitEvent(s, ctx->join_ev[i], 0);
  stage_end(ctx, CM_STAGE_TILE_COUNT, s);

  // cxadj = exclusive scan of ucount; d_sizes[1] = m'.
  stage_begin(ctx, s);
  const int64_t scan_tiles = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  k_count_scan<<<(unsigned)scan_tiles, kScanThreads, 0, s>>>(ucount, d_sizes, coarse->xadj, d_sizes, lb, st);
  ctx->launches++;
  stage_end(ctx, CM_STAGE_SCAN, s);

  // Pass 2.  Tiles sort, merge and write the short rows; the long rows'
  // unique entries are copied out on an auxiliary stream meanwhile.
  stage_begin(ctx, s);
  cudaEventRecord(ctx->fork_ev, s);
  cudaStreamWaitEvent(ctx->aux[0], ctx->fork_ev, 0);
  k_long_copy<<<sms * 4, 256, 0, ctx->aux[0]>>>(long_list, chunk_row, eoff, ctr, mid_list, mid_ctr, (int)mid_cap,
                                                 stage0, stage1, ucount, coarse->xadj, coarse->adjncy, coarse->adjwgt);
  cudaEventRecord(ctx->join_ev[0], ctx->aux[0]);
  if (small_ids)
    k_tile_emit<unsigned><<<(unsigned)ntiles, kTileThreads, emit_smem, s>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, d_sizes, first_row, row_meta, coarse->xadj, coarse->adjncy,
        coarse->adjwgt, st);
  else
    k_tile_emit<unsigned long long><<<(unsigned)ntiles, kTileThreads, emit_smem, s>>>(
        fine->adjncy, fine->adjwgt, cmap, eoff, d_sizes, first_row, row_meta, coarse->xadj, coarse->adjncy,
        coarse->adjwgt, st);
  ctx->launches += 2;
  cudaStreamWaitEvent(s, ctx->join_ev[0], 0);
  stage_end(ctx, CM_STAGE_TILE_EMIT, s);
  return check_launch(ctx, "contract");
}

}  // namespace cm
