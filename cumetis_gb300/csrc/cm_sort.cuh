// cm_sort.cuh -- shared-memory sorting helpers of the contraction.
//
// block_radix_sort: stable LSD radix sort of (key, value) pairs of a block,
// 4-bit digits.  Every thread holds ITEMS consecutive pairs in registers and
// counts its digits in two registers (4 bits per digit), which it writes once
// per pass to private 16-bit counters in shared memory (two digits per word);
// one raking scan over all counters (digit-major, thread-minor) gives every
// pair its place, and the pairs are scattered to a padded scratch buffer and
// reloaded for the next digit.  No atomics, no warp votes, four block
// barriers per digit.
//
// block_unique_sum: merges runs of equal keys of a sorted buffer into
// (key, sum of the values) pairs, in order.
#pragma once

#include <cuda_runtime.h>

#include "cm_device.cuh"

#ifndef CM_SORT_RERANK_NT
#define CM_SORT_RERANK_NT 1024
#endif

namespace cm {

// Padded shared-memory index for keys of type K: one spare word every 32
// (32-bit keys) or 16 (64-bit keys), so that lanes reading runs of E
// consecutive keys hit distinct banks.
template <typename K>
__host__ __device__ __forceinline__ int padk(int i) {
  return sizeof(K) == 4 ? i + (i >> 5) : i + (i >> 4);
}
template <typename K>
__host__ __device__ constexpr int padded_k(int n) {
  return sizeof(K) == 4 ? n + (n >> 5) + 1 : n + (n >> 4) + 1;
}

// A (key, value) pair: 8 bytes for 32-bit keys, 16 for 64-bit keys.
template <typename K> struct SortPair;
template <> struct __align__(8) SortPair<unsigned> {
  unsigned k;
  int v;
};
template <> struct __align__(16) SortPair<unsigned long long> {
  unsigned long long k;
  int v;
  int pad;
};
template <typename K>
__device__ __forceinline__ SortPair<K> make_pair_kv(K k, int v) {
  SortPair<K> p;
  p.k = k;
  p.v = v;
  return p;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Slot of pair i in a padded scratch buffer: one spare slot after every 8
// pairs, so that a thread reading its 8 (or 16) consecutive pairs does not
// share banks with its neighbours.
__host__ __device__ __forceinline__ int rslot(int i) { return i + (i >> 3); }
__host__ __device__ constexpr int rslots(int cap) { return cap + cap / 8 + 1; }

constexpr int kDigitBits = 4;
// Shared scratch of the sort and the unique pass for NT threads.
template <int NT>
struct SortScratch {
  // counter words: word (p, t) at p * (NT + NT/32) + t + t/32 holds thread
  // t's counts of digits p (low half) and p + 8 (high half)
  unsigned ctr[8 * (NT + NT / 32) + 1];
  unsigned wsum[NT / 32];
  int tab[NT];  // per (round, warp) head counts of the unique pass
  int scan[NT / 32 + 1];
};

// Stable ascending sort of the n pairs held at work[rslot(i)], i < n, by the
// low `bits` bits of their keys (the keys' other bits must be zero).  The
// result is left at work[0..n) in plain layout.  n <= NT * ITEMS.  All NT
// threads call it; it ends with a block barrier.
template <typename K, int NT, int ITEMS>
__device__ __forceinline__ void block_radix_sort(SortPair<K> *work, SortScratch<NT> &S, int n, int bits) {
  constexpr int NW = NT / 32, kStride = NT + NT / 32;
  static_assert(ITEMS >= 1 && ITEMS <= 16 && NT % 32 == 0 && NT * ITEMS <= 65535, "block_radix_sort shape");
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  // every thread holds kmax consecutive pairs (pairs past n sort last); the
  // other register slots stay idle, so the work follows n, not the capacity
  const int kmax = (n + NT - 1) / NT;
  unsigned *const cmine = S.ctr + t + (t >> 5);  // word (0, t)
  const int rt = (8 * t) % NT;                    // raking: words (8t / NT, rt .. rt + 7)
  unsigned *const crake = S.ctr + ((8 * t) / NT) * kStride + rt + (rt >> 5);
  SortPair<K> it[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int i = t * kmax + k;
    it[k] = (k < kmax && i < n) ? work[rslot(i)] : make_pair_kv<K>(~(K)0, 0);
  }
  const int passes = bits > 0 ? (bits + kDigitBits - 1) / kDigitBits : 1;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = pass * kDigitBits;
    const bool last = pass == passes - 1;
    // Blocks of CM_SORT_RERANK_NT threads or more (64 registers a thread) recount
    // the ranks in the scatter loop instead of keeping them in registers.
    constexpr bool kRerank = NT >= CM_SORT_RERANK_NT;
    unsigned lr[ITEMS];
    // The thread's digit counts live in two registers, 4 bits per digit
    // (digits 0..7 in clo, 8..15 in chi), and reach the shared counter words
    // once per pass.  A count can reach 16 only when all 16 items of the
    // thread share one digit; that carry leaves a pattern whose fields sum
    // to 0 or 1 instead of 16, and is recognised below.
    unsigned clo = 0u, chi = 0u;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      lr[k] = 0u;
      if (k < kmax) {
        const unsigned d = (unsigned)(it[k].k >> shift) & 15u;
        const unsigned s = (d & 7u) << 2, one = 1u << s;
        const bool up = (d & 8u) != 0u;
        if (!kRerank) lr[k] = ((up ? chi : clo) >> s) & 15u;
        if (up) chi += one; else clo += one;
      }
    }
    bool all16 = false;
    unsigned d0 = 0u;
    if (ITEMS == 16 && kmax == 16) {
      d0 = (unsigned)(it[0].k >> shift) & 15u;
      const unsigned s0 = (d0 & 7u) << 2;
      const unsigned ov = s0 < 28u ? 1u << (s0 + 4u) : 0u;
      const bool up = (d0 & 8u) != 0u;
      all16 = (up ? chi : clo) == ov && (up ? clo : chi) == 0u;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      // word p holds the counts of digits p (low half) and p + 8 (high half)
      const unsigned x = (clo >> (4 * q)) & 0x000f000fu, y = (chi >> (4 * q)) & 0x000f000fu;
      cmine[q * kStride] = __byte_perm(x, y, 0x5410);
      cmine[(q + 4) * kStride] = __byte_perm(x, y, 0x7632);
    }
    if (all16) {
#pragma unroll
      for (int p = 0; p < 8; ++p) cmine[p * kStride] = 0u;
      cmine[(d0 & 7u) * kStride] = 16u << ((d0 & 8u) << 1);
    }
    __syncthreads();
    unsigned cw[8], sum = 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const unsigned x = crake[j];
      cw[j] = sum;
      sum += x;  // both halves at once; no half reaches 2^16
    }
    unsigned inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    unsigned base = inc - sum, total;
    if (NW == 1) {
      total = __shfl_sync(0xffffffffu, inc, 31);
    } else {
      if (lane == 31) S.wsum[warp] = inc;
      __syncthreads();
      const unsigned v = lane < NW ? S.wsum[lane] : 0u;
      unsigned vi = v;
#pragma unroll
      for (int o = 1; o < NW; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, vi, o);
        if (lane >= o) vi += y;
      }
      base += __shfl_sync(0xffffffffu, vi - v, warp);
      total = __shfl_sync(0xffffffffu, vi, NW - 1);
    }
    base += (total & 0xffffu) << 16;  // digits 8..15 follow every digit 0..7
#pragma unroll
    for (int j = 0; j < 8; ++j) crake[j] = base + cw[j];
    __syncthreads();
    if (kRerank) {
      clo = 0u;
      chi = 0u;
    }
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      if (k < kmax) {
        const unsigned d = (unsigned)(it[k].k >> shift) & 15u;
        const unsigned c = cmine[(d & 7u) * kStride];
        unsigned lrk = lr[k];
        if (kRerank) {
          const unsigned s = (d & 7u) << 2, one = 1u << s;
          const bool up = (d & 8u) != 0u;
          lrk = ((up ? chi : clo) >> s) & 15u;
          if (up) chi += one; else clo += one;
        }
        const int pos = (int)(((c >> ((d & 8u) << 1)) & 0xffffu) + lrk);
        if (last) {
          if (pos < n) work[pos] = it[k];
        } else {
          work[rslot(pos)] = it[k];
        }
      }
    }
    __syncthreads();
    if (!last) {
#pragma unroll
      for (int k = 0; k < ITEMS; ++k)
        if (k < kmax) it[k] = work[rslot(t * kmax + k)];
    }
  }
}

// Visits the runs of equal keys of the sorted pairs s[0..n): for each run,
// emit(key, sum of the run's values (wrapping like int atomicAdd), q) with q
// the run's index in key order.  Returns the number of runs.  n <= NT * 32.
// All NT threads call it; it ends with a block barrier.
template <typename K, int NT, int ITEMS, typename F>
__device__ __forceinline__ int block_unique_emit(const SortPair<K> *s, int n, SortScratch<NT> &S, F emit) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rounds = (n + NT - 1) / NT;  // <= ITEMS
  const unsigned below = lanemask_lt();
  unsigned hm[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    hm[r] = 0u;
    if (r < rounds) {
      const int i = r * NT + threadIdx.x;
      const bool head = i < n && (i == 0 || s[i].k != s[i - 1].k);
      hm[r] = __ballot_sync(0xffffffffu, head);
      if (lane == 0) S.tab[r * NW + warp] = __popc(hm[r]);
    }
  }
  __syncthreads();
  const int ncell = rounds * NW;  // <= NT
  int total;
  const int ex = block_exclusive_scan<NT>(threadIdx.x < ncell ? S.tab[threadIdx.x] : 0, S.scan, &total);
  if (threadIdx.x < ncell) S.tab[threadIdx.x] = ex;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    if (r < rounds && (hm[r] >> lane & 1u)) {
      const int i = r * NT + threadIdx.x;
      const K key = s[i].k;
      unsigned sum = (unsigned)s[i].v;
      for (int j = i + 1; j < n && s[j].k == key; ++j) sum += (unsigned)s[j].v;
      emit(key, (int)sum, S.tab[r * NW + warp] + __popc(hm[r] & below));
    }
  }
  __syncthreads();
  return total;
}

}  // namespace cm
