// cm_sort.cuh -- block-wide merge sort of (key, weight) pairs in shared memory.
//
// Each thread first sorts runs of E items in registers with a bitonic
// network, then log2(n/E) rounds of merge-path merges double the run width.
// Runs are clipped to n (n need not be a power of two); the tail is padded to
// a multiple of E with `pad` keys, which sort last.
#pragma once

#include <cuda_runtime.h>

namespace cm {

template <typename K, int E>
__device__ __forceinline__ void reg_bitonic_sort(K (&k)[E], int (&w)[E]) {
#pragma unroll
  for (int size = 2; size <= E; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int l = i ^ stride;
        if (l > i) {
          const bool up = (i & size) == 0;
          if ((k[i] > k[l]) == up) {
            K tk = k[i]; k[i] = k[l]; k[l] = tk;
            int tw = w[i]; w[i] = w[l]; w[l] = tw;
          }
        }
      }
    }
  }
}

// Number of items taken from A when the first `diag` outputs of
// merge(A[0..alen), B[0..blen)) are produced (A wins ties).
template <typename K>
__device__ __forceinline__ int merge_path(const K *A, int alen, const K *B, int blen, int diag) {
  int lo = diag > blen ? diag - blen : 0;
  int hi = diag < alen ? diag : alen;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (A[mid] <= B[diag - 1 - mid]) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Sorts k0/w0[0..n) ascending by key; k1/w1 are scratch of the same size
// (capacity >= n rounded up to E).  Returns 0 if the result is in k0/w0, 1 if
// in k1/w1.  All NT threads of the block must call it.
template <typename K, int NT, int E>
__device__ int block_merge_sort(K *k0, int *w0, K *k1, int *w1, int n, K pad) {
  const int npad = ((n + E - 1) / E) * E;
  for (int i = n + (int)threadIdx.x; i < npad; i += NT) { k0[i] = pad; w0[i] = 0; }
  __syncthreads();
  const int nruns = npad / E;
  for (int q = threadIdx.x; q < nruns; q += NT) {
    K kk[E];
    int ww[E];
#pragma unroll
    for (int i = 0; i < E; ++i) { kk[i] = k0[q * E + i]; ww[i] = w0[q * E + i]; }
    reg_bitonic_sort<K, E>(kk, ww);
#pragma unroll
    for (int i = 0; i < E; ++i) { k0[q * E + i] = kk[i]; w0[q * E + i] = ww[i]; }
  }
  __syncthreads();
  K *sk = k0, *dk = k1;
  int *sw = w0, *dw = w1;
  int cur = 0;
  for (int width = E; width < npad; width <<= 1) {
    for (int q = threadIdx.x; q < nruns; q += NT) {
      const int out = q * E;
      const int ps = (out / (2 * width)) * (2 * width);
      const int alen = min(width, npad - ps);
      const int blen = min(width, npad - ps - alen);
      const K *A = sk + ps;
      const K *B = A + alen;
      const int diag = out - ps;
      int i;
      if (blen == 0) {
        i = diag;
      } else if (A[alen - 1] <= B[0]) {  // runs already in order
        i = diag < alen ? diag : alen;
      } else {
        i = merge_path(A, alen, B, blen, diag);
      }
      int j = diag - i;
#pragma unroll
      for (int t = 0; t < E; ++t) {
        const bool takeA = (j >= blen) || (i < alen && A[i] <= B[j]);
        if (takeA) { dk[out + t] = A[i]; dw[out + t] = sw[ps + i]; ++i; }
        else { dk[out + t] = B[j]; dw[out + t] = sw[ps + alen + j]; ++j; }
      }
    }
    __syncthreads();
    K *tk = sk; sk = dk; dk = tk;
    int *tw = sw; sw = dw; dw = tw;
    cur ^= 1;
  }
  return cur;
}

}  // namespace cm

namespace cm {

// Padded shared-memory index for 64-bit words: one spare word every 16, so
// that a warp whose lanes touch consecutive runs of 4 or 8 words (stride 32 or
// 64 bytes) spreads over all banks instead of colliding 8- or 16-fold.
__host__ __device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_size(int n) { return n + (n >> 4) + 1; }

// Block merge sort of packed 64-bit words (sort key in the high bits, payload
// in the low bits; ties among equal keys may end in any order), stored at
// padded indices pad16(i).  a and b hold padded_size(n rounded up to E)
// words.  Returns 0 if the result is in a, 1 if in b.  All NT threads must
// call it.
template <int NT, int E>
__device__ int block_merge_sort_packed(unsigned long long *a, unsigned long long *b, int n) {
  const int npad = ((n + E - 1) / E) * E;
  for (int i = n + (int)threadIdx.x; i < npad; i += NT) a[pad16(i)] = ~0ull;
  __syncthreads();
  const int nruns = npad / E;
  for (int q = threadIdx.x; q < nruns; q += NT) {
    unsigned long long v[E];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = a[pad16(q * E + i)];
#pragma unroll
    for (int size = 2; size <= E; size <<= 1) {
#pragma unroll
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const int l = i ^ stride;
          if (l > i) {
            const bool up = (i & size) == 0;
            if ((v[i] > v[l]) == up) { unsigned long long t = v[i]; v[i] = v[l]; v[l] = t; }
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < E; ++i) a[pad16(q * E + i)] = v[i];
  }
  __syncthreads();
  unsigned long long *src = a, *dst = b;
  int cur = 0;
  for (int width = E; width < npad; width <<= 1) {
    for (int q = threadIdx.x; q < nruns; q += NT) {
      const int out = q * E;
      const int ps = (out / (2 * width)) * (2 * width);
      const int alen = min(width, npad - ps);
      const int blen = min(width, npad - ps - alen);
      const int bs = ps + alen;  // B starts here
      const int diag = out - ps;
      int i;
      if (blen == 0) {
        i = diag;
      } else if (src[pad16(ps + alen - 1)] <= src[pad16(bs)]) {
        i = diag < alen ? diag : alen;
      } else {
        int lo = diag > blen ? diag - blen : 0;
        int hi = diag < alen ? diag : alen;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (src[pad16(ps + mid)] <= src[pad16(bs + diag - 1 - mid)]) lo = mid + 1;
          else hi = mid;
        }
        i = lo;
      }
      int j = diag - i;
      unsigned long long ka = i < alen ? src[pad16(ps + i)] : ~0ull;
      unsigned long long kb = j < blen ? src[pad16(bs + j)] : ~0ull;
#pragma unroll
      for (int t = 0; t < E; ++t) {
        const bool takeA = (j >= blen) || (i < alen && ka <= kb);
        dst[pad16(out + t)] = takeA ? ka : kb;
        if (takeA) { ++i; ka = i < alen ? src[pad16(ps + i)] : ~0ull; }
        else { ++j; kb = j < blen ? src[pad16(bs + j)] : ~0ull; }
      }
    }
    __syncthreads();
    unsigned long long *t = src; src = dst; dst = t;
    cur ^= 1;
  }
  return cur;
}

}  // namespace cm
