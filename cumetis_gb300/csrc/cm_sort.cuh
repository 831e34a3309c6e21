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

// Bitonic sort of the 32*E keys a warp holds, E per lane in blocked order
// (lane l holds elements l*E .. l*E+E-1), ascending.  Exchanges across lanes
// use shuffles; no shared memory, no barriers.
template <typename K, int E>
__device__ __forceinline__ void warp_bitonic_sort(K (&v)[E]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int size = 2; size <= 32 * E; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride >= E) {
        const int ls = stride / E;
        const bool lower = (lane & ls) == 0;
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const bool asc = ((lane * E + j) & size) == 0;
          const K o = __shfl_xor_sync(0xffffffffu, v[j], ls);
          v[j] = (lower == asc) ? min(v[j], o) : max(v[j], o);
        }
      } else {
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int l = j ^ stride;
          if (l > j) {
            const bool asc = ((lane * E + j) & size) == 0;
            const K lo = min(v[j], v[l]), hi = max(v[j], v[l]);
            v[j] = asc ? lo : hi;
            v[l] = asc ? hi : lo;
          }
        }
      }
    }
  }
}

// Sort of keys only (ascending), stored at padk<K>(i).  Runs of 32*E keys are
// sorted by one warp each in registers; merge-path passes then double the run
// width up to n.  The tail up to a multiple of 32*E is filled with all-ones
// keys, which must not occur in the data; a and b hold padded_k<K>(n rounded
// up to 32*E) keys.  Returns 0 if the result is in a, 1 if in b.  All NT
// threads must call it.
template <typename K, int NT, int E>
__device__ int block_sort_keys(K *a, K *b, int n) {
  constexpr int W = 32 * E;
  const K kMax = ~(K)0;
  const int npad = ((n + W - 1) / W) * W;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = warp; q * W < npad; q += NT / 32) {
    K v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const int i = q * W + lane * E + j;
      v[j] = i < n ? a[padk<K>(i)] : kMax;
    }
    warp_bitonic_sort<K, E>(v);
#pragma unroll
    for (int j = 0; j < E; ++j) a[padk<K>(q * W + lane * E + j)] = v[j];
  }
  __syncthreads();
  const int nruns = npad / E;
  K *src = a, *dst = b;
  int cur = 0;
  for (int width = W; width < npad; width <<= 1) {
    for (int q = threadIdx.x; q < nruns; q += NT) {
      const int out = q * E;
      const int ps = (out / (2 * width)) * (2 * width);
      const int alen = min(width, npad - ps);
      const int blen = min(width, npad - ps - alen);
      const int bs = ps + alen;
      const int diag = out - ps;
      int i;
      if (blen == 0) {
        i = diag;
      } else if (src[padk<K>(ps + alen - 1)] <= src[padk<K>(bs)]) {
        i = diag < alen ? diag : alen;
      } else {
        int lo = diag > blen ? diag - blen : 0;
        int hi = diag < alen ? diag : alen;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (src[padk<K>(ps + mid)] <= src[padk<K>(bs + diag - 1 - mid)]) lo = mid + 1;
          else hi = mid;
        }
        i = lo;
      }
      int j = diag - i;
      K ka = i < alen ? src[padk<K>(ps + i)] : kMax;
      K kb = j < blen ? src[padk<K>(bs + j)] : kMax;
#pragma unroll
      for (int t = 0; t < E; ++t) {
        const bool takeA = (j >= blen) || (i < alen && ka <= kb);
        dst[padk<K>(out + t)] = takeA ? ka : kb;
        if (takeA) { ++i; ka = i < alen ? src[padk<K>(ps + i)] : kMax; }
        else { ++j; kb = j < blen ? src[padk<K>(bs + j)] : kMax; }
      }
    }
    __syncthreads();
    K *t = src; src = dst; dst = t;
    cur ^= 1;
  }
  return cur;
}

}  // namespace cm
