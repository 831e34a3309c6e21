// cm_sort.cuh -- block-wide sort of keys in shared memory.
//
// Each warp first sorts a run of 32*E keys in registers with a bitonic
// network (shuffles across lanes), then merge-path passes double the run
// width.  Keys live at padded indices so that lanes reading runs of
// consecutive keys hit distinct banks.
#pragma once

#include <cuda_runtime.h>

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
