// cm_device.cuh -- device helpers shared by the libcm kernels: the per-context
// status block, time-bounded waits, a grid barrier for cooperative launches,
// relaxed/acquire/release global accesses, and a 64-bit warp maximum.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cm_internal.h"

namespace cm {

// Device status block (one per context, in device memory).
struct DevStatus {
  int error;            // first error code recorded by a kernel (0 = none)
  int error_site;       // which wait or check gave up (kernel-specific code)
  int rounds;           // matching rounds of the last cm_match
  int max_row;          // longest expanded coarse row of the last contraction
  unsigned bar_count;   // grid barrier arrival counter
  unsigned bar_gen;     // grid barrier generation
  unsigned tile_ticket; // dynamic tile id counter for look-back scans
  int pad;
};

enum : int {
  ERR_SITE_BARRIER = 1,
  ERR_SITE_LOOKBACK = 2,
  ERR_SITE_ROUNDS = 3,
  ERR_SITE_BOUNDS = 4,
  ERR_SITE_MATCH_INVALID = 5,
};

// Every device-side wait gives up after this many nanoseconds and records
// CM_ERR_LIMIT instead of spinning forever.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void record_error(DevStatus *st, int code, int site) {
  if (atomicCAS(&st->error, 0, code) == 0) atomicExch(&st->error_site, site);
}

__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Grid-wide barrier for kernels launched cooperatively (all blocks resident).
// Returns false (and records CM_ERR_LIMIT) if the wait timed out or another
// block already failed; callers then leave the kernel.
__device__ __forceinline__ bool grid_barrier(DevStatus *st, unsigned nblocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned gen = ld_acquire(&st->bar_gen);
    __threadfence();
    unsigned arrived = atomicAdd(&st->bar_count, 1u);
    if (arrived == nblocks - 1) {
      st->bar_count = 0;
      __threadfence();
      st_release(&st->bar_gen, gen + 1);
    } else {
      uint64_t t0 = global_timer_ns();
      while (ld_acquire(&st->bar_gen) == gen) {
        if (ld_relaxed(&st->error) != 0) { ok = 0; break; }
        if (global_timer_ns() - t0 > kWaitLimitNs) {
          record_error(st, CM_ERR_LIMIT, ERR_SITE_BARRIER);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    if (ld_relaxed(&st->error) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Edge priority hash for the hashed tie-break (lo < hi); equals
// or_edge_hash() of the oracle.
__host__ __device__ __forceinline__ uint32_t edge_hash(uint32_t lo, uint32_t hi) {
  uint64_t x = ((uint64_t)lo << 32) | hi;
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (uint32_t)(x >> 32);
}

// ---------------------------------------------------------------------------
// Decoupled look-back (single-pass tile prefix).  Status words are 64-bit:
// bits 62-63 = flag (0 unpublished, 1 tile aggregate, 2 inclusive prefix),
// bits 0-61 = value.  status[0] is the dynamic tile ticket, tiles start at 1.
// ---------------------------------------------------------------------------
constexpr unsigned long long kLbFlagAgg = 1ull << 62;
constexpr unsigned long long kLbFlagInc = 2ull << 62;
constexpr unsigned long long kLbValMask = (1ull << 62) - 1;

// Publishes tile `tile`'s aggregate (lane 0 of the calling warp).  Tile 0
// publishes its inclusive prefix directly.
__device__ __forceinline__ void lookback_publish(unsigned long long *status, int tile, unsigned long long aggregate) {
  unsigned long long *ts = status + 1;
  if ((threadIdx.x & 31) == 0) st_release64(&ts[tile], (tile == 0 ? kLbFlagInc : kLbFlagAgg) | aggregate);
}

// Called by one full warp after lookback_publish: returns the exclusive
// prefix of all earlier tiles and publishes this tile's inclusive prefix.  On
// a timed-out wait it records CM_ERR_LIMIT and returns 0.
__device__ __forceinline__ unsigned long long lookback_resolve(unsigned long long *status, int tile,
                                                               unsigned long long aggregate, DevStatus *st) {
  const int lane = threadIdx.x & 31;
  unsigned long long *ts = status + 1;
  if (tile == 0) return 0;
  unsigned long long excl = 0;
  int idx = tile - 1;
  const uint64_t t0 = global_timer_ns();
  while (true) {
    const int j = idx - lane;
    unsigned long long s = j >= 0 ? ld_acquire64(&ts[j]) : kLbFlagInc;
    unsigned flag = (unsigned)(s >> 62);
    // Only the predecessors up to the nearest published inclusive prefix are
    // needed; wait while one of those has not published anything yet.
    const unsigned inc_mask = __ballot_sync(0xffffffffu, flag == 2);
    const int last = inc_mask ? (__ffs(inc_mask) - 1) : 31;
    if (__any_sync(0xffffffffu, lane <= last && flag == 0)) {
      if (global_timer_ns() - t0 > kWaitLimitNs) {
        if (lane == 0) record_error(st, CM_ERR_LIMIT, ERR_SITE_LOOKBACK);
        excl = 0;
        break;
      }
      continue;
    }
    unsigned long long v = s & kLbValMask;
    unsigned long long part = lane <= last ? v : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    excl += part;
    if (inc_mask) break;
    idx -= 32;
  }
  if (lane == 0) st_release64(&ts[tile], kLbFlagInc | ((excl + aggregate) & kLbValMask));
  return excl;
}

// Both steps at once, for tiles whose aggregate is ready only at the end.
__device__ __forceinline__ unsigned long long lookback_exclusive(unsigned long long *status, int tile,
                                                                 unsigned long long aggregate, DevStatus *st) {
  lookback_publish(status, tile, aggregate);
  return lookback_resolve(status, tile, aggregate, st);
}

// Inclusive warp scan of 64-bit values.
__device__ __forceinline__ unsigned long long warp_inclusive_scan_u64(unsigned long long v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__device__ __forceinline__ int warp_inclusive_scan_i32(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one int per thread (NT threads, multiple of
// 32).  `sh` needs NT/32 + 1 ints.  Returns the exclusive prefix; *total gets
// the block sum.
template <int NT>
__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = warp_inclusive_scan_i32(v);
  if (lane == 31) sh[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int x = lane < NT / 32 ? sh[lane] : 0;
    int xi = warp_inclusive_scan_i32(x);
    if (lane < NT / 32) sh[lane] = xi - x;
    if (lane == NT / 32 - 1) sh[NT / 32] = xi;
  }
  __syncthreads();
  int r = sh[wid] + inc - v;
  *total = sh[NT / 32];
  __syncthreads();
  return r;
}

}  // namespace cm
