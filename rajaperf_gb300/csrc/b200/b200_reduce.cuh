// Deterministic block reductions and the single-launch "last CTA finishes"
// grid reduction used by DOT, REDUCE_SUM and FIRST_MIN.
//
// Determinism: the grid shape is a pure function of (n, tuning, SM count);
// each thread accumulates its elements in a fixed order; the warp tree uses
// fixed xor-shuffle partners; warps combine in warp order; and the last CTA
// to arrive sums the per-CTA partials in CTA-index order.  Which CTA happens
// to arrive last does not change the arithmetic.
#pragma once

#include "b200_internal.cuh"

namespace b200 {

// Layout of a reduction workspace: [counter (256 B)] [partials...].
struct ReduceWorkspace {
  unsigned int* counter;
  void* partials;
};

inline int reduce_grid(int64_t n, const b200_tune* t, int block, int items) {
  int64_t cap = static_cast<int64_t>(device_info().sm_count) * 8;
  if (t && t->grid_blocks) cap = t->grid_blocks;
  int64_t tiles = ceil_div(n > 0 ? n : 1, static_cast<int64_t>(block) * items);
  if (tiles > cap) tiles = cap;
  return static_cast<int>(tiles < 1 ? 1 : tiles);
}

inline size_t reduce_ws_bytes_for_grid(int grid) {
  return 256 + static_cast<size_t>(grid) * 16;
}

template <int BS>
__device__ __forceinline__ double block_sum(double v, double* smem) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < BS / 32) ? smem[lane] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  }
  __syncthreads();
  return v;  // valid in thread 0
}

// Min-loc with first-index tie-break: smaller value wins; equal values keep
// the smaller index (the sequential loop's strict '<' keeps the first hit).
struct MinLoc {
  double val;
  long long loc;
};

__device__ __forceinline__ MinLoc minloc_pick(MinLoc a, MinLoc b) {
  if (b.val < a.val) return b;
  if (a.val < b.val) return a;
  return (b.loc < a.loc) ? b : a;
}

template <int BS>
__device__ __forceinline__ MinLoc block_minloc(MinLoc v, MinLoc* smem) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    MinLoc o;
    o.val = __shfl_xor_sync(0xffffffffu, v.val, off);
    o.loc = __shfl_xor_sync(0xffffffffu, v.loc, off);
    v = minloc_pick(v, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  if (warp == 0) {
    if (lane < BS / 32) {
      v = smem[lane];
    } else {
      v.val = __longlong_as_double(0x7ff0000000000000LL);  // +inf
      v.loc = 0x7fffffffffffffffLL;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      MinLoc o;
      o.val = __shfl_xor_sync(0xffffffffu, v.val, off);
      o.loc = __shfl_xor_sync(0xffffffffu, v.loc, off);
      v = minloc_pick(v, o);
    }
  }
  __syncthreads();
  return v;
}

// Min-loc over order-preserving integer keys of doubles.  On GB300 a double
// compare issues on the (narrow) FP64 pipe; comparing keys runs on the
// integer pipe.  key(x) orders exactly as '<' on doubles: -0.0 is folded onto
// +0.0 (they compare equal) and NaN maps to the largest key (a NaN never
// compares less, so it is never selected).
__device__ __forceinline__ long long order_key(long long bits) {
  if (bits == static_cast<long long>(0x8000000000000000ULL)) bits = 0;  // -0 -> +0
  const long long mag = bits & 0x7fffffffffffffffLL;
  if (mag > 0x7ff0000000000000LL) return 0x7fffffffffffffffLL;          // NaN
  return bits ^ ((bits >> 63) & 0x7fffffffffffffffLL);
}

struct KeyLoc {
  long long key;
  long long loc;
};

__device__ __forceinline__ KeyLoc keyloc_pick(KeyLoc a, KeyLoc b) {
  if (b.key < a.key) return b;
  if (a.key < b.key) return a;
  return (b.loc < a.loc) ? b : a;
}

template <int BS>
__device__ __forceinline__ KeyLoc block_keyloc(KeyLoc v, KeyLoc* smem) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    KeyLoc o;
    o.key = __shfl_xor_sync(0xffffffffu, v.key, off);
    o.loc = __shfl_xor_sync(0xffffffffu, v.loc, off);
    v = keyloc_pick(v, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  if (warp == 0) {
    if (lane < BS / 32) {
      v = smem[lane];
    } else {
      v.key = 0x7fffffffffffffffLL;
      v.loc = 0x7fffffffffffffffLL;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      KeyLoc o;
      o.key = __shfl_xor_sync(0xffffffffu, v.key, off);
      o.loc = __shfl_xor_sync(0xffffffffu, v.loc, off);
      v = keyloc_pick(v, o);
    }
  }
  __syncthreads();
  return v;
}

// Publishes this CTA's partial and reports whether this CTA arrived last.
// Thread 0 must call it; the result is broadcast through `flag`.
__device__ __forceinline__ bool arrive_last(unsigned int* counter,
                                            bool* flag) {
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int prev = atomicAdd(counter, 1u);
    *flag = (prev == gridDim.x - 1);
  }
  __syncthreads();
  bool last = *flag;
  if (last) __threadfence();
  return last;
}

}  // namespace b200
