// Element-wise "map" launcher shared by the LCALS, Apps and Basic kernels.
//
// A functor `f` with `__device__ void operator()(int64_t i) const` is applied
// to i in [0, n).  CTAs own tiles of BS*IT consecutive indices; inside a tile
// the IT items of a thread are BS apart, so every warp access is contiguous.
// Loads in the functors go through the read-only path (__ldg), which lets
// the compiler issue the IT items' loads back to back.
#pragma once

#include "b200_internal.cuh"

namespace b200 {

template <int BS, int IT, typename F>
__global__ void __launch_bounds__(BS) map_kernel(F f, int64_t n) {
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < n;
       t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t i = t0 + u * BS + threadIdx.x;
      if (i < n) f(i);
    }
  }
}

// Launches map_kernel with the tuning's block size and items per thread.
template <typename F>
int launch_map1d(const char* name, const F& f, int64_t n, const b200_tune* tune,
                 cudaStream_t st, int def_block = 256, int def_items = 4) {
  if (n <= 0) return B200_OK;
  Shape s = resolve_1d(tune, n, def_block, def_items, 1);
  if (!valid_block(s.block)) return invalid("%s: bad block size %d", name, s.block);
  B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
    map_kernel<BS, IT, F><<<s.grid, BS, 0, st>>>(f, n)));
  return after_launch(name);
}

template <typename T>
__device__ __forceinline__ T ld(const T* p) { return __ldg(p); }

}  // namespace b200
