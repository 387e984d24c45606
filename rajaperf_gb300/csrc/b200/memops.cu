// MEMCPY (y[i] = x[i]) and MEMSET (x[i] = val) of the Algorithm group.
//
// MEMCPY is Stream COPY's kernel (16-byte vectors, all loads of a tile before
// its stores).  MEMSET stores 16-byte vectors of the value, block x items
// vectors per CTA tile; a pointer that is not 16-byte aligned takes 8-byte
// stores.
#include "b200_internal.cuh"

using namespace b200;

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 4;

template <int BS, int IT, typename V>
__global__ void __launch_bounds__(BS) memset_kernel(V* __restrict__ x, V v, int64_t units) {
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < units;
       t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      const int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) x[j] = v;
    }
  }
}

}  // namespace

extern "C" {

int b200_algorithm_memcpy(const double* x, double* y, int64_t n, const b200_tune* tune,
                          b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return invalid("b200_algorithm_memcpy: bad args");
  return b200_stream_copy(x, y, n, tune, stream);
}

int b200_algorithm_memset(double* x, double val, int64_t n, const b200_tune* tune,
                          b200_stream_t stream) {
  if (n < 0 || (n > 0 && !x)) return invalid("b200_algorithm_memset: bad args");
  if (n == 0) return B200_OK;
  cudaStream_t st = as_stream(stream);
  const bool vec = aligned16(x) && !(tune && tune->vec == 1) && n >= 2;
  int launches = 0;
  if (vec) {
    const int64_t units = n >> 1;
    Shape s = resolve_1d(tune, units, kBlock, kItems, 2);
    if (!valid_block(s.block)) return invalid("b200_algorithm_memset: bad block size");
    B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
      memset_kernel<BS, IT, double2><<<s.grid, BS, 0, st>>>(reinterpret_cast<double2*>(x),
                                                            make_double2(val, val), units)));
    ++launches;
    if (n & 1) {
      memset_kernel<32, 1, double><<<1, 32, 0, st>>>(x + n - 1, val, 1);
      ++launches;
    }
  } else {
    Shape s = resolve_1d(tune, n, kBlock, kItems, 1);
    if (!valid_block(s.block)) return invalid("b200_algorithm_memset: bad block size");
    B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
      memset_kernel<BS, IT, double><<<s.grid, BS, 0, st>>>(x, val, n)));
    ++launches;
  }
  return after_launch("b200_algorithm_memset", launches);
}

}  // extern "C"
