// HISTOGRAM (counts[bins[i]] += 1) and MULTI_REDUCE (values[bins[i]] +=
// data[i]): per-bin reductions over a bin index per item.
//
// HISTOGRAM: up to 16 bins (the suite's default is 10), each thread counts in
// packed 8-bit register counters; up to 16384 bins, a CTA counts into a
// shared-memory histogram, lanes of a warp that hit the same bin combined
// first (__match_any_sync: the suite's default bin layout is long runs of
// one bin); the CTA then adds its counts to the global counters with 64-bit
// atomics.  Integer
// sums do not depend on order, so the counts are exact.  The global counters
// start from counts_init (one small copy kernel).
//
// MULTI_REDUCE: deterministic.  Every thread accumulates into its own row of
// bins in shared memory (bin-major, thread-minor: a warp's 32 accesses hit
// 32 banks whatever the bins), visiting its items in index order; the CTA
// sums the 256 rows per bin in a fixed tree and writes one partial per bin;
// the last CTA to finish sums the partials per bin in a fixed tree and adds
// values_init.
// Up to kPrivateBins bins; beyond that the items are added with global FP64
// atomics (order-dependent rounding, within the reassociation bound).
//
// Items whose bin is outside [0, num_bins) are skipped (the suite's loop
// would write out of bounds).
#include "b200_internal.cuh"
#include "b200_reduce.cuh"

using namespace b200;

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 8;
constexpr int64_t kSharedBins = 16384;  // HISTOGRAM: 64 KB of 32-bit counters
constexpr int64_t kPrivateBins = 96;    // MULTI_REDUCE: 256 x 96 x 8 B = 192 KB

int bin_grid(int64_t n) {
  int64_t g = ceil_div(n > 0 ? n : 1, static_cast<int64_t>(kBlock) * kItems);
  const int64_t cap = static_cast<int64_t>(device_info().sm_count) * 4;
  return static_cast<int>(g < cap ? g : cap);
}

__global__ void copy_u64_kernel(const unsigned long long* __restrict__ src,
                                unsigned long long* __restrict__ dst, int64_t m) {
  for (int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; b < m;
       b += static_cast<int64_t>(gridDim.x) * blockDim.x)
    dst[b] = src[b];
}

__global__ void __launch_bounds__(kBlock)
histogram_shared_kernel(const int64_t* __restrict__ bins, int64_t n, int64_t num_bins,
                        unsigned long long* __restrict__ counts) {
  extern __shared__ unsigned int s_cnt[];
  for (int64_t b = threadIdx.x; b < num_bins; b += kBlock) s_cnt[b] = 0u;
  __syncthreads();
  const unsigned int lane = threadIdx.x & 31u;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (kBlock * kItems); t0 < n;
       t0 += static_cast<int64_t>(gridDim.x) * (kBlock * kItems)) {
    int64_t b[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = t0 + u * kBlock + threadIdx.x;
      b[u] = (i < n) ? __ldcs(bins + i) : -1;
    }
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const bool ok = b[u] >= 0 && b[u] < num_bins;
      const unsigned int key = ok ? static_cast<unsigned int>(b[u]) : 0xffffffffu;
      const unsigned int peers = __match_any_sync(0xffffffffu, key);
      if (ok && (__ffs(peers) - 1) == static_cast<int>(lane))
        atomicAdd(&s_cnt[key], static_cast<unsigned int>(__popc(peers)));
    }
  }
  __syncthreads();
  for (int64_t b = threadIdx.x; b < num_bins; b += kBlock)
    if (s_cnt[b]) atomicAdd(&counts[b], static_cast<unsigned long long>(s_cnt[b]));
}

// Up to 16 bins: every thread counts in two 64-bit words of 8-bit counters
// (bin b adds 1 << 8*(b mod 8) to word b / 8: a shift and an add per item),
// unpacked into 32-bit totals before any byte can overflow; warp and CTA
// sums follow, and one 64-bit atomic per bin and CTA.
constexpr int64_t kRegisterBins = 16;

__global__ void __launch_bounds__(kBlock)
histogram_register_kernel(const int64_t* __restrict__ bins, int64_t n, int num_bins,
                          bool vec, unsigned long long* __restrict__ counts) {
  __shared__ unsigned int s_tot[kBlock / 32][kRegisterBins];
  unsigned int acc[kRegisterBins];
#pragma unroll
  for (int k = 0; k < kRegisterBins; ++k) acc[k] = 0u;
  unsigned long long lo = 0ull, hi = 0ull;
  int pending = 0;
  auto flush = [&]() {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      acc[k] += static_cast<unsigned int>((lo >> (8 * k)) & 0xffull);
      acc[8 + k] += static_cast<unsigned int>((hi >> (8 * k)) & 0xffull);
    }
    lo = hi = 0ull;
    pending = 0;
  };
  auto count = [&](int64_t b) {
    const bool ok = b >= 0 && b < num_bins;
    const unsigned long long one = ok ? (1ull << (8 * (b & 7))) : 0ull;
    if (b < 8) lo += one; else hi += one;
  };
  // item pairs with 16-byte loads (bins is 16-byte aligned when `vec`)
  const int64_t units = vec ? (n >> 1) : n;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (kBlock * kItems); t0 < units;
       t0 += static_cast<int64_t>(gridDim.x) * (kBlock * kItems)) {
    longlong2 b[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = t0 + u * kBlock + threadIdx.x;
      if (vec) {
        b[u] = (i < units) ? __ldcs(reinterpret_cast<const longlong2*>(bins) + i)
                           : make_longlong2(-1, -1);
      } else {
        b[u] = make_longlong2((i < units) ? __ldcs(bins + i) : -1, -1);
      }
    }
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      count(b[u].x);
      count(b[u].y);
    }
    pending += 2 * kItems;
    if (pending > 255 - 2 * kItems) flush();
  }
  if (vec && (n & 1) && blockIdx.x == 0 && threadIdx.x == 0) count(__ldcs(bins + n - 1));
  flush();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < kRegisterBins; ++k) {
    unsigned int v = acc[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) s_tot[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < num_bins) {
    unsigned long long t = 0ull;
#pragma unroll
    for (int w = 0; w < kBlock / 32; ++w) t += s_tot[w][threadIdx.x];
    if (t) atomicAdd(&counts[threadIdx.x], t);
  }
}

__global__ void histogram_global_kernel(const int64_t* __restrict__ bins, int64_t n,
                                        int64_t num_bins,
                                        unsigned long long* __restrict__ counts) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t b = __ldcs(bins + i);
    if (b >= 0 && b < num_bins) atomicAdd(&counts[b], 1ull);
  }
}

// s_rows: num_bins x kBlock doubles (bin-major).  partials: gridDim.x x num_bins.
__global__ void __launch_bounds__(kBlock)
multi_reduce_private_kernel(const int64_t* __restrict__ bins, const double* __restrict__ data,
                            int64_t n, int num_bins, const double* __restrict__ values_init,
                            double* __restrict__ values, double* __restrict__ partials,
                            unsigned int* __restrict__ counter) {
  extern __shared__ double s_rows[];
  __shared__ bool last_flag;
  for (int k = threadIdx.x; k < num_bins * kBlock; k += kBlock) s_rows[k] = 0.0;
  __syncthreads();
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (kBlock * kItems); t0 < n;
       t0 += static_cast<int64_t>(gridDim.x) * (kBlock * kItems)) {
    int64_t b[kItems];
    double v[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = t0 + u * kBlock + threadIdx.x;
      b[u] = (i < n) ? __ldcs(bins + i) : -1;
      v[u] = (i < n) ? __ldcs(data + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kItems; ++u)
      if (b[u] >= 0 && b[u] < num_bins) s_rows[b[u] * kBlock + threadIdx.x] += v[u];
  }
  __syncthreads();
  // per bin: lane l sums rows l, l+32, ..., then a fixed warp tree
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int bb = warp; bb < num_bins; bb += kBlock / 32) {
    double s = 0.0;
#pragma unroll
    for (int r = lane; r < kBlock; r += 32) s += s_rows[bb * kBlock + r];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) {
      partials[static_cast<int64_t>(blockIdx.x) * num_bins + bb] = s;
      __threadfence();  // every writer's partial is visible before the arrival
    }
  }
  if (arrive_last(counter, &last_flag)) {
    // per bin: lane l sums the partials of CTAs l, l+32, ..., then a fixed tree
    for (int bb = warp; bb < num_bins; bb += kBlock / 32) {
      double s = 0.0;
      for (int c = lane; c < static_cast<int>(gridDim.x); c += 32)
        s += __ldcg(partials + static_cast<int64_t>(c) * num_bins + bb);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
      if (lane == 0) values[bb] = values_init[bb] + s;
    }
    if (threadIdx.x == 0) *counter = 0u;
  }
}

__global__ void copy_f64_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                int64_t m) {
  for (int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; b < m;
       b += static_cast<int64_t>(gridDim.x) * blockDim.x)
    dst[b] = src[b];
}

__global__ void multi_reduce_global_kernel(const int64_t* __restrict__ bins,
                                           const double* __restrict__ data, int64_t n,
                                           int64_t num_bins, double* __restrict__ values) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t b = __ldcs(bins + i);
    if (b >= 0 && b < num_bins) atomicAdd(&values[b], __ldcs(data + i));
  }
}

int small_grid(int64_t m) {
  const int64_t g = ceil_div(m > 0 ? m : 1, 256);
  return static_cast<int>(g < 1024 ? g : 1024);
}

}  // namespace

extern "C" {

int b200_algorithm_histogram(const int64_t* bins, int64_t n, int64_t num_bins,
                             const unsigned long long* counts_init, unsigned long long* counts,
                             const b200_tune* tune, b200_stream_t stream) {
  (void)tune;
  if (n < 0 || num_bins < 1 || !counts_init || !counts || (n > 0 && !bins))
    return invalid("b200_algorithm_histogram: bad args");
  cudaStream_t st = as_stream(stream);
  copy_u64_kernel<<<small_grid(num_bins), 256, 0, st>>>(counts_init, counts, num_bins);
  int launches = 1;
  if (n > 0) {
    if (num_bins <= kRegisterBins) {
      histogram_register_kernel<<<bin_grid(n), kBlock, 0, st>>>(
          bins, n, static_cast<int>(num_bins), aligned16(bins), counts);
    } else if (num_bins <= kSharedBins) {
      const size_t smem = static_cast<size_t>(num_bins) * sizeof(unsigned int);
      if (smem > 48 * 1024) {
        const int rc = allow_dynamic_smem(reinterpret_cast<const void*>(histogram_shared_kernel),
                                          smem, "b200_algorithm_histogram");
        if (rc != B200_OK) return rc;
      }
      histogram_shared_kernel<<<bin_grid(n), kBlock, smem, st>>>(bins, n, num_bins, counts);
    } else {
      histogram_global_kernel<<<bin_grid(n) * 4, kBlock, 0, st>>>(bins, n, num_bins, counts);
    }
    ++launches;
  }
  return after_launch("b200_algorithm_histogram", launches);
}

size_t b200_multi_reduce_workspace_bytes(int64_t n, int64_t num_bins) {
  if (num_bins < 1 || num_bins > kPrivateBins) return 256;
  return 256 + static_cast<size_t>(bin_grid(n)) * static_cast<size_t>(num_bins) * 8;
}

int b200_basic_multi_reduce(const int64_t* bins, const double* data, int64_t n,
                            int64_t num_bins, const double* values_init, double* values,
                            void* workspace, size_t workspace_bytes, const b200_tune* tune,
                            b200_stream_t stream) {
  (void)tune;
  if (n < 0 || num_bins < 1 || !values_init || !values || (n > 0 && (!bins || !data)))
    return invalid("b200_basic_multi_reduce: bad args");
  cudaStream_t st = as_stream(stream);
  if (num_bins > kPrivateBins || n == 0) {
    copy_f64_kernel<<<small_grid(num_bins), 256, 0, st>>>(values_init, values, num_bins);
    if (n > 0)
      multi_reduce_global_kernel<<<bin_grid(n) * 4, kBlock, 0, st>>>(bins, data, n, num_bins,
                                                                      values);
    return after_launch("b200_basic_multi_reduce", n > 0 ? 2 : 1);
  }
  const size_t need = b200_multi_reduce_workspace_bytes(n, num_bins);
  if (!workspace || workspace_bytes < need) {
    set_error("b200_basic_multi_reduce: workspace %zu bytes, need %zu", workspace_bytes, need);
    return B200_ERR_WORKSPACE;
  }
  const size_t smem = static_cast<size_t>(num_bins) * kBlock * sizeof(double);
  if (smem > 48 * 1024) {
    const int rc = allow_dynamic_smem(reinterpret_cast<const void*>(multi_reduce_private_kernel),
                                      smem, "b200_basic_multi_reduce");
    if (rc != B200_OK) return rc;
  }
  char* w = static_cast<char*>(workspace);
  multi_reduce_private_kernel<<<bin_grid(n), kBlock, smem, st>>>(
      bins, data, n, static_cast<int>(num_bins), values_init, values,
      reinterpret_cast<double*>(w + 256), reinterpret_cast<unsigned int*>(w));
  return after_launch("b200_basic_multi_reduce");
}

}  // extern "C"
