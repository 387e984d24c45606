// Algorithm group: SCAN (exclusive prefix sum, FP64 and int64) and REDUCE_SUM.
//
// SCAN is a single-pass decoupled-lookback scan: every CTA takes the next
// tile id from a counter (so a CTA only ever waits on tiles already owned by
// running CTAs).  A dedicated lookback warp starts walking its predecessors'
// aggregates / inclusive prefixes at once, while eight loader warps stage
// the tile in shared memory, reduce it and publish its aggregate; the
// lookback warp then publishes the tile's inclusive prefix and the loaders
// write the tile out.  Flags carry a launch epoch, so the workspace never
// needs re-zeroing between calls (and the call can be captured in a CUDA
// graph): the last CTA to finish resets the tile counter and advances the
// epoch.  Every wait is bounded; a wait that gives up sets the error word of
// the workspace header (byte offset 16) and the call's results are invalid.
#include "b200_internal.cuh"
#include "b200_reduce.cuh"

using namespace b200;

namespace {

constexpr int kScanBlock = 256;                         // loader threads
constexpr int kScanThreads = kScanBlock + 32;           // + the lookback warp
constexpr int kScanItemsMin = 16;                       // smallest tile: 4096 items
constexpr int kScanItemsDefault = 32;                   // default tile: 8192 items
constexpr int kScanTileMin = kScanBlock * kScanItemsMin;
constexpr int kLookbackPerLane = 4;                     // 128 predecessors per round
constexpr long long kSpinLimit = 1LL << 22;

struct ScanHeader {
  unsigned long long epoch;
  unsigned int tile_counter;
  unsigned int done_counter;
  unsigned int error;
  unsigned int pad[59];
};
static_assert(sizeof(ScanHeader) == 256, "scan header is 256 bytes");

// A tile's descriptor: {status, value} in one 16-byte word, read and written
// as single 128-bit accesses (PTX .b128), so a reader that sees a status also
// sees the value published with it; no other data is ordered by a
// descriptor, so relaxed accesses suffice and a lane's loads of several
// descriptors are in flight together.  status = epoch * 4 + (AGG 1 | INC 2).
struct alignas(16) TileDesc {
  unsigned long long status;
  unsigned long long value;  // the T's bits
};

__device__ __forceinline__ void desc_load(const TileDesc* d, unsigned long long& status,
                                          unsigned long long& value) {
  asm volatile(
      "{\n\t.reg .b128 t;\n\t"
      "ld.relaxed.gpu.global.b128 t, [%2];\n\t"
      "mov.b128 {%0, %1}, t;\n\t}"
      : "=l"(status), "=l"(value)
      : "l"(d)
      : "memory");
}

__device__ __forceinline__ void desc_store(TileDesc* d, unsigned long long status,
                                           unsigned long long value) {
  asm volatile(
      "{\n\t.reg .b128 t;\n\t"
      "mov.b128 t, {%1, %2};\n\t"
      "st.relaxed.gpu.global.b128 [%0], t;\n\t}" ::"l"(d),
      "l"(status), "l"(value)
      : "memory");
}

template <typename T>
__device__ __forceinline__ unsigned long long to_bits(T v) {
  unsigned long long b;
  memcpy(&b, &v, sizeof(b));
  return b;
}
template <typename T>
__device__ __forceinline__ T from_bits(unsigned long long b) {
  T v;
  memcpy(&v, &b, sizeof(v));
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T o = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v += o;
  }
  return v;
}

// Waits (bounded) until predecessor p has published at least its aggregate
// for this launch; returns its status and value.  A wait that gives up
// records the error and reports an inclusive prefix so the lookback ends.
__device__ __forceinline__ unsigned long long wait_desc(const TileDesc* descs, int64_t p,
                                                        unsigned long long AGG,
                                                        unsigned long long INC,
                                                        ScanHeader* hdr,
                                                        unsigned long long& value) {
  unsigned long long st;
  desc_load(descs + p, st, value);
  long long spins = 0;
  while (st < AGG) {
    if (++spins > kSpinLimit) {
      atomicExch(&hdr->error, 1u);
      value = 0ull;
      return INC;
    }
    if (spins > 64) __nanosleep(64);
    desc_load(descs + p, st, value);
  }
  return st;
}

__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// One CTA per tile of kScanBlock * IT items.  Warp 0 is the lookback warp:
// it walks the predecessors' flags as soon as the tile id is known, while
// warps 1..8 (the loaders) stage the tile in shared memory (padded so the
// per-thread runs of IT consecutive items are conflict-free), reduce it and
// publish the aggregate.  The lookback warp then publishes the inclusive
// prefix, and the loaders write the tile out.  Named barriers: 1 = loaders
// only, 2 = aggregate ready (loaders arrive, lookback warp waits), 3 =
// exclusive prefix ready (lookback warp arrives, loaders wait).
template <typename T, int IT>
__global__ void __launch_bounds__(kScanThreads)
scan_kernel(const T* __restrict__ x, T* __restrict__ y, int64_t n, T init,
            ScanHeader* __restrict__ hdr, TileDesc* __restrict__ descs) {
  constexpr int kTile = kScanBlock * IT;
  constexpr int kPadShift = (IT == 32) ? 5 : 4;
  extern __shared__ __align__(16) unsigned char s_raw[];
  T* s_tile = reinterpret_cast<T*>(s_raw);
  __shared__ T s_warp[kScanBlock / 32];
  __shared__ T s_excl;
  __shared__ T s_agg;
  __shared__ unsigned int s_tile_id;
  __shared__ unsigned long long s_epoch;
  __shared__ bool s_last;
  auto pad = [](int i) { return i + (i >> kPadShift); };

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_epoch = *reinterpret_cast<volatile unsigned long long*>(&hdr->epoch);
    s_tile_id = atomicAdd(&hdr->tile_counter, 1u);
  }
  __syncthreads();
  const unsigned int tile = s_tile_id;
  const unsigned long long epoch = s_epoch;
  const unsigned long long AGG = epoch * 4 + 1, INC = epoch * 4 + 2;
  const int64_t base = static_cast<int64_t>(tile) * kTile;

  if (warp == 0) {
    // ---- lookback warp ----
    // One round examines 32 * kLookbackPerLane predecessors, nearest first
    // (window slot w = j * 32 + lane is predecessor p_hi - w).
    T exclusive = init;
    if (tile > 0) {
      T acc = T(0);
      int64_t p_hi = static_cast<int64_t>(tile) - 1;  // nearest unexamined predecessor
      bool done = false;
      while (!done) {
        unsigned long long f[kLookbackPerLane];
        T v[kLookbackPerLane];
        unsigned long long bits[kLookbackPerLane];
#pragma unroll
        for (int j = 0; j < kLookbackPerLane; ++j) {  // all loads first
          const int64_t p = p_hi - (j * 32 + lane);
          f[j] = INC;                                  // p < 0: end of the lookback
          bits[j] = 0ull;
          if (p >= 0) desc_load(descs + p, f[j], bits[j]);
        }
#pragma unroll
        for (int j = 0; j < kLookbackPerLane; ++j) {  // then wait for the late ones
          const int64_t p = p_hi - (j * 32 + lane);
          if (p >= 0 && f[j] < AGG) f[j] = wait_desc(descs, p, AGG, INC, hdr, bits[j]);
          v[j] = from_bits<T>(bits[j]);
        }
        // nearest window slot holding an inclusive prefix
        int stop = 32 * kLookbackPerLane;
#pragma unroll
        for (int j = kLookbackPerLane - 1; j >= 0; --j) {
          const unsigned int m = __ballot_sync(0xffffffffu, f[j] == INC);
          if (m) stop = j * 32 + __ffs(m) - 1;
        }
        // fixed order: slots j = 0.. summed per lane, then a fixed lane tree
        T val = T(0);
#pragma unroll
        for (int j = 0; j < kLookbackPerLane; ++j)
          if (j * 32 + lane <= stop) val += v[j];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) val += __shfl_down_sync(0xffffffffu, val, off);
        acc += __shfl_sync(0xffffffffu, val, 0);
        if (stop < 32 * kLookbackPerLane) done = true;
        p_hi -= 32 * kLookbackPerLane;
      }
      exclusive = acc;
    }
    named_sync(2, kScanThreads);  // the loaders have the tile aggregate
    if (lane == 0) {
      desc_store(descs + tile, INC, to_bits<T>(exclusive + s_agg));
      s_excl = exclusive;
    }
    named_arrive(3, kScanThreads);
  } else {
    // ---- loaders ----
    const int ltid = tid - 32, lwarp = warp - 1;
    if (base + kTile <= n) {
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int k = u * kScanBlock + ltid;
        s_tile[pad(k)] = __ldcs(x + base + k);
      }
    } else {
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int k = u * kScanBlock + ltid;
        const int64_t i = base + k;
        s_tile[pad(k)] = (i < n) ? __ldcs(x + i) : T(0);
      }
    }
    named_sync(1, kScanBlock);
    // Each thread sums its IT consecutive items; a scan of the thread totals
    // gives every thread its offset inside the tile.
    T run = T(0);
#pragma unroll
    for (int u = 0; u < IT; ++u) run += s_tile[pad(ltid * IT + u)];
    const T incl = warp_inclusive_scan(run);
    if (lane == 31) s_warp[lwarp] = incl;
    named_sync(1, kScanBlock);
    if (lwarp == 0) {
      const T w = (lane < kScanBlock / 32) ? s_warp[lane] : T(0);
      const T wi = warp_inclusive_scan(w);
      if (lane < kScanBlock / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
      if (lane == kScanBlock / 32 - 1) {
        s_agg = wi;                                       // tile aggregate
        if (tile > 0) desc_store(descs + tile, AGG, to_bits<T>(wi));
      }
    }
    named_sync(1, kScanBlock);
    named_arrive(2, kScanThreads);
    // tile-local exclusive prefixes, in place
    {
      T r = s_warp[lwarp] + (incl - run);
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int k = pad(ltid * IT + u);
        const T xv = s_tile[k];
        s_tile[k] = r;
        r += xv;
      }
    }
    named_sync(1, kScanBlock);
    named_sync(3, kScanThreads);  // the lookback warp has the exclusive prefix
    const T prefix = s_excl;
    if (base + kTile <= n) {
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int k = u * kScanBlock + ltid;
        __stcs(y + base + k, prefix + s_tile[pad(k)]);
      }
    } else {
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int k = u * kScanBlock + ltid;
        const int64_t i = base + k;
        if (i < n) __stcs(y + i, prefix + s_tile[pad(k)]);
      }
    }
  }

  // the last CTA to finish prepares the workspace for the next call
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    unsigned int prev = atomicAdd(&hdr->done_counter, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && tid == 0) {
    hdr->tile_counter = 0u;
    hdr->done_counter = 0u;
    __threadfence();
    *reinterpret_cast<volatile unsigned long long*>(&hdr->epoch) = epoch + 1;
  }
}

// The workspace is sized for the smallest tile, so it serves every tile size.
int64_t scan_tiles_max(int64_t n) { return ceil_div(n > 0 ? n : 1, kScanTileMin); }

template <typename T, int IT>
int launch_scan_it(const T* x, T* y, int64_t n, T init, char* w, cudaStream_t st) {
  constexpr int kTile = kScanBlock * IT;
  constexpr size_t kSmem = static_cast<size_t>(kTile + kTile / IT) * sizeof(T);
  const cudaError_t attr = cudaFuncSetAttribute(
      scan_kernel<T, IT>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmem));
  if (attr != cudaSuccess) {
    set_error("scan: shared memory attribute: %s", cudaGetErrorString(attr));
    return B200_ERR_LAUNCH;
  }
  const int64_t tiles = ceil_div(n, kTile);
  ScanHeader* hdr = reinterpret_cast<ScanHeader*>(w);
  TileDesc* descs = reinterpret_cast<TileDesc*>(w + 256);
  scan_kernel<T, IT><<<static_cast<int>(tiles), kScanThreads, kSmem, st>>>(x, y, n, init, hdr,
                                                                          descs);
  return B200_OK;
}

template <typename T>
int launch_scan(const char* name, const T* x, T* y, int64_t n, T init, void* ws,
                size_t ws_bytes, const b200_tune* tune, cudaStream_t st) {
  if (n < 0 || (n > 0 && (!x || !y))) return invalid("%s: bad args", name);
  if (n == 0) return B200_OK;
  const int64_t slots = scan_tiles_max(n);
  if (slots > 0x7fffffffLL) return invalid("%s: n too large", name);
  if (tune && tune->block_size && tune->block_size != kScanBlock)
    return invalid("%s: block size %d (only %d)", name, tune->block_size, kScanBlock);
  const int items = (tune && tune->items) ? tune->items : kScanItemsDefault;
  if (items != 16 && items != 32) return invalid("%s: items %d (16 or 32)", name, items);
  size_t need = 256 + static_cast<size_t>(slots) * sizeof(TileDesc);
  if (ws && !aligned16(ws)) return invalid("%s: workspace not 16-byte aligned", name);
  if (!ws || ws_bytes < need) {
    set_error("%s: workspace %zu bytes, need %zu", name, ws_bytes, need);
    return B200_ERR_WORKSPACE;
  }
  char* w = static_cast<char*>(ws);
  const int rc = (items == 16) ? launch_scan_it<T, 16>(x, y, n, init, w, st)
                               : launch_scan_it<T, 32>(x, y, n, init, w, st);
  if (rc != B200_OK) return rc;
  return after_launch(name);
}

// ---- REDUCE_SUM -------------------------------------------------------------
template <int BS, int IT>
__global__ void __launch_bounds__(BS)
reduce_sum_kernel(const double* __restrict__ x, int64_t n, double init,
                  double* __restrict__ out, double* __restrict__ partials,
                  unsigned int* __restrict__ counter) {
  __shared__ double smem[BS / 32];
  __shared__ bool last_flag;
  double s = 0.0;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < n;
       t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
    double v[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t i = t0 + u * BS + threadIdx.x;
      v[u] = (i < n) ? __ldg(x + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) s += v[u];
  }
  s = block_sum<BS>(s, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  if (arrive_last(counter, &last_flag)) {
    double t = 0.0;
    for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += BS)
      t += __ldcg(partials + i);
    t = block_sum<BS>(t, smem);
    if (threadIdx.x == 0) {
      *out = init + t;
      *counter = 0u;
    }
  }
}

}  // namespace

extern "C" {

size_t b200_scan_workspace_bytes(int64_t n) {
  return 256 + static_cast<size_t>(scan_tiles_max(n)) * sizeof(TileDesc);
}

int b200_algorithm_scan(const double* x, double* y, int64_t n, double init,
                        void* workspace, size_t workspace_bytes, const b200_tune* tune,
                        b200_stream_t stream) {
  return launch_scan<double>("b200_algorithm_scan", x, y, n, init, workspace,
                             workspace_bytes, tune, as_stream(stream));
}

int b200_algorithm_scan_i64(const int64_t* x, int64_t* y, int64_t n, int64_t init,
                            void* workspace, size_t workspace_bytes,
                            const b200_tune* tune, b200_stream_t stream) {
  return launch_scan<long long>("b200_algorithm_scan_i64",
                                reinterpret_cast<const long long*>(x),
                                reinterpret_cast<long long*>(y), n,
                                static_cast<long long>(init), workspace, workspace_bytes,
                                tune, as_stream(stream));
}

int b200_algorithm_reduce_sum(const double* x, int64_t n, double sum_init, double* sum,
                              void* workspace, size_t workspace_bytes,
                              const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && !x) || !sum) return invalid("b200_algorithm_reduce_sum: bad args");
  int block = (tune && tune->block_size) ? tune->block_size : 256;
  int items = (tune && tune->items) ? tune->items : 8;
  if (!valid_block(block))
    return invalid("b200_algorithm_reduce_sum: bad block size %d", block);
  int grid = reduce_grid(n, tune, block, items);
  size_t need = reduce_ws_bytes_for_grid(grid);
  if (!workspace || workspace_bytes < need) {
    set_error("b200_algorithm_reduce_sum: workspace %zu bytes, need %zu", workspace_bytes,
              need);
    return B200_ERR_WORKSPACE;
  }
  unsigned int* counter = static_cast<unsigned int*>(workspace);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(workspace) + 256);
  cudaStream_t st = as_stream(stream);
  B200_DISPATCH_BLOCK(block, BS, B200_DISPATCH_ITEMS(items, IT,
    reduce_sum_kernel<BS, IT><<<grid, BS, 0, st>>>(x, n, sum_init, sum, partials, counter)));
  return after_launch("b200_algorithm_reduce_sum");
}

}  // extern "C"
