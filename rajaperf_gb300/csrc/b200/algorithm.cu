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
// graph): the CTA that draws the launch's last tile id resets the tile
// counter and advances the epoch.  Every wait is bounded; a wait that gives up sets the error word of
// the workspace header (byte offset 16) and the call's results are invalid.
#include "b200_internal.cuh"
#include "b200_fma_form.cuh"
#include "b200_async.cuh"
#include "b200_lookback.cuh"
#include "b200_pipeline.cuh"
#include "b200_reduce.cuh"

#include <type_traits>

using namespace b200;

namespace {

constexpr int kScanBlock = 256;                         // loader threads
constexpr int kScanThreads = kScanBlock + 32;           // + the lookback warp
constexpr int kScanItemsMin = 16;                       // smallest tile: 4096 items
constexpr int kScanItemsDefault = 32;                   // default tile: 8192 items
constexpr int kScanTileMin = kScanBlock * kScanItemsMin;

// One CTA per tile of kScanBlock * IT items.  Warp 0 is the lookback warp:
// it walks the predecessors' flags as soon as the tile id is known, while
// warps 1..8 (the loaders) stage the tile in shared memory (padded so the
// per-thread runs of IT consecutive items are conflict-free), reduce it and
// publish the aggregate.  The lookback warp then publishes the inclusive
// prefix, and the loaders write the tile out.  Named barriers: 1 = loaders
// only, 2 = aggregate ready (loaders arrive, lookback warp waits), 3 =
// exclusive prefix ready (lookback warp arrives, loaders wait).
// 16-byte vector of two T (double2 / longlong2).
template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<long long> { using type = longlong2; };

template <typename T, int IT, bool VEC>
__global__ void __launch_bounds__(kScanThreads, 3)
scan_kernel(const T* __restrict__ x, T* __restrict__ y, int64_t n, T init,
            ScanHeader* __restrict__ hdr, TileDesc* __restrict__ descs, uint64_t limit_ns) {
  using V2 = typename Vec2<T>::type;
  constexpr int kTile = kScanBlock * IT;
  constexpr int kPadShift = (IT == 32) ? 5 : 4;
  extern __shared__ __align__(16) unsigned char s_raw[];
  T* s_tile = reinterpret_cast<T*>(s_raw);
  __shared__ T s_warp[kScanBlock / 32];
  __shared__ T s_excl;
  __shared__ T s_agg;
  __shared__ unsigned int s_tile_id;
  __shared__ unsigned long long s_epoch;
  auto pad = [](int i) { return i + (i >> kPadShift); };

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  take_tile(hdr, &s_tile_id, &s_epoch);
  const unsigned int tile = s_tile_id;
  const unsigned long long epoch = s_epoch;
  const unsigned long long AGG = epoch * 4 + 1, INC = epoch * 4 + 2;
  const int64_t base = static_cast<int64_t>(tile) * kTile;

  if (warp == 0) {
    // ---- lookback warp ----
    // One round examines 32 * kLookbackPerLane predecessors, nearest first
    // (window slot w = j * 32 + lane is predecessor p_hi - w).
    const T exclusive =
        (tile > 0) ? lookback_exclusive<T>(descs, tile, AGG, INC, hdr, limit_ns) : init;
    named_sync(2, kScanThreads);  // the loaders have the tile aggregate
    if (lane == 0) {
      desc_store(descs + tile, INC, to_bits<T>(exclusive + s_agg));
      s_excl = exclusive;
    }
    named_arrive(3, kScanThreads);
  } else {
    // ---- loaders ----
    const int ltid = tid - 32, lwarp = warp - 1;
    if (VEC && base + kTile <= n) {
      // 16-byte loads of item pairs (x 16-byte aligned, tiles start even)
      const V2* xv = reinterpret_cast<const V2*>(x + base);
#pragma unroll
      for (int u = 0; u < IT / 2; ++u) {
        const int k2 = u * kScanBlock + ltid;
        const V2 v = __ldcs(xv + k2);
        s_tile[pad(2 * k2)] = v.x;
        s_tile[pad(2 * k2 + 1)] = v.y;
      }
    } else if (base + kTile <= n) {
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
    if (VEC && base + kTile <= n) {
      V2* yv = reinterpret_cast<V2*>(y + base);
#pragma unroll
      for (int u = 0; u < IT / 2; ++u) {
        const int k2 = u * kScanBlock + ltid;
        V2 v;
        v.x = prefix + s_tile[pad(2 * k2)];
        v.y = prefix + s_tile[pad(2 * k2 + 1)];
        __stcs(yv + k2, v);
      }
    } else if (base + kTile <= n) {
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

}

// ---- pipelined persistent SCAN ---------------------------------------------
// One CTA per SM on the stage ring of b200_pipeline.cuh (producer warp 0,
// lookback warps 2-3), plus:
//  * aggregator (warp 1): sums each tile as it lands and publishes the
//    aggregate at once;
//  * compute (warps 4-7): a thread owns a run of 32 consecutive items (16
//    item pairs), sums it, scans the run sums across the tile and, when the
//    tile's exclusive prefix arrives, writes every item's prefix in place;
//  * store (warp 8): writes a finished tile back with one bulk store and
//    frees the stage once the store has read it (mbarrier ready[s]: compute
//    -> store).
// A compute thread visits its pairs rotated by (run mod 16), so every 16-byte
// shared-memory access of a warp is conflict-free without padding the
// bulk-copied tile.  Measured on GB300 (int64, 2^26 items, time marks per
// tile and role): the bare load -> store pipeline runs at the copy peak; what
// the lookback adds is its L2 round trips under saturated HBM, which the
// seven stages of loads in flight are there to cover.
namespace pipe {

using ring::kStages;
using ring::kTile;
using ring::kEnd;
constexpr int kComputeWarps = 4;
constexpr int kFirstCompute = 2 + ring::kLookbackWarps;
constexpr int kStoreWarp = kFirstCompute + kComputeWarps;
constexpr int kThreads = 32 * (kStoreWarp + 1);
constexpr int kRuns = 32 * kComputeWarps;    // 128 runs per tile
constexpr int kPairs = kTile / kRuns / 2;    // 16 pairs per run

template <typename T>
struct Smem {
  ring::Ring<T, T> r;
  T warp_total[kComputeWarps];
  uint64_t ready[kStages];  // compute -> store warp: the stage holds results
  int fail_loaded;          // compute group: a wait before its first barrier gave up
  int fail_prefix;          // compute group: a wait before its second barrier gave up
};

template <typename T>
constexpr size_t smem_bytes() { return sizeof(Smem<T>) + 128; }
static_assert(sizeof(Smem<double>) + 128 <= 232448, "shared memory budget");

template <typename T>
__global__ void __launch_bounds__(kThreads, 1)
scan_pipelined(const T* __restrict__ x, T* __restrict__ y, int64_t n, T init,
               unsigned int tiles, ScanHeader* __restrict__ hdr,
               TileDesc* __restrict__ descs, uint64_t limit_ns) {
  using V2 = typename Vec2<T>::type;
  extern __shared__ unsigned char s_raw[];
  Smem<T>& sm = *reinterpret_cast<Smem<T>*>(
      (reinterpret_cast<uintptr_t>(s_raw) + 127) & ~static_cast<uintptr_t>(127));
  ring::Ring<T, T>& r = sm.r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    ring::init(r, limit_ns);
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.ready[s], 1);
    sm.fail_loaded = 0;
    sm.fail_prefix = 0;
    mbar_init_fence();
  }
  __syncthreads();

  if (warp == 0) {
    ring::produce(r, x, n, tiles, hdr);
  } else if (warp == 1) {
    // ---- aggregator: lane L sums pairs L, L + 32, ... (conflict-free) ----
    for (int k = 0;; ++k) {
      const int s = k % kStages;
      if (!ring::wait(r, &r.full[s], (k / kStages) & 1, hdr)) break;
      const unsigned int tile = r.ticket[s];
      if (tile == kEnd) break;
      const V2* tv = reinterpret_cast<const V2*>(r.tile[s]);
      T total = T(0);
#pragma unroll 16
      for (int q = lane; q < kTile / 2; q += 32) {
        const V2 v = tv[q];
        total += v.x;
        total += v.y;
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) total += __shfl_xor_sync(0xffffffffu, total, off);
      if (lane == 0) ring::publish_aggregate(r, descs, s, tile, total);
      __syncwarp();
      if (lane == 0) mbar_arrive(&r.summed[s]);
    }
  } else if (warp < kFirstCompute) {
    ring::look_back(r, descs, init, hdr, warp - 2);
  } else if (warp < kStoreWarp) {
    // ---- compute ----
    // The four warps decide together whether to go on: a warp whose wait
    // gave up sets a flag before the next group barrier and every thread
    // reads it after that barrier, so no thread is left at a later barrier.
    // The two barriers of an iteration use separate flags: a failure in the
    // next iteration can only be recorded after every thread has passed
    // this iteration's reads of the flag it sets.
    const int ct = tid - 32 * kFirstCompute, cw = ct >> 5;
    const int rot = ct & (kPairs - 1);
    volatile int* fail_loaded = &sm.fail_loaded;
    volatile int* fail_prefix = &sm.fail_prefix;
    for (int k = 0;; ++k) {
      const int s = k % kStages;
      const uint32_t par = (k / kStages) & 1;
      const bool loaded = ring::wait(r, &r.full[s], par, hdr);
      const unsigned int tile = r.ticket[s];
      if (!loaded) *fail_loaded = 1;
      V2* tv = reinterpret_cast<V2*>(r.tile[s]) + ct * kPairs;
      V2 v[kPairs];
      T head = T(0), tail = T(0);  // pairs q < rot come first in index order
      if (loaded && tile != kEnd) {
#pragma unroll
        for (int w = 0; w < kPairs; ++w) v[w] = tv[(w + rot) & (kPairs - 1)];
#pragma unroll
        for (int w = 0; w < kPairs; ++w) {
          if (w >= kPairs - rot) {
            head += v[w].x;
            head += v[w].y;
          } else {
            tail += v[w].x;
            tail += v[w].y;
          }
        }
      }
      const T rs = head + tail;
      const T inc = warp_inclusive_scan(rs);
      if (lane == 31) sm.warp_total[cw] = inc;
      named_sync(1, 32 * kComputeWarps);
      if (*fail_loaded || tile == kEnd) {
        if (ct == 0 && !*fail_loaded) mbar_arrive(&sm.ready[s]);  // end marker for the store warp
        break;
      }
      T woff = T(0);
      for (int w = 0; w < cw; ++w) woff += sm.warp_total[w];
      const bool have_prefix = ring::wait(r, &r.prefix[s], par, hdr);
      if (have_prefix) {
        const T base = r.excl[s] + (woff + (inc - rs));
        T run = base + head;
#pragma unroll
        for (int w = 0; w < kPairs; ++w) {
          if (w == kPairs - rot) run = base;
          V2 o;
          o.x = run;
          run += v[w].x;
          o.y = run;
          run += v[w].y;
          tv[(w + rot) & (kPairs - 1)] = o;
        }
        fence_proxy_async_smem();
      } else {
        *fail_prefix = 1;
      }
      named_sync(2, 32 * kComputeWarps);
      if (*fail_prefix) break;
      const int64_t first = static_cast<int64_t>(tile) * kTile;
      if (first + kTile > n) {
        // the ragged last tile: plain stores
        for (int i = ct; first + i < n; i += 32 * kComputeWarps) y[first + i] = r.tile[s][i];
      }
      if (ct == 0) mbar_arrive(&sm.ready[s]);
    }
  } else {
    // ---- store: one bulk store per finished tile, then the stage is free ----
    for (int k = 0;; ++k) {
      const int s = k % kStages;
      if (!ring::wait(r, &sm.ready[s], (k / kStages) & 1, hdr)) break;
      const unsigned int tile = r.ticket[s];
      if (tile == kEnd) break;
      const int64_t first = static_cast<int64_t>(tile) * kTile;
      if (lane == 0) {
        if (first + kTile <= n) {
          bulk_store(y + first, r.tile[s], kTile * sizeof(T));
          bulk_commit();
          bulk_wait_read<0>();
        }
        mbar_arrive(&r.empty[s]);
      }
      __syncwarp();
    }
    if (lane == 0) bulk_wait_all();
  }

  __syncthreads();
  if (tid == 0) ring::drain(r);
}

}  // namespace pipe

// The workspace is sized for the smallest tile, so it serves every tile size.
int64_t scan_tiles_max(int64_t n) { return ceil_div(n > 0 ? n : 1, kScanTileMin); }

template <typename T, int IT, bool VEC>
int launch_scan_it(const T* x, T* y, int64_t n, T init, char* w, uint64_t limit_ns,
                   cudaStream_t st) {
  constexpr int kTile = kScanBlock * IT;
  constexpr size_t kSmem = static_cast<size_t>(kTile + kTile / IT) * sizeof(T);
  const int rc = allow_dynamic_smem(reinterpret_cast<const void*>(scan_kernel<T, IT, VEC>),
                                    kSmem, "scan");
  if (rc != B200_OK) return rc;
  const int64_t tiles = ceil_div(n, kTile);
  ScanHeader* hdr = reinterpret_cast<ScanHeader*>(w);
  TileDesc* descs = reinterpret_cast<TileDesc*>(w + 256);
  scan_kernel<T, IT, VEC><<<static_cast<int>(tiles), kScanThreads, kSmem, st>>>(
      x, y, n, init, hdr, descs, limit_ns);
  return B200_OK;
}

template <typename T>
int launch_scan_pipelined(const T* x, T* y, int64_t n, T init, char* w, uint64_t limit_ns,
                          cudaStream_t st) {
  constexpr size_t kSmem = pipe::smem_bytes<T>();
  const int rc = allow_dynamic_smem(reinterpret_cast<const void*>(pipe::scan_pipelined<T>),
                                    kSmem, "scan");
  if (rc != B200_OK) return rc;
  const int64_t tiles = ceil_div(n, pipe::kTile);
  const int grid = static_cast<int>(std::min<int64_t>(tiles, device_info().sm_count));
  pipe::scan_pipelined<T><<<grid, pipe::kThreads, kSmem, st>>>(
      x, y, n, init, static_cast<unsigned int>(tiles), reinterpret_cast<ScanHeader*>(w),
      reinterpret_cast<TileDesc*>(w + 256), limit_ns);
  return B200_OK;
}

template <typename T>
int launch_scan(const char* name, const T* x, T* y, int64_t n, T init, void* ws,
                size_t ws_bytes, const b200_tune* tune, cudaStream_t st) {
  if (n < 0 || (n > 0 && (!x || !y))) return invalid("%s: bad args", name);
  if (n == 0) return B200_OK;
  const int64_t slots = scan_tiles_max(n);
  if (slots > 0x7fffffffLL) return invalid("%s: n too large", name);
  const int algo = tune ? tune->algo : 0;
  if (algo < 0 || algo > 2) return invalid("%s: algo %d (0, 1 or 2)", name, algo);
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
  const bool vec = aligned16(x) && aligned16(y) && !(tune && tune->vec == 1);
  const uint64_t lim = wait_limit_ns(tune, kDefaultWaitNs);
  int rc;
  // the ring's aggregator warp sums a tile on one sub-partition's FP64 unit
  // (FP64-bound at 4 us per tile), so FP64 takes the tile kernel by default
  const bool ring = vec && (algo == 2 || (algo == 0 && std::is_same<T, long long>::value));
  if (ring)
    rc = launch_scan_pipelined<T>(x, y, n, init, w, lim, st);
  else
    rc = (items == 16) ? (vec ? launch_scan_it<T, 16, true>(x, y, n, init, w, lim, st)
                              : launch_scan_it<T, 16, false>(x, y, n, init, w, lim, st))
                       : (vec ? launch_scan_it<T, 32, true>(x, y, n, init, w, lim, st)
                              : launch_scan_it<T, 32, false>(x, y, n, init, w, lim, st));
  if (rc != B200_OK) return rc;
  return after_launch(name);
}

// ---- REDUCE_SUM -------------------------------------------------------------
template <int BS, int IT>
__global__ void __launch_bounds__(BS)
reduce_sum_kernel(const double* __restrict__ x, int64_t n, double init,
                  double* __restrict__ out, double* __restrict__ partials,
                  unsigned int* __restrict__ counter, int zero) {
  __shared__ double smem[BS / 32];
  __shared__ bool last_flag;
  double s = 0.0;
  // s + v as a register-operand FMA (fform: bit-identical, full FP64 rate
  // where DADD gets 5/6 of it); `zero` is 0 at run time
  const double one = fform::regs(zero).one;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < n;
       t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
    double v[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t i = t0 + u * BS + threadIdx.x;
      v[u] = (i < n) ? __ldg(x + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) s = fma(v[u], one, s);  // s + v[u]
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
    reduce_sum_kernel<BS, IT><<<grid, BS, 0, st>>>(x, n, sum_init, sum, partials, counter, 0)));
  return after_launch("b200_algorithm_reduce_sum");
}

}  // extern "C"
