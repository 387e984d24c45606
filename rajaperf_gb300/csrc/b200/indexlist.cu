// INDEXLIST (and INDEXLIST_3LOOP): list[count++] = i for every i with
// x[i] < 0, in index order, and the final count.
//
// One pass, stream compaction on the decoupled lookback of b200_lookback.cuh.
// A CTA owns a tile of 8 warps x 32 lanes x 32 items; each warp owns a
// contiguous segment of 1024 items and reads it row by row (coalesced,
// 16-byte item pairs when x is aligned).  Ballots per row give every selected
// item its rank inside the row; the warp's running count orders the rows; a
// scan of the warp counts orders the warps; the lookback gives the tile's
// base count.  The indices are then written to consecutive list entries.
// The suite's INDEXLIST_3LOOP
// (counts, exclusive scan of counts, list from count changes) produces the
// same list and count; it runs through the same single pass.
//
// Default (x 16-byte aligned): the persistent form on the stage ring of
// b200_pipeline.cuh, as SCAN: bulk copies keep up to seven 4096-item tiles in
// flight per SM, an aggregator warp publishes each tile's count as soon as it
// lands, two lookback warps resolve the tiles' base counts, and four compute
// warps rank and write the indices.  tune->algo = 1 (and an unaligned x) runs
// the one-CTA-per-tile kernel below.  Both test x < 0 on the integer pipe
// (f64emu::lt_zero, exact): GB300's FP64 pipe compares 2 items per clock per
// SM, which alone bounded the first kernel at 43% of the copy peak.
#include "b200_internal.cuh"
#include "b200_async.cuh"
#include "b200_f64emu.cuh"
#include "b200_lookback.cuh"
#include "b200_pipeline.cuh"

using namespace b200;

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 32;
constexpr int kTile = kBlock * kItems;  // 8192 items
constexpr int kSeg = 32 * kItems;       // a warp's segment: 1024 items

// VEC: 16-byte loads, lane L of row u holds items seg + 64u + 2L and +1 (x
// 16-byte aligned, n even or the tile full); otherwise 8-byte loads, lane L
// of row u holds item seg + 32u + L.  Ranks follow index order either way.
template <bool VEC>
__global__ void __launch_bounds__(kBlock, 3)
indexlist_kernel(const double* __restrict__ x, int32_t* __restrict__ list, int64_t n,
                 int64_t* __restrict__ len, ScanHeader* __restrict__ hdr,
                 TileDesc* __restrict__ descs, uint64_t limit_ns) {
  constexpr int kRows = VEC ? kItems / 2 : kItems;
  __shared__ long long s_woff[kBlock / 32];
  __shared__ long long s_agg;
  __shared__ long long s_excl;
  __shared__ unsigned int s_tile_id;
  __shared__ unsigned long long s_epoch;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  take_tile(hdr, &s_tile_id, &s_epoch);
  const unsigned int tile = s_tile_id;
  const unsigned long long epoch = s_epoch;
  const unsigned long long AGG = epoch * 4 + 1, INC = epoch * 4 + 2;
  const int64_t seg = static_cast<int64_t>(tile) * kTile + warp * kSeg;

  unsigned int b0[kRows], b1[kRows];  // ballots of the even / odd items of a row
  int wcount = 0;
#pragma unroll
  for (int u = 0; u < kRows; ++u) {
    if (VEC) {
      const int64_t i = seg + 64 * u + 2 * lane;
      double2 v = make_double2(0.0, 0.0);
      if (i + 1 < n) {
        v = __ldcs(reinterpret_cast<const double2*>(x + i));
      } else if (i < n) {
        v.x = __ldcs(x + i);
      }
      b0[u] = __ballot_sync(0xffffffffu, i < n && f64emu::lt_zero(v.x));
      b1[u] = __ballot_sync(0xffffffffu, i + 1 < n && f64emu::lt_zero(v.y));
      wcount += __popc(b0[u]) + __popc(b1[u]);
    } else {
      const int64_t i = seg + 32 * u + lane;
      b0[u] = __ballot_sync(0xffffffffu, (i < n) && f64emu::lt_zero(__ldcs(x + i)));
      b1[u] = 0u;
      wcount += __popc(b0[u]);
    }
  }
  if (lane == 0) s_woff[warp] = wcount;
  __syncthreads();
  if (warp == 0) {
    const long long w = (lane < kBlock / 32) ? s_woff[lane] : 0;
    long long wi = w;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const long long o = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi += o;
    }
    if (lane < kBlock / 32) s_woff[lane] = wi - w;
    const long long agg = __shfl_sync(0xffffffffu, wi, kBlock / 32 - 1);
    if (tile > 0) {
      if (lane == 0) desc_store(descs + tile, AGG, to_bits<long long>(agg));
      const long long excl = lookback_exclusive<long long>(descs, tile, AGG, INC, hdr, limit_ns);
      if (lane == 0) {
        desc_store(descs + tile, INC, to_bits<long long>(excl + agg));
        s_excl = excl;
        s_agg = agg;
      }
    } else if (lane == 0) {
      desc_store(descs, INC, to_bits<long long>(agg));
      s_excl = 0;
      s_agg = agg;
    }
  }
  __syncthreads();
  long long off = s_excl + s_woff[warp];
  const unsigned int below = (1u << lane) - 1u;
#pragma unroll
  for (int u = 0; u < kRows; ++u) {
    if (VEC) {
      const int64_t i = seg + 64 * u + 2 * lane;
      const int r = __popc(b0[u] & below) + __popc(b1[u] & below);
      const bool s0 = (b0[u] >> lane) & 1u, s1 = (b1[u] >> lane) & 1u;
      if (s0) list[off + r] = static_cast<int32_t>(i);
      if (s1) list[off + r + (s0 ? 1 : 0)] = static_cast<int32_t>(i + 1);
      off += __popc(b0[u]) + __popc(b1[u]);
    } else {
      if ((b0[u] >> lane) & 1u)
        list[off + __popc(b0[u] & below)] = static_cast<int32_t>(seg + 32 * u + lane);
      off += __popc(b0[u]);
    }
  }
  // the tile holding item n-1 knows the total
  if (tid == 0 && static_cast<int64_t>(tile + 1) * kTile >= n) *len = s_excl + s_agg;
}

int64_t tiles_of(int64_t n) { return ceil_div(n > 0 ? n : 1, kTile); }

// ---- persistent form on the stage ring ---------------------------------------
namespace ilpipe {

using ring::kEnd;
using ring::kStages;
constexpr int kTile = ring::kTile;
constexpr int kAggWarps = 2;                 // warps 1-2 (alternate tiles)
constexpr int kComputeWarps = 4;
constexpr int kFirstLookback = 1 + kAggWarps;
constexpr int kFirstCompute = kFirstLookback + ring::kLookbackWarps;
constexpr int kThreads = 32 * (kFirstCompute + kComputeWarps);
constexpr int kSeg = kTile / kComputeWarps;  // 1024 items per compute warp
static_assert(kAggWarps <= ring::kLookbackWarps, "an end marker for every aggregator");
constexpr int kRows = kSeg / 64;             // rows of 64 items (a lane holds a pair)

struct Smem {
  ring::Ring<double, long long> r;
  long long warp_count[kComputeWarps];
  int fail_loaded;  // compute group: a wait before its first barrier gave up
  int fail_prefix;  // compute group: a wait before its second barrier gave up
};
static_assert(sizeof(Smem) + 128 <= 232448, "shared memory budget");

__global__ void __launch_bounds__(kThreads, 1)
indexlist_pipelined(const double* __restrict__ x, int32_t* __restrict__ list, int64_t n,
                    int64_t* __restrict__ len, unsigned int tiles,
                    ScanHeader* __restrict__ hdr, TileDesc* __restrict__ descs,
                    uint64_t limit_ns) {
  extern __shared__ unsigned char s_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(
      (reinterpret_cast<uintptr_t>(s_raw) + 127) & ~static_cast<uintptr_t>(127));
  ring::Ring<double, long long>& r = sm.r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    ring::init(r, limit_ns);
    sm.fail_loaded = 0;
    sm.fail_prefix = 0;
    mbar_init_fence();
  }
  __syncthreads();

  if (warp == 0) {
    ring::produce(r, x, n, tiles, hdr);
  } else if (warp < kFirstLookback) {
    // ---- aggregators (alternate tiles): count of negative items; zero-filled
    // padding never counts.
    for (int k = warp - 1;; k += kAggWarps) {
      const int s = k % kStages;
      const uint32_t par = (k / kStages) & 1;
      // drawn[s] first: its phases complete in tile order, and this phase
      // means the stage's previous tile is done, so full[s] is waited on the
      // right phase (bulk copies can land out of order across stages)
      if (!ring::wait(r, &r.drawn[s], par, hdr) || !ring::wait(r, &r.full[s], par, hdr)) break;
      const unsigned int tile = r.ticket[s];
      if (tile == kEnd) break;
      const double2* tv = reinterpret_cast<const double2*>(r.tile[s]);
      int count = 0;
#pragma unroll 16
      for (int q = lane; q < kTile / 2; q += 32) {
        const double2 v = tv[q];
        count += f64emu::lt_zero(v.x) + f64emu::lt_zero(v.y);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) count += __shfl_xor_sync(0xffffffffu, count, off);
      if (lane == 0) ring::publish_aggregate(r, descs, s, tile, static_cast<long long>(count));
      __syncwarp();
      if (lane == 0) mbar_arrive(&r.summed[s]);
    }
  } else if (warp < kFirstCompute) {
    ring::look_back(r, descs, 0LL, hdr, warp - kFirstLookback);
  } else {
    // ---- compute: warp cw owns items [cw * 1024, cw * 1024 + 1024) of a tile,
    // row u = items 64u .. 64u + 63, lane L the pair 64u + 2L, +1 (consecutive
    // lanes read consecutive 16-byte words: conflict-free).  The group
    // decides together whether to go on, as in the scan (two flags, one per
    // barrier).  The stage is freed once its prefix has been read.
    const int ct = tid - 32 * kFirstCompute, cw = ct >> 5;
    const unsigned int below = (1u << lane) - 1u;
    volatile int* fail_loaded = &sm.fail_loaded;
    volatile int* fail_prefix = &sm.fail_prefix;
    for (int k = 0;; ++k) {
      const int s = k % kStages;
      const uint32_t par = (k / kStages) & 1;
      const bool loaded = ring::wait(r, &r.full[s], par, hdr);
      const unsigned int tile = r.ticket[s];
      if (!loaded) *fail_loaded = 1;
      unsigned int b0[kRows], b1[kRows];
      int wcount = 0;
      if (loaded && tile != kEnd) {
        const double2* tv = reinterpret_cast<const double2*>(r.tile[s] + cw * kSeg);
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          const double2 v = tv[u * 32 + lane];
          b0[u] = __ballot_sync(0xffffffffu, f64emu::lt_zero(v.x));
          b1[u] = __ballot_sync(0xffffffffu, f64emu::lt_zero(v.y));
          wcount += __popc(b0[u]) + __popc(b1[u]);
        }
      }
      if (lane == 0) sm.warp_count[cw] = wcount;
      named_sync(1, 32 * kComputeWarps);
      if (*fail_loaded || tile == kEnd) break;
      long long off = 0;
      for (int w = 0; w < cw; ++w) off += sm.warp_count[w];
      if (ring::wait(r, &r.prefix[s], par, hdr)) {
        off += r.excl[s];
        const int64_t seg = static_cast<int64_t>(tile) * kTile + cw * kSeg;
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          const int rank = __popc(b0[u] & below) + __popc(b1[u] & below);
          const bool s0 = (b0[u] >> lane) & 1u, s1 = (b1[u] >> lane) & 1u;
          const int32_t i = static_cast<int32_t>(seg + 64 * u + 2 * lane);
          if (s0) list[off + rank] = i;
          if (s1) list[off + rank + (s0 ? 1 : 0)] = i + 1;
          off += __popc(b0[u]) + __popc(b1[u]);
        }
        // the last tile knows the total
        if (ct == 0 && tile == tiles - 1u) *len = r.excl[s] + r.agg[s];
      } else {
        *fail_prefix = 1;
      }
      named_sync(2, 32 * kComputeWarps);
      if (*fail_prefix) break;
      if (ct == 0) mbar_arrive(&r.empty[s]);
    }
  }

  __syncthreads();
  if (tid == 0) ring::drain(r);
}

}  // namespace ilpipe

}  // namespace

extern "C" {

size_t b200_indexlist_workspace_bytes(int64_t n) {
  // one descriptor per 4096-item tile: enough for either kernel
  return 256 + static_cast<size_t>(ceil_div(n > 0 ? n : 1, ilpipe::kTile)) * sizeof(TileDesc);
}

int b200_basic_indexlist(const double* x, int32_t* list, int64_t n, int64_t* len,
                         void* workspace, size_t workspace_bytes, const b200_tune* tune,
                         b200_stream_t stream) {
  if (n < 0 || !len || (n > 0 && (!x || !list)))
    return invalid("b200_basic_indexlist: bad args");
  if (n > 0x7fffffffLL) return invalid("b200_basic_indexlist: n exceeds the int32 list range");
  const size_t need = b200_indexlist_workspace_bytes(n);
  if (workspace && !aligned16(workspace))
    return invalid("b200_basic_indexlist: workspace not 16-byte aligned");
  if (!workspace || workspace_bytes < need) {
    set_error("b200_basic_indexlist: workspace %zu bytes, need %zu", workspace_bytes, need);
    return B200_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    const cudaError_t e = cudaMemsetAsync(len, 0, sizeof(int64_t), st);
    if (e != cudaSuccess) {
      set_error("b200_basic_indexlist: %s", cudaGetErrorString(e));
      return B200_ERR_LAUNCH;
    }
    return B200_OK;
  }
  char* w = static_cast<char*>(workspace);
  ScanHeader* hdr = reinterpret_cast<ScanHeader*>(w);
  TileDesc* descs = reinterpret_cast<TileDesc*>(w + 256);
  const int algo = tune ? tune->algo : 0;
  if (algo != 0 && algo != 1) return invalid("b200_basic_indexlist: algo %d (0 or 1)", algo);
  const bool vec = aligned16(x) && !(tune && tune->vec == 1);
  const uint64_t lim = wait_limit_ns(tune, kDefaultWaitNs);
  if (algo == 0 && vec) {
    constexpr size_t kSmem = sizeof(ilpipe::Smem) + 128;
    const int rc = allow_dynamic_smem(reinterpret_cast<const void*>(ilpipe::indexlist_pipelined),
                                      kSmem, "b200_basic_indexlist");
    if (rc != B200_OK) return rc;
    const int64_t tiles = ceil_div(n, ilpipe::kTile);
    const int grid = static_cast<int>(std::min<int64_t>(tiles, device_info().sm_count));
    ilpipe::indexlist_pipelined<<<grid, ilpipe::kThreads, kSmem, st>>>(
        x, list, n, len, static_cast<unsigned int>(tiles), hdr, descs, lim);
    return after_launch("b200_basic_indexlist");
  }
  const unsigned tiles = static_cast<unsigned>(tiles_of(n));
  if (vec)
    indexlist_kernel<true><<<tiles, kBlock, 0, st>>>(x, list, n, len, hdr, descs, lim);
  else
    indexlist_kernel<false><<<tiles, kBlock, 0, st>>>(x, list, n, len, hdr, descs, lim);
  return after_launch("b200_basic_indexlist");
}

}  // extern "C"
