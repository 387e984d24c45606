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
// Default (x 16-byte aligned): a persistent form on bulk copies and the
// lookback warps of b200_pipeline.cuh (one CTA per SM).  Unlike SCAN it frees
// a tile's shared-memory stage as soon as the tile's items are ranked (their
// selection bits are all the list needs), so the stages keep loading while
// tiles wait for their base counts in small slots.  tune->algo = 1 (and an unaligned x) runs
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

// ---- persistent form: data stages and selection slots ------------------------
// INDEXLIST needs a tile's items only to select them: once the ballot warps
// have turned a tile into its selection bits (4096 bits, 512 bytes) the
// tile's shared-memory stage is refilled, and the tile waits for its base
// count in a small slot instead.  So the x stages stay busy loading while
// the lookback (the wait for every predecessor's count) is covered by many
// cheap slots: kData 32 KB stages, kSlots 512-byte slots.
//   warp 0                  producer: draws runs of four consecutive tile ids
//                           per atomic, one bulk copy per tile
//   warps 1-4               lookback: one global walk per run, the run's
//                           other base counts from its own tile counts
//   warps 5-12 (ballot)     two groups of four on alternate tiles: rank the
//                           tile's items in rows of 64 (two ballots per row),
//                           publish the tile's count, free the stage
//   warps 13-20 (writer)    two groups of four on alternate tiles: with the
//                           base count, write the selected indices to
//                           consecutive list entries, free the slot
// Measured per tile on GB300 (2^27 items, %globaltimer marks) with one
// lookback pair and four-warp groups: load 3.1 us, ballots 0.9 us, a walk
// 2.5 us, writes 1.3 us; two walks in flight per SM bounded the draw rate at
// 0.7 tiles per us per SM (60% of the copy peak), the four-warp groups close
// behind.  Each role now keeps two to four tiles in flight.
// Per slot b, one arrival each: drawn[b] (producer), summed[b] (ballot
// group), prefix[b] (lookback), empty[b] (writer group); per stage d: full[d]
// (bulk copy), data_empty[d] (ballot group).  The ballot and writer groups
// and the lookback warps take alternate tiles and wait on drawn[b] first (the
// ring's rule).
namespace ilpipe {

using ring::kEnd;
constexpr int kTile = ring::kTile;           // 4096 items
constexpr int kData = 6;                     // x stages (6 x 32 KB)
constexpr int kSlots = 24;                   // selection slots
constexpr int kGroups = 2;                   // ballot groups, and writer groups (alternate tiles)
constexpr int kGroupWarps = 4;               // warps per group
constexpr int kSeg = kTile / kGroupWarps;    // 1024 items per warp
constexpr int kRows = kSeg / 64;             // 16 rows of 64 items (a lane holds a pair)
constexpr int kLookbackWarps = 4;            // runs in flight per SM
constexpr int kDraw = 4;                     // tile ids per draw: a run
constexpr int kEnds = kDraw * kLookbackWarps;  // end markers
constexpr int kFirstLookback = 1;
constexpr int kFirstBallot = kFirstLookback + kLookbackWarps;
constexpr int kFirstWriter = kFirstBallot + kGroups * kGroupWarps;
constexpr int kThreads = 32 * (kFirstWriter + kGroups * kGroupWarps);
static_assert(kGroups < kData && kGroups < kSlots, "alternate-tile groups see phases in order");
static_assert(kGroups <= kEnds, "every group meets an end marker");
static_assert(kEnds + kDraw < kSlots, "end markers fit in the slots");
static_assert(kRows <= 32, "a lane holds one row's ballots");

// Per-slot state of the tiles between their draw and their list writes
// (with the ring's limit_ns and abort, for ring::wait and
// ring::publish_aggregate).
struct Slots {
  using AccT = long long;
  long long agg[kSlots];
  long long excl[kSlots];
  unsigned int ticket[kSlots];
  uint64_t drawn[kSlots];
  uint64_t summed[kSlots];
  uint64_t prefix[kSlots];
  uint64_t empty[kSlots];
  unsigned long long epoch;
  uint64_t limit_ns;
  int abort;
};

struct Smem {
  double tile[kData][kTile];
  uint2 bits[kSlots][kGroupWarps][kRows];    // (even, odd) item ballots per row
  int wcount[kSlots][kGroupWarps];
  uint64_t full[kData];
  uint64_t data_empty[kData];
  unsigned int phases[kData];                // full-barrier phases started per stage
  Slots r;
  int fail_ballot[kGroups];  // per ballot group: a wait gave up
  int fail_writer[kGroups];  // per writer group: a wait gave up
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
  Slots& r = sm.r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (tid == 0) {
    for (int b = 0; b < kSlots; ++b) {
      mbar_init(&r.drawn[b], 1);
      mbar_init(&r.summed[b], 1);
      mbar_init(&r.prefix[b], 1);
      mbar_init(&r.empty[b], 1);
    }
    for (int d = 0; d < kData; ++d) {
      mbar_init(&sm.full[d], 1);
      mbar_init(&sm.data_empty[d], 1);
      sm.phases[d] = 0u;
    }
    r.limit_ns = limit_ns;
    r.abort = 0;
    for (int g = 0; g < kGroups; ++g) sm.fail_ballot[g] = sm.fail_writer[g] = 0;
    mbar_init_fence();
  }
  __syncthreads();

  if (warp == 0) {
    // ---- producer: tile k takes slot k % kSlots and stage k % kData.  One
    // atomic draws a run of kDraw consecutive tile ids once their slots are
    // free (a round trip to the ticket counter per tile bounded the CTA's
    // tile rate, and a run needs one global lookback, not kDraw); each tile's
    // bulk copy is issued as soon as its stage is free.  A CTA stops at the
    // first draw that reaches the end: floor(tiles / kDraw) draws stop no
    // CTA, so the launch makes floor(tiles / kDraw) + gridDim.x draws and the
    // CTA making the last one resets the count and advances the epoch.  Ids
    // past the end are end markers, then more, kEnds in all, so that every
    // lookback warp's next run starts with one; end markers take no stage.
    const unsigned long long draws = tiles / kDraw + gridDim.x;
    volatile int* abort_flag = &r.abort;
    int ends = 0;
    for (int k = 0; ends < kEnds && !__any_sync(0xffffffffu, *abort_flag);) {
      const int batch = (ends == 0) ? kDraw : 1;
      bool ok = true;
      for (int j = 0; ok && j < batch; ++j) {
        const int kk = k + j;
        if (kk >= kSlots)
          ok = ring::wait(r, &r.empty[kk % kSlots], ((kk / kSlots) - 1) & 1, hdr);
      }
      if (!ok) break;
      unsigned int first = kEnd;
      if (ends == 0) {
        unsigned long long t = 0;
        if (lane == 0) {
          t = atomicAdd(&hdr->ticket, static_cast<unsigned long long>(kDraw));
          if (static_cast<unsigned int>(t) == kDraw * (draws - 1))
            atomicAdd(&hdr->ticket, (1ull << 32) - kDraw * draws);
        }
        t = __shfl_sync(0xffffffffu, t, 0);
        if (k == 0 && lane == 0) r.epoch = t >> 32;
        first = static_cast<unsigned int>(t);
      }
      const bool drawing = ends == 0;
      if (lane == 0)
        for (int j = 0; j < batch; ++j) {
          const int b = (k + j) % kSlots;
          r.ticket[b] = (drawing && first + j < tiles) ? first + static_cast<unsigned int>(j)
                                                       : kEnd;
          mbar_arrive(&r.drawn[b]);
        }
      for (int j = 0; ok && j < batch; ++j, ++k) {
        const int d = k % kData;
        const unsigned int tile =
            (drawing && first + j < tiles) ? first + static_cast<unsigned int>(j) : kEnd;
        if (tile == kEnd) {
          ++ends;
          continue;
        }
        if (k >= kData && !ring::wait(r, &sm.data_empty[d], ((k / kData) - 1) & 1, hdr)) {
          ok = false;
          break;
        }
        const int64_t base = static_cast<int64_t>(tile) * kTile;
        if (base + kTile <= n) {
          if (lane == 0) {
            ++sm.phases[d];
            mbar_arrive_expect_tx(&sm.full[d], kTile * sizeof(double));
            bulk_load(sm.tile[d], x + base, kTile * sizeof(double), &sm.full[d]);
          }
        } else {  // the ragged last tile: plain loads, zero-filled (0 is not < 0)
          for (int i = lane; i < kTile; i += 32)
            sm.tile[d][i] = (base + i < n) ? x[base + i] : 0.0;
          __syncwarp();
          if (lane == 0) {
            ++sm.phases[d];
            mbar_arrive(&sm.full[d]);
          }
        }
      }
      if (!ok) break;
    }
  } else if (warp < kFirstBallot) {
    // ---- lookback: warp lw takes the runs q = lw, lw + W, ...  (run q = the
    // CTA's tiles q kDraw .. q kDraw + kDraw - 1, consecutive ids).  One
    // global walk gives the run's first tile its exclusive count; each next
    // tile's is the previous one's plus that tile's count (no global walk).
    // Every tile's inclusive count is published as soon as it is known.
    const int lw = warp - kFirstLookback;
    bool done = false;
    for (int q = lw; !done; q += kLookbackWarps) {
      long long excl = 0;
      for (int i = 0; i < kDraw; ++i) {
        const int k = q * kDraw + i, b = k % kSlots;
        const uint32_t par = (k / kSlots) & 1;
        if (!ring::wait(r, &r.drawn[b], par, hdr)) {
          done = true;
          break;
        }
        const unsigned int tile = r.ticket[b];
        if (tile == kEnd) {
          done = true;
          break;
        }
        const unsigned long long AGG = r.epoch * 4 + 1, INC = r.epoch * 4 + 2;
        if (i == 0 && tile > 0)
          excl = lookback_exclusive<long long, ring::kLookbackLanes>(descs, tile, AGG, INC, hdr,
                                                                     r.limit_ns);
        if (!ring::wait(r, &r.summed[b], par, hdr)) {
          done = true;
          break;
        }
        if (lane == 0) {
          desc_store(descs + tile, INC, to_bits<long long>(excl + r.agg[b]));
          r.excl[b] = excl;
        }
        excl += r.agg[b];
        __syncwarp();
        if (lane == 0) mbar_arrive(&r.prefix[b]);
      }
    }
  } else if (warp < kFirstWriter) {
    // ---- ballot group: warp cw owns items [cw * kSeg, cw * kSeg + kSeg) of a
    // tile; row u = items 64u .. 64u + 63, lane L the pair 64u + 2L, +1
    // (consecutive lanes read consecutive 16-byte words: conflict-free).
    // Lane u keeps row u's two ballots and stores them to the slot.
    const int gid = (warp - kFirstBallot) / kGroupWarps;
    const int ct = tid - 32 * (kFirstBallot + gid * kGroupWarps), cw = ct >> 5;
    volatile int* fail = &sm.fail_ballot[gid];
    for (int k = gid;; k += kGroups) {
      const int b = k % kSlots, d = k % kData;
      bool ok = ring::wait(r, &r.drawn[b], (k / kSlots) & 1, hdr);
      const unsigned int tile = ok ? r.ticket[b] : kEnd;
      if (ok && tile != kEnd) ok = ring::wait(r, &sm.full[d], (k / kData) & 1, hdr);
      if (!ok) *fail = 1;
      if (ok && tile != kEnd) {
        const double2* tv = reinterpret_cast<const double2*>(sm.tile[d] + cw * kSeg);
        uint2 mine = make_uint2(0u, 0u);
        int wcount = 0;
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          const double2 v = tv[u * 32 + lane];
          const unsigned int b0 = __ballot_sync(0xffffffffu, f64emu::lt_zero(v.x));
          const unsigned int b1 = __ballot_sync(0xffffffffu, f64emu::lt_zero(v.y));
          if (lane == u) mine = make_uint2(b0, b1);
          wcount += __popc(b0) + __popc(b1);
        }
        if (lane < kRows) sm.bits[b][cw][lane] = mine;
        if (lane == 0) sm.wcount[b][cw] = wcount;
      }
      named_sync(1 + gid, 32 * kGroupWarps);
      if (*fail || tile == kEnd) break;
      if (ct == 0) {
        mbar_arrive(&sm.data_empty[d]);  // the stage is read: refill it
        long long total = 0;
#pragma unroll
        for (int w = 0; w < kGroupWarps; ++w) total += sm.wcount[b][w];
        ring::publish_aggregate(r, descs, b, tile, total);
        mbar_arrive(&r.summed[b]);
      }
    }
  } else {
    // ---- writer group: warp cw writes the indices of its kSeg items in row
    // order; a row's selected items take consecutive entries (ranks from the
    // two ballots), so a warp's stores cover consecutive list words.
    const int gid = (warp - kFirstWriter) / kGroupWarps;
    const int ct = tid - 32 * (kFirstWriter + gid * kGroupWarps), cw = ct >> 5;
    const unsigned int below = (1u << lane) - 1u;
    volatile int* fail = &sm.fail_writer[gid];
    for (int k = gid;; k += kGroups) {
      const int b = k % kSlots;
      const uint32_t par = (k / kSlots) & 1;
      bool ok = ring::wait(r, &r.drawn[b], par, hdr);
      const unsigned int tile = ok ? r.ticket[b] : kEnd;
      if (ok && tile != kEnd) ok = ring::wait(r, &r.prefix[b], par, hdr);
      if (!ok) *fail = 1;
      if (ok && tile != kEnd) {
        long long off = r.excl[b];
        for (int w = 0; w < cw; ++w) off += sm.wcount[b][w];
        const int64_t seg = static_cast<int64_t>(tile) * kTile + cw * kSeg;
#pragma unroll 4
        for (int u = 0; u < kRows; ++u) {
          const uint2 bb = sm.bits[b][cw][u];  // broadcast read
          const int rank = __popc(bb.x & below) + __popc(bb.y & below);
          const bool s0 = (bb.x >> lane) & 1u, s1 = (bb.y >> lane) & 1u;
          const int32_t i = static_cast<int32_t>(seg + 64 * u + 2 * lane);
          if (s0) list[off + rank] = i;
          if (s1) list[off + rank + (s0 ? 1 : 0)] = i + 1;
          off += __popc(bb.x) + __popc(bb.y);
        }
        // the last tile knows the total
        if (ct == 0 && tile == tiles - 1u) *len = r.excl[b] + r.agg[b];
      }
      named_sync(1 + kGroups + gid, 32 * kGroupWarps);
      if (*fail || tile == kEnd) break;
      if (ct == 0) mbar_arrive(&r.empty[b]);
    }
  }

  __syncthreads();
  // after an abort, bulk copies may still be landing: wait (bounded) for the
  // last phase started in each stage
  if (tid == 0 && r.abort)
    for (int d = 0; d < kData; ++d)
      if (sm.phases[d] > 0u) mbar_wait_for(&sm.full[d], (sm.phases[d] - 1u) & 1u, r.limit_ns);
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
