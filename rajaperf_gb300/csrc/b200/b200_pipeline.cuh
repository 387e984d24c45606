// The stage ring of SCAN's persistent single-pass lookback kernel: one CTA
// per SM streams tiles of 4096 items of a 1-D array through seven
// shared-memory stages.  This header holds the ring's layout and bounded
// waits, the producer warp (draws tile ids, issues one bulk copy per tile)
// and the lookback warps (walk back to the nearest inclusive prefix, publish
// the tile's own); the kernel adds an aggregator warp (publishes a tile's
// aggregate as soon as it lands), its compute warps, and the role that frees
// a stage.  INDEXLIST's persistent kernel (indexlist.cu) keeps its own slots
// and roles and shares the bounded wait and the aggregate's publication.
//
// Per stage s, mbarriers with one arrival each link the roles:
//   drawn[s]  producer -> lookback      the stage's tile id is set
//   full[s]   producer (TMA) -> all     the tile's items have landed
//   summed[s] aggregator -> lookback    the tile's aggregate is in agg[s]
//   prefix[s] lookback -> compute       its exclusive prefix is in excl[s]
//   empty[s]  kernel -> producer        the stage may be refilled
// A tile id is drawn only once its stage is free: an id held while waiting
// would delay that tile's aggregate and stall its successors' lookback.
// A parity wait for phase p of a barrier passes at once while phase p-1 is
// still open, so a warp that takes alternate tiles (k, k + W, ...) must know
// that stage s's previous tile is done before waiting on s: drawn[s] gives
// that (the producer draws in order and refills a stage only after its
// tile is done), so such a warp waits on drawn[s] before any other barrier
// of stage s.  full[s] alone does not: bulk copies can complete out of order.  After
// the last tile the producer places one end marker (tile id kEnd) per warp of
// the role with the most warps taking alternate tiles.  Every wait is bounded (Ring::limit_ns); one that gives up sets the
// workspace error word and stops every role of the CTA.
#pragma once

#include <cstdint>

#include "b200_async.cuh"
#include "b200_lookback.cuh"

namespace b200 {
namespace ring {

constexpr int kTile = 4096;                  // items per tile
constexpr int kStages = 7;
constexpr int kLookbackWarps = 2;
constexpr int kLookbackLanes = 8;            // 256 predecessors per lookback round
constexpr unsigned int kEnd = 0xffffffffu;   // end marker in ticket[]

template <typename In, typename Acc>
struct Ring {
  using AccT = Acc;
  In tile[kStages][kTile];
  Acc agg[kStages];
  Acc excl[kStages];
  unsigned int ticket[kStages];
  unsigned int phases[kStages];  // full-barrier phases started per stage
  uint64_t drawn[kStages];
  uint64_t full[kStages];
  uint64_t summed[kStages];
  uint64_t prefix[kStages];
  uint64_t empty[kStages];
  unsigned long long epoch;
  uint64_t limit_ns;  // limit of every bounded wait of the launch
  int abort;
};

// Thread 0, before the CTA's first barrier.
template <typename In, typename Acc>
__device__ __forceinline__ void init(Ring<In, Acc>& r, uint64_t limit_ns) {
  for (int s = 0; s < kStages; ++s) {
    mbar_init(&r.drawn[s], 1);
    mbar_init(&r.full[s], 1);
    mbar_init(&r.summed[s], 1);
    mbar_init(&r.prefix[s], 1);
    mbar_init(&r.empty[s], 1);
    r.phases[s] = 0u;
  }
  r.limit_ns = limit_ns;
  r.abort = 0;
}

// Bounded wait by a whole warp; the result is the same in every lane (a lane
// that gave up fails the warp).  On expiry records the error and stops every
// role of the CTA.  R: a Ring, or any struct with its limit_ns and abort.
template <class R>
__device__ __forceinline__ bool wait(R& r, uint64_t* bar, uint32_t parity, ScanHeader* hdr) {
  const bool ok = __all_sync(0xffffffffu, mbar_wait_for(bar, parity, r.limit_ns));
  if (!ok && (threadIdx.x & 31) == 0) {
    atomicExch(&hdr->error, 1u);
    *reinterpret_cast<volatile int*>(&r.abort) = 1;
  }
  return ok;
}

// Warp 0: for k = 0, 1, ... waits for stage k mod kStages to be free, draws
// the next tile id and fills the stage with one bulk copy (the ragged last
// tile with plain loads, zero-filled), then places `end_markers` end markers
// (at least the number of warps of any role that takes alternate tiles, and
// fewer than kStages).  The CTA
// that draws the launch's last ticket (tiles + gridDim.x draws: every CTA
// draws exactly one id past the end) resets the count and advances the epoch.
template <typename In, typename Acc>
__device__ void produce(Ring<In, Acc>& r, const In* __restrict__ x, int64_t n,
                        unsigned int tiles, ScanHeader* hdr, int end_markers = kLookbackWarps) {
  const int lane = threadIdx.x & 31;
  const unsigned long long draws = static_cast<unsigned long long>(tiles) + gridDim.x;
  volatile int* abort_flag = &r.abort;
  int ends = 0;
  for (int k = 0; ends < end_markers && !__any_sync(0xffffffffu, *abort_flag); ++k) {
    const int s = k % kStages;
    if (k >= kStages && !wait(r, &r.empty[s], ((k / kStages) - 1) & 1, hdr)) break;
    unsigned int tile = kEnd;
    if (ends == 0) {
      unsigned long long t = 0;
      if (lane == 0) {
        t = atomicAdd(&hdr->ticket, 1ull);
        if (static_cast<unsigned int>(t) == draws - 1)
          atomicAdd(&hdr->ticket, (1ull << 32) - draws);
      }
      t = __shfl_sync(0xffffffffu, t, 0);
      if (k == 0 && lane == 0) r.epoch = t >> 32;
      if (static_cast<unsigned int>(t) < tiles) tile = static_cast<unsigned int>(t);
    }
    if (lane == 0) {
      r.ticket[s] = tile;
      mbar_arrive(&r.drawn[s]);
    }
    if (tile == kEnd) {  // end markers in consecutive stages, one per warp of a role
      ++ends;
      __syncwarp();
      if (lane == 0) {
        ++r.phases[s];
        mbar_arrive(&r.full[s]);
      }
      continue;
    }
    const int64_t base = static_cast<int64_t>(tile) * kTile;
    if (base + kTile <= n) {
      if (lane == 0) {
        ++r.phases[s];
        mbar_arrive_expect_tx(&r.full[s], kTile * sizeof(In));
        bulk_load(r.tile[s], x + base, kTile * sizeof(In), &r.full[s]);
      }
    } else {
      for (int i = lane; i < kTile; i += 32) r.tile[s][i] = (base + i < n) ? x[base + i] : In(0);
      __syncwarp();
      if (lane == 0) {
        ++r.phases[s];
        mbar_arrive(&r.full[s]);
      }
    }
  }
}

// Lookback warp lw (0 .. kLookbackWarps-1) takes tiles k = lw, lw + W, ...:
// starts when the tile id is drawn, walks back to the nearest inclusive
// prefix, then, with the tile's aggregate, publishes its inclusive prefix and
// hands the exclusive prefix to the compute warps.
template <typename In, typename Acc>
__device__ void look_back(Ring<In, Acc>& r, TileDesc* descs, Acc init, ScanHeader* hdr,
                          int lw) {
  const int lane = threadIdx.x & 31;
  for (int k = lw;; k += kLookbackWarps) {
    const int s = k % kStages;
    const uint32_t par = (k / kStages) & 1;
    if (!wait(r, &r.drawn[s], par, hdr)) break;
    const unsigned int tile = r.ticket[s];
    if (tile == kEnd) break;
    const unsigned long long AGG = r.epoch * 4 + 1, INC = r.epoch * 4 + 2;
    const Acc excl =
        (tile > 0) ? lookback_exclusive<Acc, kLookbackLanes>(descs, tile, AGG, INC, hdr,
                                                             r.limit_ns)
                   : init;
    if (!wait(r, &r.summed[s], par, hdr)) break;
    if (lane == 0) {
      desc_store(descs + tile, INC, to_bits<Acc>(excl + r.agg[s]));
      r.excl[s] = excl;
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&r.prefix[s]);
  }
}

// The aggregator's publish step (lane 0): the tile's aggregate, for tile 0
// only locally (its inclusive prefix comes from its lookback warp).  R: a
// Ring, or any struct with per-slot agg (of R::AccT) and the epoch.
template <class R>
__device__ __forceinline__ void publish_aggregate(R& r, TileDesc* descs, int s,
                                                  unsigned int tile, typename R::AccT total) {
  r.agg[s] = total;
  if (tile > 0) desc_store(descs + tile, r.epoch * 4 + 1, to_bits<typename R::AccT>(total));
}

// Thread 0 after the CTA's final barrier: after an abort, bulk copies may
// still be landing; wait (bounded) for the last phase started in each stage.
template <typename In, typename Acc>
__device__ __forceinline__ void drain(Ring<In, Acc>& r) {
  if (!r.abort) return;
  for (int s = 0; s < kStages; ++s)
    if (r.phases[s] > 0u) mbar_wait_for(&r.full[s], (r.phases[s] - 1u) & 1u, r.limit_ns);
}

}  // namespace ring
}  // namespace b200
