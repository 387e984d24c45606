// Single-pass decoupled lookback (shared by SCAN and INDEXLIST).
//
// Each launch takes tile ids from a counter, so a CTA only waits on tiles
// owned by CTAs that are already running.  A tile publishes its aggregate
// (AGG) as soon as it has reduced its own items, and its inclusive prefix
// (INC) once it knows its exclusive prefix; a successor sums predecessors'
// values back to the nearest INC.  Statuses carry the launch epoch, so the
// workspace is never re-zeroed between calls: the CTA that draws a launch's
// last ticket resets the ticket count and advances the epoch.  A status
// counts only when its epoch equals the launch's (so a wrapped epoch cannot
// make an old status look new).  Every wait is bounded; one that gives up
// sets the header's error word and the call's results are invalid.
#pragma once

#include <cstdint>
#include <cstring>

#include "b200_async.cuh"

namespace b200 {

constexpr int kLookbackPerLane = 4;   // a lookback round covers 128 predecessors
// Default limit of a bounded wait (b200_tune.wait_limit_us = 0).
constexpr uint64_t kDefaultWaitNs = 2000000000ull;  // 2 s

struct ScanHeader {
  // Low 32 bits: tickets taken in this launch; high 32 bits: the launch
  // epoch.  One 64-bit atomic hands a CTA its tile and the epoch together.
  unsigned long long ticket;
  unsigned long long unused;
  unsigned int error;   // byte offset 16
  unsigned int pad[59];
};
static_assert(sizeof(ScanHeader) == 256, "lookback header is 256 bytes");

// A tile's descriptor: {status, value} in one 16-byte word, read and written
// as single 128-bit accesses (PTX .b128), so a reader that sees a status also
// sees the value published with it; no other data is ordered by a
// descriptor, so relaxed accesses suffice and a lane's loads of several
// descriptors are in flight together.  status = epoch * 4 + (AGG 1 | INC 2),
// epoch < 2^32.
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

// A descriptor status belongs to this launch (AGG or INC of its epoch).
__device__ __forceinline__ bool published(unsigned long long st, unsigned long long AGG,
                                          unsigned long long INC) {
  return st == AGG || st == INC;
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

// Thread 0 takes the CTA's tile id and the launch epoch with one atomic.
// The CTA that draws the launch's last ticket (gridDim.x - 1) knows every
// other CTA has drawn its own, so it clears the ticket count and advances the
// epoch in the same word right away; the next launch on the stream starts
// only after this one has finished.  No CTA has to wait for the others to
// finish, and no per-call reset of the workspace is needed.
__device__ __forceinline__ void take_tile(ScanHeader* hdr, unsigned int* s_tile,
                                          unsigned long long* s_epoch) {
  if (threadIdx.x == 0) {
    const unsigned long long t = atomicAdd(&hdr->ticket, 1ull);
    const unsigned int tile = static_cast<unsigned int>(t);
    if (tile == gridDim.x - 1u)
      atomicAdd(&hdr->ticket, (1ull << 32) - static_cast<unsigned long long>(gridDim.x));
    *s_tile = tile;
    *s_epoch = t >> 32;
  }
  __syncthreads();
}

// Run by one full warp for tile > 0: the sum of the predecessors' values back
// to (and including) the nearest inclusive prefix.  A round loads the
// descriptors of 32 * PER_LANE predecessors, nearest first (slot w = j * 32 +
// lane is predecessor p_hi - w), all at once.  Only slots nearer than the
// nearest inclusive prefix matter; those still unpublished are re-read
// together (one memory round trip per retry, however many are late) until
// every one has at least its aggregate.  Values are summed in a fixed order
// (slots per lane, then a lane tree).  A slot that stays unpublished for
// longer than limit_ns (%globaltimer, from the first retry of the call)
// records the error and counts as an inclusive prefix of 0.
template <typename T, int PER_LANE = kLookbackPerLane>
__device__ T lookback_exclusive(const TileDesc* descs, unsigned int tile,
                                unsigned long long AGG, unsigned long long INC,
                                ScanHeader* hdr, uint64_t limit_ns) {
  const int lane = threadIdx.x & 31;
  T acc = T(0);
  int64_t p_hi = static_cast<int64_t>(tile) - 1;  // nearest unexamined predecessor
  uint64_t t0 = 0;                                 // time of the first retry
  for (;;) {
    unsigned long long f[PER_LANE], bits[PER_LANE];
#pragma unroll
    for (int j = 0; j < PER_LANE; ++j) {
      const int64_t p = p_hi - (j * 32 + lane);
      f[j] = INC;                                  // p < 0: end of the lookback
      bits[j] = 0ull;
      if (p >= 0) desc_load(descs + p, f[j], bits[j]);
    }
    int stop;
    for (long long spins = 0;; ++spins) {
      stop = 32 * PER_LANE;  // nearest slot holding an inclusive prefix
#pragma unroll
      for (int j = PER_LANE - 1; j >= 0; --j) {
        const unsigned int m = __ballot_sync(0xffffffffu, f[j] == INC);
        if (m) stop = j * 32 + __ffs(m) - 1;
      }
      bool pending = false;
#pragma unroll
      for (int j = 0; j < PER_LANE; ++j)
        pending |= (j * 32 + lane < stop) && !published(f[j], AGG, INC);
      if (!__any_sync(0xffffffffu, pending)) break;
      // lane 0's clock decides for the warp
      uint64_t now = 0;
      if (lane == 0) now = globaltimer();
      now = __shfl_sync(0xffffffffu, now, 0);
      if (t0 == 0) t0 = now;
      const bool give_up = now - t0 > limit_ns;
      if (give_up && lane == 0) atomicExch(&hdr->error, 1u);
      if (spins > 16) __nanosleep(64);
#pragma unroll
      for (int j = 0; j < PER_LANE; ++j) {
        if ((j * 32 + lane < stop) && !published(f[j], AGG, INC)) {
          if (give_up) {
            f[j] = INC;
            bits[j] = 0ull;
          } else {
            desc_load(descs + (p_hi - (j * 32 + lane)), f[j], bits[j]);
          }
        }
      }
    }
    T val = T(0);
#pragma unroll
    for (int j = 0; j < PER_LANE; ++j)
      if (j * 32 + lane <= stop) val += from_bits<T>(bits[j]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) val += __shfl_down_sync(0xffffffffu, val, off);
    acc += __shfl_sync(0xffffffffu, val, 0);
    if (stop < 32 * PER_LANE) return acc;
    p_hi -= 32 * PER_LANE;
  }
}

}  // namespace b200
