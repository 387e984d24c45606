// Single-pass decoupled lookback (shared by SCAN and INDEXLIST).
//
// Each launch takes tile ids from a counter, so a CTA only waits on tiles
// owned by CTAs that are already running.  A tile publishes its aggregate
// (AGG) as soon as it has reduced its own items, and its inclusive prefix
// (INC) once it knows its exclusive prefix; a successor sums predecessors'
// values back to the nearest INC.  Statuses carry the launch epoch, so the
// workspace is never re-zeroed between calls: the last CTA of a launch resets
// the counters and advances the epoch.  Every wait is bounded; one that gives
// up sets the header's error word and the call's results are invalid.
#pragma once

#include <cstdint>
#include <cstring>

namespace b200 {

constexpr int kLookbackPerLane = 4;   // a lookback round covers 128 predecessors
constexpr long long kSpinLimit = 1LL << 22;

struct ScanHeader {
  unsigned long long epoch;
  unsigned int tile_counter;
  unsigned int done_counter;
  unsigned int error;   // byte offset 16
  unsigned int pad[59];
};
static_assert(sizeof(ScanHeader) == 256, "lookback header is 256 bytes");

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


// Thread 0 takes the CTA's tile id and reads the launch epoch.
__device__ __forceinline__ void take_tile(ScanHeader* hdr, unsigned int* s_tile,
                                          unsigned long long* s_epoch) {
  if (threadIdx.x == 0) {
    *s_epoch = *reinterpret_cast<volatile unsigned long long*>(&hdr->epoch);
    *s_tile = atomicAdd(&hdr->tile_counter, 1u);
  }
  __syncthreads();
}

// Called by every thread of the CTA after its last use of the tile: the last
// CTA of the launch resets the counters and advances the epoch.
__device__ __forceinline__ void finish_launch(ScanHeader* hdr, unsigned long long epoch,
                                              bool* s_last) {
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int prev = atomicAdd(&hdr->done_counter, 1u);
    *s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (*s_last && threadIdx.x == 0) {
    hdr->tile_counter = 0u;
    hdr->done_counter = 0u;
    __threadfence();
    *reinterpret_cast<volatile unsigned long long*>(&hdr->epoch) = epoch + 1;
  }
}

// Run by one full warp for tile > 0: the sum of the predecessors' values back
// to (and including) the nearest inclusive prefix.  A round examines
// 32 * kLookbackPerLane predecessors, nearest first (slot w = j * 32 + lane is
// predecessor p_hi - w); every lane issues its loads before waiting on any,
// and values are summed in a fixed order (slots per lane, then a lane tree).
template <typename T>
__device__ T lookback_exclusive(const TileDesc* descs, unsigned int tile,
                                unsigned long long AGG, unsigned long long INC,
                                ScanHeader* hdr) {
  const int lane = threadIdx.x & 31;
  T acc = T(0);
  int64_t p_hi = static_cast<int64_t>(tile) - 1;  // nearest unexamined predecessor
  for (;;) {
    unsigned long long f[kLookbackPerLane], bits[kLookbackPerLane];
    T v[kLookbackPerLane];
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
    int stop = 32 * kLookbackPerLane;  // nearest slot holding an inclusive prefix
#pragma unroll
    for (int j = kLookbackPerLane - 1; j >= 0; --j) {
      const unsigned int m = __ballot_sync(0xffffffffu, f[j] == INC);
      if (m) stop = j * 32 + __ffs(m) - 1;
    }
    T val = T(0);
#pragma unroll
    for (int j = 0; j < kLookbackPerLane; ++j)
      if (j * 32 + lane <= stop) val += v[j];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) val += __shfl_down_sync(0xffffffffu, val, off);
    acc += __shfl_sync(0xffffffffu, val, 0);
    if (stop < 32 * kLookbackPerLane) return acc;
    p_hi -= 32 * kLookbackPerLane;
  }
}

}  // namespace b200
