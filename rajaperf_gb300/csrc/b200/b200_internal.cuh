// Internal helpers shared by the libb200 translation units: error state,
// launch accounting, device properties and the grid-shape rules.
#pragma once

#include "b200.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

namespace b200 {

// ---- error state -----------------------------------------------------------

void set_error(const char* fmt, ...);
void clear_error();

// Records a failed argument check and returns B200_ERR_INVALID_ARG.
int invalid(const char* fmt, ...);

// Records an unsupported device or configuration; returns B200_ERR_UNSUPPORTED.
int unsupported(const char* fmt, ...);

// Checks the launch that was just issued and counts it.  Returns B200_OK or
// B200_ERR_LAUNCH with the CUDA error recorded.
int after_launch(const char* what, int nlaunches = 1);

// Raises `kernel`'s dynamic shared-memory limit to at least `bytes` on the
// current device; the attribute is set once per kernel and device (later
// calls are a map lookup).  Returns B200_OK or B200_ERR_LAUNCH (recorded).
int allow_dynamic_smem(const void* kernel, size_t bytes, const char* what);

// ---- device properties -----------------------------------------------------

struct DeviceInfo {
  int device = -1;
  int sm_count = 0;
  int cc_major = 0;
  int cc_minor = 0;
  size_t global_mem = 0;
  int l2_bytes = 0;
  int max_smem_optin = 0;
};

// Properties of the current device (cached per device id).
const DeviceInfo& device_info();

inline cudaStream_t as_stream(b200_stream_t s) {
  return reinterpret_cast<cudaStream_t>(s);
}

// ---- tuning ----------------------------------------------------------------

struct Shape {
  int block;   // threads per CTA
  int items;   // elements (or vectors) per thread per tile
  int vec;     // 1 or 2 doubles per access
  int grid;    // CTAs launched
};

// Resolves a tuning (NULL or partly zero) for a 1-D streaming kernel over
// `units` work items, where one tile covers block*items units.  The grid is
// one tile per CTA up to `max_grid` CTAs (0 = as many as tiles); kernels
// loop over any remaining tiles.
Shape resolve_1d(const b200_tune* t, int64_t units, int def_block,
                 int def_items, int def_vec, int64_t max_grid = 0);

// Limit of the bounded device-side waits of a call (b200_tune.wait_limit_us;
// 0 or negative = `def_ns`).
inline uint64_t wait_limit_ns(const b200_tune* t, uint64_t def_ns) {
  return (t && t->wait_limit_us > 0) ? static_cast<uint64_t>(t->wait_limit_us) * 1000ull
                                     : def_ns;
}

inline bool valid_block(int b) {
  return b == 64 || b == 128 || b == 256 || b == 512 || b == 1024;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

inline bool aligned16(const void* p) {
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

}  // namespace b200

// Dispatches a runtime block size onto a compile-time constant BS.
#define B200_DISPATCH_BLOCK(bs, BS, ...)                                      \
  switch (bs) {                                                               \
    case 64: { constexpr int BS = 64; __VA_ARGS__; } break;                   \
    case 128: { constexpr int BS = 128; __VA_ARGS__; } break;                 \
    case 512: { constexpr int BS = 512; __VA_ARGS__; } break;                 \
    case 1024: { constexpr int BS = 1024; __VA_ARGS__; } break;               \
    default: { constexpr int BS = 256; __VA_ARGS__; } break;                  \
  }

// Dispatches a runtime items-per-thread count onto a constant IT.
#define B200_DISPATCH_ITEMS(it, IT, ...)                                      \
  switch (it) {                                                               \
    case 1: { constexpr int IT = 1; __VA_ARGS__; } break;                     \
    case 2: { constexpr int IT = 2; __VA_ARGS__; } break;                     \
    case 8: { constexpr int IT = 8; __VA_ARGS__; } break;                     \
    default: { constexpr int IT = 4; __VA_ARGS__; } break;                    \
  }
