/*
 * b200.h -- C ABI of libb200, the sm_103a kernel library behind the
 * RAJA Performance Suite's Base_GB300 variant.
 *
 * Every entry point replaces the body of one reference kernel's Base_CUDA
 * rep loop (the launch inside "for irep < run_reps" of K-Cuda.cpp).  The
 * citations name the reference file:line whose semantics each call follows;
 * paths are relative to the RAJAPerf source tree (src/).
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller.
 *  - No call allocates, frees, synchronises or touches host memory, so every
 *    call can be captured into a CUDA graph.
 *  - Scalars are passed by value; reduction results are written to caller
 *    device memory.
 *  - Reductions and the scan take a caller-owned device workspace whose
 *    size comes from the matching *_workspace_bytes() query (two-phase, like
 *    CUB).  A workspace must be zero-filled once (cudaMemset) before its
 *    first use; each call leaves it ready for the next call.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).
 *  - `tune` may be NULL (library default tuning for the size).
 *  - Return value: B200_OK or a b200_status code; b200_last_error_string()
 *    describes the last failure on the calling host thread.
 *  - Thread-compatible: concurrent calls on different streams are fine;
 *    calls sharing a workspace must be ordered on one stream.
 */
#ifndef B200_H
#define B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* b200_stream_t; /* cudaStream_t */

typedef enum b200_status {
  B200_OK = 0,
  B200_ERR_INVALID_ARG = 1,  /* bad size, null pointer, bad tuning       */
  B200_ERR_LAUNCH = 2,       /* CUDA launch or runtime error              */
  B200_ERR_TIMEOUT = 3,      /* a bounded device-side wait gave up        */
  B200_ERR_WORKSPACE = 4,    /* workspace missing or too small            */
  B200_ERR_UNSUPPORTED = 5   /* device or configuration not supported     */
} b200_status;

/* Launch-shape tuning.  Zero fields take the library default.
 * block_size: threads per CTA.  items: elements per thread per tile.
 * vec: elements per vector memory access (1, 2).  grid_blocks: CTA count
 * cap (0 = one tile per CTA).  tile_*: stencil tile shape.  time_block:
 * stencil time steps fused per launch.  algo: kernel-specific algorithm
 * selector (documented per entry point). */
typedef struct b200_tune {
  int32_t block_size;
  int32_t items;
  int32_t vec;
  int32_t grid_blocks;
  int32_t tile_x;
  int32_t tile_y;
  int32_t tile_z;
  int32_t time_block;
  int32_t algo;
  int32_t reserved[3];
} b200_tune;

typedef struct b200_caps {
  int32_t device;
  int32_t sm_count;
  int32_t cc_major;
  int32_t cc_minor;
  int64_t global_mem_bytes;
  int64_t l2_bytes;
  int32_t max_smem_per_block_optin;
  int32_t reserved;
} b200_caps;

/* ---- library ------------------------------------------------------------ */

/* Last error message on this host thread ("" when none). */
const char* b200_last_error_string(void);

/* Properties of the current device, cached per device. */
int b200_device_caps(b200_caps* out);

/* Number of kernels this library has launched since it was loaded. */
int64_t b200_launch_count(void);

/* ---- data initialisation (DataUtils.cpp) -------------------------------- */

/* p[i] = factor*(i + 1.1)/(i + 1.12345)  -- common/DataUtils.cpp:504-513. */
int b200_init_reference(double* p, int64_t n, double factor,
                        b200_stream_t stream);

/* p[i] = sign[i]*factor*(i + 1.1)/(i + 1.12345) with sign[i] = +/-1 given as
 * int8 -- common/DataUtils.cpp:542-555 (signs come from the host's rand()). */
int b200_init_reference_signed(double* p, const int8_t* sign, int64_t n,
                               double factor, b200_stream_t stream);

/* p[i] = value  -- common/DataUtils.cpp:518-536. */
int b200_init_const(double* p, int64_t n, double value, b200_stream_t stream);
int b200_init_const_i64(int64_t* p, int64_t n, int64_t value,
                        b200_stream_t stream);

/* Seeded counter-based uniform values in [lo, hi):
 * p[i] = lo + (hi-lo) * (splitmix64(seed, stream_id, i) >> 11) * 2^-53.
 * Not in the reference; implements the uniform input mode. */
int b200_init_uniform(double* p, int64_t n, uint64_t seed, uint64_t stream_id,
                      double lo, double hi, b200_stream_t stream);

/* Seeded integers uniform in [lo, hi) from the same generator. */
int b200_init_uniform_i64(int64_t* p, int64_t n, uint64_t seed,
                          uint64_t stream_id, int64_t lo, int64_t hi,
                          b200_stream_t stream);

/* ---- Stream ------------------------------------------------------------- */

/* c[i] = a[i]                    -- stream/COPY.hpp:24, COPY-Cuda.cpp:26  */
int b200_stream_copy(const double* a, double* c, int64_t n,
                     const b200_tune* tune, b200_stream_t stream);

/* b[i] = alpha*c[i]              -- stream/MUL.hpp:25, MUL-Cuda.cpp:26    */
int b200_stream_mul(double* b, const double* c, double alpha, int64_t n,
                    const b200_tune* tune, b200_stream_t stream);

/* c[i] = a[i] + b[i]             -- stream/ADD.hpp:25, ADD-Cuda.cpp:27    */
int b200_stream_add(const double* a, const double* b, double* c, int64_t n,
                    const b200_tune* tune, b200_stream_t stream);

/* a[i] = b[i] + alpha*c[i]       -- stream/TRIAD.hpp:26, TRIAD-Cuda.cpp:24 */
int b200_stream_triad(double* a, const double* b, const double* c,
                      double alpha, int64_t n, const b200_tune* tune,
                      b200_stream_t stream);

/* Workspace for b200_stream_dot, b200_algorithm_reduce_sum and
 * b200_lcals_first_min on n elements. */
size_t b200_reduce_workspace_bytes(int64_t n, const b200_tune* tune);

/* *dot_accum += dot_init + sum_i a[i]*b[i]
 *   -- stream/DOT.hpp:24, DOT-Seq.cpp:34-47 (m_dot += dot per rep).
 * Deterministic fixed-shape tree: one pass of per-CTA partials, the last CTA
 * to finish sums the partials in CTA order.  One launch. */
int b200_stream_dot(const double* a, const double* b, int64_t n,
                    double dot_init, double* dot_accum, void* workspace,
                    size_t workspace_bytes, const b200_tune* tune,
                    b200_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* B200_H */
