/*
 * rajaperf_gb300.h -- C ABI of the Base_GB300 host layer.
 *
 * rp_run() runs the suite for a command line exactly as the rajaperf-gb300
 * driver does (the suite's RAJAPerfSuiteDriver.cpp:22-61 with the variant
 * Base_GB300) and returns one record per kernel and tuning: the suite's
 * checksum (common/DataUtils.cpp:600-621), rep-loop times and the kernel's
 * Bytes/rep and FLOPs/rep (common/KernelBase.hpp:215-225).  Command-line
 * options are those of the suite's RunParams (--size, --checkrun, -k, -t,
 * ...) plus the GB300 options listed by --help.  With --host-data the
 * kernels' arrays live in pinned host memory (the suite's CudaPinned data
 * space, --cuda-data-space in common/RunParams.cpp:907-957 of the suite) and
 * each rep's timed work includes moving its data across the host link.
 */
#ifndef RAJAPERF_GB300_H
#define RAJAPERF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { RP_OK = 0, RP_ERR_INPUT = 1, RP_ERR_RUN = 2 };

typedef struct rp_result {
  char kernel[64];
  char variant[32];
  char tuning[64];
  double checksum;           /* long double checksum rounded to double   */
  double checksum_residual;  /* checksum - (double)checksum              */
  double min_time_s;         /* rep-loop time, min over passes           */
  double avg_time_s;
  double max_time_s;
  int64_t reps;
  int64_t actual_size;
  int64_t its_per_rep;
  int64_t kernels_per_rep;
  int64_t bytes_per_rep;
  int64_t flops_per_rep;
  int32_t passes;
  int32_t failed;            /* nonzero when this kernel/tuning failed   */
  int64_t h2d_bytes_per_rep; /* --host-data: bytes a rep moves from host
                                memory to the device (copies, or the
                                kernel's own reads of host memory)      */
  int64_t d2h_bytes_per_rep; /* ... and back                            */
} rp_result;

typedef struct rp_batch_result {
  int32_t kernels;
  int32_t reserved;
  int64_t reps;
  int64_t launches_per_rep;
  double launch_time_s;       /* reps x kernels as individual launches     */
  double graph_time_s;        /* the same work as one CUDA graph with one
                                 branch per kernel (branches concurrent)    */
  double graph_serial_time_s; /* the same work as one CUDA graph holding a
                                 single chain in launch order               */
} rp_batch_result;

/* Last error on this host thread. */
const char* rp_last_error(void);

/* Runs the suite; fills up to `capacity` results and sets *count.
 * Returns RP_OK, RP_ERR_INPUT (bad command line) or RP_ERR_RUN (a kernel
 * failed; its record has failed != 0). */
int rp_run(int argc, const char* const* argv, rp_result* out, int capacity,
           int* count);

/* Runs the selected kernels' rep loops with --graph-batch semantics. */
int rp_graph_batch(int argc, const char* const* argv, rp_batch_result* out);

#ifdef __cplusplus
}
#endif

#endif /* RAJAPERF_GB300_H */
