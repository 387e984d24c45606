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
 * cap (0 = one tile per CTA).  tile_*: stencil tile shape, or, where an
 * entry point documents it, how many of a point's FP64 operations run in an
 * exact integer-pipe form (JACOBI_2D, HEAT_3D, HYDRO_2D, EOS,
 * DEL_DOT_VEC_2D: tile_z = 1 + count).  time_block:
 * stencil time steps fused per launch.  algo: kernel-specific algorithm
 * selector (documented per entry point).  wait_limit_us: limit of every
 * bounded device-side wait of the call (scan and index-list lookback and
 * stage waits, split-GEMM pipeline waits); 0 = the library default (2 s for
 * the scan and index list, 1 s for the split GEMM).  A wait that runs out
 * sets the workspace's error word, which b200_workspace_status() reports. */
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
  int32_t wait_limit_us;
  int32_t reserved[2];
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

/* Status of the calls that used a workspace with bounded device-side waits
 * (b200_algorithm_scan*, b200_basic_indexlist*, b200_gemm_split): waits for
 * `stream`, then reads the workspace's error word.  Returns B200_OK, or
 * B200_ERR_TIMEOUT when a wait of an earlier call on that workspace gave up
 * (its results are invalid); in that case the whole workspace is zero-filled
 * again (stream-ordered, then waited for), so it is ready for the next call.
 * The reference has no device-side waits to report: its Base_CUDA variants
 * check every CUDA call and abort on an error (common/CudaDataUtils.hpp:67).
 * This call synchronises the stream, unlike the kernel entry points. */
int b200_workspace_status(void* workspace, size_t workspace_bytes, b200_stream_t stream);

/* FP64 pipe probe: launches 16 independent fma chains of `iters` steps in
 * each of b200_probe_dfma_threads() threads (out must hold that many
 * doubles) and reports the number of fused multiply-adds issued.  Timing the
 * launch gives the device's FP64 FMA rate, the roofline of the FP64-bound
 * kernels.  Not in the reference. */
int64_t b200_probe_dfma_threads(void);
int b200_probe_dfma(double* out, int32_t iters, int64_t* fma_count,
                    b200_stream_t stream);

/* Self-test of the integer-pipe FP64 arithmetic used by the mixed-pipe
 * stencils and by the power-of-two scalings of DEL_DOT_VEC_2D and HEAT_3D:
 * n operand pairs from `seed` (arbitrary bit patterns, close and distant
 * exponents, range edges, [0.5, 1.5)), op 0 = add, 1 = sub, 2 = mul,
 * 3 = a * 0.5, 4 = a * 0.125, 5 = a * 2, 6 = a / b (the FP64-free division
 * of HYDRO_2D and DEL_DOT_VEC_2D, with quotients near rounding midpoints, near
 * 1 and extreme divisor significands added), 7 = a < 0 (INDEXLIST's
 * integer test; signed zeros, infinities and NaNs added), 8 = a * b on the
 * integer pipe (JACOBI_2D's a * 0.2 for every other pair), 9 = a + b for a b
 * below a's last bit (DEL_DOT_VEC_2D's + ptiny; exponent gaps 50-60 around
 * the fast path's bound of 55, powers of two, special values added), 10 =
 * a + b with close exponents (JACOBI_2D's integer-pipe adds: exponents 0-4
 * apart, mostly one sign, the top of the exponent range, zeros, subnormals
 * and non-finite values added), 11 = a + b of either sign with close
 * exponents (HEAT_3D's integer-pipe b(+1) - 2a: exponents 0-4 apart, b near
 * -a with differences of 0 to 53 bits, results below the normal range, the
 * top of the range, special values added), 12 = a * b + c on the integer
 * pipes (EOS's FMAs: positive operands, c 0 to 74 bits above the product's
 * last bit and a little past that window, products with low bits cleared for
 * near-ties, the top and bottom of the range, zeros, subnormals, negatives
 * and non-finite values added); adds to *mismatches (device) the number of
 * results whose bits differ from the FP64 pipe's.  Not in the reference. */
int b200_f64emu_selftest(int64_t n, uint64_t seed, int32_t op,
                         unsigned long long* mismatches, b200_stream_t stream);

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

/* The same dot product for callers that cannot allocate device memory where
 * they need it -- code whose device heap is owned by someone else (a
 * framework's caching allocator, a fixed arena) or a latency-critical loop
 * that must not pay cudaMalloc's implicit synchronisation.  No counterpart in
 * the reference.  The scratch is a library-owned __device__ array of
 * b200_stream_dot_static_max_scratch_bytes() bytes (room for 4096 CTAs),
 * held by every GPU that loads the library until the process exits; a launch
 * shape needing more returns B200_ERR_WORKSPACE.  The call allocates nothing
 * and clears the scratch counter itself.  All calls share the array, so
 * calls that overlap on the GPU race and must be ordered by the caller.  The
 * first call in a CUDA context looks the array's address up
 * (cudaGetSymbolAddress) and caches it under that context's unique id, so a
 * context created later (after a device reset, or a second context on the
 * device) gets its own lookup; that first call should come before any stream
 * capture that contains this call. */
size_t b200_stream_dot_static_max_scratch_bytes(void);
int b200_stream_dot_static(const double* a, const double* b, int64_t n,
                           double dot_init, double* dot_accum,
                           const b200_tune* tune, b200_stream_t stream);

/* ---- Basic (kernels of the batched small-size suite) --------------------- */

/* y[i] += a*x[i]                   -- basic/DAXPY.hpp, DAXPY-Cuda.cpp        */
int b200_basic_daxpy(double* y, const double* x, double a, int64_t n,
                     const b200_tune* tune, b200_stream_t stream);

/* out1 = out2 = out3 = -in1 - in2  -- basic/INIT3.hpp, INIT3-Cuda.cpp        */
int b200_basic_init3(double* out1, double* out2, double* out3, const double* in1,
                     const double* in2, int64_t n, const b200_tune* tune,
                     b200_stream_t stream);

/* out1 = in1*in2, out2 = in1+in2, out3 = in1-in2 -- basic/MULADDSUB.hpp      */
int b200_basic_muladdsub(double* out1, double* out2, double* out3,
                         const double* in1, const double* in2, int64_t n,
                         const b200_tune* tune, b200_stream_t stream);

/* ---- LCALS -------------------------------------------------------------- */

/* x[i] = q + y[i]*(r*z[i+10] + t*z[i+11]); z holds >= n+11 values
 *   -- lcals/HYDRO_1D.hpp:30, HYDRO_1D-Cuda.cpp:26                          */
int b200_lcals_hydro_1d(double* x, const double* y, const double* z, double q,
                        double r, double t, int64_t n, const b200_tune* tune,
                        b200_stream_t stream);

/* One rep of HYDRO_2D on a kn x jn row-major grid (index j + k*jn): BODY1
 * (za, zb) then BODY2 (zu, zv +=) and BODY3 (zrout, zzout) over the interior
 *   -- lcals/HYDRO_2D.hpp:66-90, HYDRO_2D-Cuda.cpp:104-140.  Two launches.
 * tune->tile_z - 1 of BODY2's eight differences (0, 2, 4, 6, 8; default 6)
 * run on the integer pipes (exact, bit-identical).                          */
int b200_lcals_hydro_2d(double* za, double* zb, const double* zm,
                        const double* zp, const double* zq, const double* zr,
                        double* zu, double* zv, const double* zz, double* zrout,
                        double* zzout, double s, double t, int64_t kn,
                        int64_t jn, const b200_tune* tune, b200_stream_t stream);

/* x[i] = EOS polynomial; y, z, u hold >= n+7 values
 *   -- lcals/EOS.hpp:33, EOS-Cuda.cpp:26
 * Default: tune->tile_z - 1 of each element's eight FMAs (1..3; default 2)
 * run on the integer pipes (exact a * b + c for positive operands,
 * bit-identical; other operands take the FP64 pipe), tune->items elements
 * per thread (1, 2, 4, 8; default 2), tune->block_size threads (128, 256,
 * 512; default 128).  tune->tile_z = 1, or another block size: the
 * element-map kernel, all eight FMAs on the FP64 pipe.                      */
int b200_lcals_eos(double* x, const double* y, const double* z, const double* u,
                   double q, double r, double t, int64_t n,
                   const b200_tune* tune, b200_stream_t stream);

/* x[i] = y[i+1] - y[i]             -- lcals/FIRST_DIFF.hpp:25                */
int b200_lcals_first_diff(double* x, const double* y, int64_t n,
                          const b200_tune* tune, b200_stream_t stream);

/* px[i] = 9-term predictor over planes px[i + k*n], k = 2..12 (px has 13n)
 *   -- lcals/INT_PREDICT.hpp:40, INT_PREDICT-Cuda.cpp:26                    */
int b200_lcals_int_predict(double* px, double dm22, double dm23, double dm24,
                           double dm25, double dm26, double dm27, double dm28,
                           double c0, int64_t n, const b200_tune* tune,
                           b200_stream_t stream);

/* First-index minimum: *minloc = smallest i with x[i] minimal (strict '<'
 * scan seeded with (xmin_init, initloc)); *minval (optional) = the minimum.
 * Workspace from b200_reduce_workspace_bytes.  One launch; exact.
 *   -- lcals/FIRST_MIN.hpp:29-54, FIRST_MIN-Seq.cpp:34-48                   */
int b200_lcals_first_min(const double* x, int64_t n, double xmin_init,
                         int64_t initloc, int64_t* minloc, double* minval,
                         void* workspace, size_t workspace_bytes,
                         const b200_tune* tune, b200_stream_t stream);

/* Divided-difference predictor over planes px[i + k*n], k = 4..13 (px has
 * 14n), in place   -- lcals/DIFF_PREDICT.hpp                               */
int b200_lcals_diff_predict(double* px, const double* cx, int64_t n,
                            const b200_tune* tune, b200_stream_t stream);

/* y[i] = u[i]/v[i]; w[i] = x[i]/(exp(y[i]) - 1)  -- lcals/PLANCKIAN.hpp     */
int b200_lcals_planckian(const double* x, double* y, const double* u,
                         const double* v, double* w, int64_t n,
                         const b200_tune* tune, b200_stream_t stream);

/* ---- Apps --------------------------------------------------------------- */

/* BODY1 and BODY2 of PRESSURE fused per element
 *   -- apps/PRESSURE.hpp:39-46, PRESSURE-Cuda.cpp:26,38                     */
int b200_apps_pressure(const double* compression, double* bvc, double* p_new,
                       const double* e_old, const double* vnewc, double cls,
                       double p_cut, double pmin, double eosvmax, int64_t n,
                       const b200_tune* tune, b200_stream_t stream);

/* BODY1..BODY6 of ENERGY fused per element
 *   -- apps/ENERGY.hpp:111-178, ENERGY-Cuda.cpp:26-182                      */
int b200_apps_energy(double* e_new, const double* e_old, const double* delvc,
                     const double* p_new, const double* p_old, double* q_new,
                     const double* q_old, const double* work,
                     const double* compHalfStep, const double* pHalfStep,
                     const double* bvc, const double* pbvc, const double* ql_old,
                     const double* qq_old, const double* vnewc, double rho0,
                     double e_cut, double emin, double q_cut, int64_t n,
                     const b200_tune* tune, b200_stream_t stream);

/* Hexahedron volumes for i in [ibegin, iend) from the 8 corners i + {0, 1,
 * jp, 1+jp, kp, 1+kp, jp+kp, 1+jp+kp}  -- apps/VOL3D.hpp:88-146,
 * VOL3D-Cuda.cpp:26-75                                                      */
int b200_apps_vol3d(const double* x, const double* y, const double* z,
                    double* vol, double vnormq, int64_t jp, int64_t kp,
                    int64_t ibegin, int64_t iend, const b200_tune* tune,
                    b200_stream_t stream);

/* Nodal divergence for each real zone i = real_zones[ii], corners i, i+1,
 * i+1+jp, i+jp  -- apps/DEL_DOT_VEC_2D.hpp:65-90, DEL_DOT_VEC_2D-Cuda.cpp:30-60
 * With half = 0.5 the halvings are exponent moves, the divisions and five
 * products integer-pipe arithmetic and the first add of six of the eight
 * corner sums integer-pipe adds, all bit-identical to the FP64 pipe;
 * tune->tile_z = 1 + corner sums opened on the integer pipes (0, 2, 4, 6 or 8;
 * default 6). */
int b200_apps_del_dot_vec_2d(const double* x, const double* y,
                             const double* xdot, const double* ydot,
                             double* div, const int64_t* real_zones,
                             int64_t n_real_zones, int64_t jp, double ptiny,
                             double half, const b200_tune* tune,
                             b200_stream_t stream);

/* ---- Polybench ---------------------------------------------------------- */

/* tsteps x (B <- 5-point average of A, then A <- of B) on an N x N grid
 *   -- polybench/POLYBENCH_JACOBI_2D.hpp:38-44, -Cuda.cpp:86-114
 * Default: column segments of tune->items rows per thread (2, 4 or 8;
 * default 4), the product by 0.2 and the first of each point's four adds on
 * the integer pipes (bit-identical: f64emu, exact rounding), the other three
 * adds on the FP64 pipe; tune->tile_z = 1 + integer-pipe adds per four
 * points (0, 4, 8, 9, 10 or 12; default 4), tune->tile_y 2 puts the product
 * on the FP64 pipe; tune->items 1: one point per
 * thread.  tune->algo > 0 selects the
 * mixed-pipe kernel: algo-1 of every 8 warps run bit-identical integer-pipe
 * FP64 (rows per warp: tile_y emulated, tile_z native).                     */
int b200_polybench_jacobi_2d(double* A, double* B, int64_t N, int64_t tsteps,
                             const b200_tune* tune, b200_stream_t stream);

/* tsteps x (B <- 7-point heat update of A, then A <- of B) on N^3
 *   -- polybench/POLYBENCH_HEAT_3D.hpp:47-82, -Cuda.cpp:97-113
 * Default: each thread walks tune->tile_x consecutive planes (2 or 4;
 * default 4) with the plane neighbours in registers; 2.0 * a and the three
 * 0.125 * (...) are exponent moves, and tune->tile_z - 1 of the six
 * differences b(+1) - 2a of every two planes (0..6; default 5) run on the
 * integer pipes (f64emu::sub_near_fast: exact rounding, bit-identical); the
 * remaining adds are FP64 FMAs.  tune->algo > 0 selects the mixed-pipe
 * kernel as for JACOBI_2D (tile_x = planes per CTA).                        */
int b200_polybench_heat_3d(double* A, double* B, int64_t N, int64_t tsteps,
                           const b200_tune* tune, b200_stream_t stream);

/* tsteps of the 2-D FDTD update on nx x ny (fict holds tsteps values)
 *   -- polybench/POLYBENCH_FDTD_2D.hpp:52-69, -Cuda.cpp:164-190             */
int b200_polybench_fdtd_2d(double* ex, double* ey, double* hz,
                           const double* fict, int64_t nx, int64_t ny,
                           int64_t tsteps, const b200_tune* tune,
                           b200_stream_t stream);

/* Workspace for b200_polybench_fdtd_2d_ws: two snapshots of the tile edges
 * (three rows per tile row and three columns per tile column; for 8-row
 * tiles about 0.8 of one nx x ny array). */
size_t b200_fdtd_2d_workspace_bytes(int64_t nx, int64_t ny);

/* The same tsteps of FDTD_2D with one launch per time step: every CTA
 * updates ex and ey (BODY1-3) and then hz (BODY4) of its tile of
 * tune->tile_y rows (8 by default, or 16, 32) x 128 columns in place, taking
 * the old values across tile edges from a snapshot of the edges in the
 * workspace (one extra small launch per call takes the first snapshot).
 * 48 bytes per point and step instead of 72; bit-identical to
 * b200_polybench_fdtd_2d.  tune->algo 1 runs b200_polybench_fdtd_2d instead
 * (no workspace needed).  The workspace needs no initialisation.
 *   -- polybench/POLYBENCH_FDTD_2D.hpp:52-69, -Cuda.cpp:164-190             */
int b200_polybench_fdtd_2d_ws(double* ex, double* ey, double* hz,
                              const double* fict, int64_t nx, int64_t ny,
                              int64_t tsteps, void* workspace,
                              size_t workspace_bytes, const b200_tune* tune,
                              b200_stream_t stream);

/* C[i][j] = sum_k (alpha*A[i][k]) * B[k][j], row-major, FP64 (the suite's
 * GEMM: its beta scaling is overwritten by BODY4)
 *   -- polybench/POLYBENCH_GEMM.hpp:40-56, -Cuda.cpp:27-59                  */
int b200_polybench_gemm(const double* A, const double* B, double* C, int64_t ni,
                        int64_t nj, int64_t nk, double alpha,
                        const b200_tune* tune, b200_stream_t stream);

/* E = A*B, F = C*D, G = E*F (FP64)
 *   -- polybench/POLYBENCH_3MM.hpp:61-86, -Cuda.cpp:144-160                 */
int b200_polybench_3mm(const double* A, const double* B, const double* C,
                       const double* D, double* E, double* F, double* G,
                       int64_t ni, int64_t nj, int64_t nk, int64_t nl,
                       int64_t nm, const b200_tune* tune, b200_stream_t stream);

/* C = alpha*A*B + beta*C, row-major m x k times k x n, native FP64 (the
 * classic GEMM form the split-precision path is measured against).        */
int b200_gemm_f64(const double* A, const double* B, double* C, int64_t m,
                  int64_t n, int64_t k, double alpha, double beta,
                  const b200_tune* tune, b200_stream_t stream);

/* Workspace for b200_gemm_split (slices and scales of A and B). */
size_t b200_gemm_split_workspace_bytes(int64_t m, int64_t n, int64_t k,
                                       const b200_tune* tune);

/* C = alpha*A*B + beta*C in FP64 by split precision on FP8 tensor cores:
 * rows of A / columns of B are scaled by powers of two and cut into
 * tune->items (default 10) balanced 5-bit integer slices (digits of
 * magnitude <= 16, held exactly in e4m3 or bf16); slice products of equal
 * weight accumulate exactly in FP32 on the tensor cores over chunks of at
 * most 8192 values of k (the bound under which the FP32 accumulation stays
 * exact), each chunk folded into an FP64 accumulator; the weighted sum is
 * formed in FP64.  k <= 524288.  tune->algo picks the engine: 0 (default) =
 * 4, tcgen05 MMA (kind::f8f6f4) on e4m3 slices with TMA-fed operands and
 * tensor-memory accumulators, digit weights w and w+1 formed together by
 * 128x256 MMAs; 3 the same with one weight at a time (128x128 MMAs); 2 that on
 * bf16 slices (kind::f16); 1 the legacy mma.sync path.  Every engine forms
 * the same digits, so all agree bit for bit whenever the accumulation is
 * exact and k <= 8192 (beyond, chunk sums are folded in a different order).  Zero the workspace once before its first use.  The
 * 32-bit word at byte offset 16 of the workspace is set to 1 if a bounded
 * wait of a tcgen05 engine gave up (C is then invalid); it stays set until
 * b200_workspace_status() reports and clears it.  Not in the reference: the
 * split-precision form of polybench/POLYBENCH_GEMM.hpp:40-56. */
int b200_gemm_split(const double* A, const double* B, double* C, int64_t m,
                    int64_t n, int64_t k, double alpha, double beta,
                    void* workspace, size_t workspace_bytes,
                    const b200_tune* tune, b200_stream_t stream);

/* ---- Algorithm ---------------------------------------------------------- */

/* Workspace for b200_algorithm_scan / _scan_i64 on n elements.  Zero it
 * once before first use; calls leave it ready for the next call.  The
 * 32-bit word at byte offset 16 becomes nonzero if a bounded wait gave up;
 * the results of that call are invalid and the workspace must be zeroed
 * again before the next call, which b200_workspace_status() does. */
size_t b200_scan_workspace_bytes(int64_t n);

/* y[i] = init + sum_{j<i} x[j] (exclusive), single-pass decoupled lookback.
 * Two kernels: the ring (one persistent CTA per SM streams 4096-item tiles
 * through a ring of shared-memory stages with bulk copies (TMA), with warps
 * dedicated to loading, tile aggregates, lookback and the in-place scan) and
 * the tile kernel (one CTA per tile with a dedicated lookback warp;
 * tune->items selects its tile, 32: 8192 items, the default; 16: 4096).
 * tune->algo 0 picks the ring for int64 and the tile kernel for FP64 (a
 * ring tile's FP64 aggregate is summed by one warp, on one sub-partition's
 * FP64 unit: 659 vs 466 us at 2^26); 1 forces the tile kernel, 2 the ring.
 * Unaligned x or y take the tile kernel.
 *   -- algorithm/SCAN.hpp:23-36, SCAN-Cuda.cpp:143-300.  One launch.        */
int b200_algorithm_scan(const double* x, double* y, int64_t n, double init,
                        void* workspace, size_t workspace_bytes,
                        const b200_tune* tune, b200_stream_t stream);

/* The same over int64 values: exact. */
int b200_algorithm_scan_i64(const int64_t* x, int64_t* y, int64_t n,
                            int64_t init, void* workspace,
                            size_t workspace_bytes, const b200_tune* tune,
                            b200_stream_t stream);

/* y[i] = x[i]  -- algorithm/MEMCPY.hpp:27-28, MEMCPY-Cuda.cpp:26.  The Stream
 * COPY kernel (16-byte vectors).                                            */
int b200_algorithm_memcpy(const double* x, double* y, int64_t n,
                          const b200_tune* tune, b200_stream_t stream);

/* x[i] = val  -- algorithm/MEMSET.hpp:27-28, MEMSET-Cuda.cpp:26.            */
int b200_algorithm_memset(double* x, double val, int64_t n,
                          const b200_tune* tune, b200_stream_t stream);

/* counts[b] = counts_init[b] + #{i : bins[i] == b}, b in [0, num_bins);
 * items with a bin outside the range are skipped.  Exact (integer counts)
 *   -- algorithm/HISTOGRAM.hpp:37-64, HISTOGRAM-Cuda.cpp:31.  Two launches. */
int b200_algorithm_histogram(const int64_t* bins, int64_t n, int64_t num_bins,
                             const unsigned long long* counts_init,
                             unsigned long long* counts, const b200_tune* tune,
                             b200_stream_t stream);

/* ---- Basic: index lists and multi-reductions ----------------------------- */

/* Workspace for b200_basic_indexlist on n items (zero it before first use;
 * calls leave it ready for the next; word at byte 16 = wait-gave-up flag). */
size_t b200_indexlist_workspace_bytes(int64_t n);

/* list[count++] = i for every i (in order) with x[i] < 0; *len = count.
 * n <= 2^31 - 1 (the list is int32, the suite's Int_type).  One launch,
 * single-pass compaction on a decoupled lookback.  tune->algo 0 (x 16-byte
 * aligned): one persistent CTA per SM; tiles of 4096 items arrive by bulk
 * copy, are ranked into 512-byte selection slots (freeing their stage at
 * once) and wait there for their base counts; runs of 4 consecutive tiles per
 * ticket need one global lookback each.  tune->algo 1 (and an unaligned x):
 * one CTA per 8192-item tile.
 *   -- basic/INDEXLIST.hpp:28-34, INDEXLIST-Cuda.cpp:33; also the list and
 *   count of basic/INDEXLIST_3LOOP.hpp:39-45, INDEXLIST_3LOOP-Cuda.cpp:34-56. */
int b200_basic_indexlist(const double* x, int32_t* list, int64_t n, int64_t* len,
                         void* workspace, size_t workspace_bytes,
                         const b200_tune* tune, b200_stream_t stream);

/* Workspace for b200_basic_multi_reduce (n items, num_bins bins).          */
size_t b200_multi_reduce_workspace_bytes(int64_t n, int64_t num_bins);

/* values[b] = values_init[b] + sum of data[i] over i with bins[i] == b.
 * Deterministic for num_bins <= 96 (fixed-order sums); more bins use FP64
 * atomics.  Items with a bin outside [0, num_bins) are skipped
 *   -- basic/MULTI_REDUCE.hpp:38-65, MULTI_REDUCE-Cuda.cpp:28.              */
int b200_basic_multi_reduce(const int64_t* bins, const double* data, int64_t n,
                            int64_t num_bins, const double* values_init,
                            double* values, void* workspace,
                            size_t workspace_bytes, const b200_tune* tune,
                            b200_stream_t stream);

/* ---- Comm: halo packing (one process) ----------------------------------- */

/* One (neighbour, variable) piece of a halo exchange: `len` entries of the
 * int32 index `list` into `var`, packed into / unpacked from `buffer`.  All
 * pointers are device addresses. */
typedef struct b200_halo_seg {
  double* var;
  const int32_t* list;
  double* buffer;
  int64_t len;
} b200_halo_seg;

/* buffer[i] = var[list[i]] for every segment of `pack` (HALO_PACK_BODY), then
 * var[list[i]] = buffer[i] for every segment of `unpack` (HALO_UNPACK_BODY),
 * in that order; at most 256 segments per direction, tables in host memory.
 * Unpack segments run concurrently: two of them writing the same element
 * land in unspecified order (halo lists never overlap).
 * Two launches, where the suite launches one kernel per segment
 *   -- comm/HALO_base.hpp:25-29, HALO_PACKING-Cuda.cpp,
 *      HALO_PACKING_FUSED-Cuda.cpp.                                         */
int b200_comm_halo_packing(const b200_halo_seg* pack, int32_t n_pack,
                           const b200_halo_seg* unpack, int32_t n_unpack,
                           const b200_tune* tune, b200_stream_t stream);

/* *sum = sum_init + sum_i x[i], fixed-shape tree (deterministic)
 *   -- algorithm/REDUCE_SUM.hpp:25-32, REDUCE_SUM-Seq.cpp:34-48             */
int b200_algorithm_reduce_sum(const double* x, int64_t n, double sum_init,
                              double* sum, void* workspace,
                              size_t workspace_bytes, const b200_tune* tune,
                              b200_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* B200_H */
