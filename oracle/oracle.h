/*
 * oracle.h -- CPU oracle for the Base_GB300 kernels.  TEST INFRASTRUCTURE:
 * only the test suite, the smoke check and the CPU-baseline leg of bench.py
 * use it; the product never links or calls it.
 *
 * A plain-C restatement of the RAJA Performance Suite's Base_Seq variant
 * (and, with threads > 0, its Base_OpenMP variant) for the kernels of the
 * hot path: the kernel constructors' sizes and byte/FLOP counts (K.cpp), the
 * data set-up order and formulas (K.cpp setUp + common/DataUtils.cpp), the
 * rep loops (K-Seq.cpp / K-OMP.cpp) and the checksum
 * (common/DataUtils.cpp:600-621).  Each function cites the file:line it
 * follows.  The restatement is pinned against the suite's own Base_Seq code,
 * compiled from the suite's sources by oracle/ref_build/ (golden checksums in
 * tests/golden/ref_checksums.json).
 */
#ifndef RAJAPERF_ORACLE_H
#define RAJAPERF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_opts {
  double size;             /* target size as --size; < 0 = kernel default   */
  long reps;               /* reps (as --checkrun)                          */
  int init_mode;           /* 0 = suite formulas, 1 = seeded uniform        */
  int threads;             /* 0 = Base_Seq, > 0 = Base_OpenMP with N threads */
  unsigned long long seed; /* uniform mode seed                              */
  double lo, hi;           /* uniform mode range                             */
  long tsteps;             /* Polybench time-step override; < 0 = default   */
  int variant;             /* kernel-specific: SCAN 1 = int64 values         */
  int skip_checksum;       /* 1: time the rep loop only (checksum = 0)      */
  long num_bins;           /* HISTOGRAM / MULTI_REDUCE bins; <= 0 = 10       */
  int bin_algo;            /* 0 Random, 1 RunsRandomSizes (default), 2 RunsEvenSizes, 3 Single */
  long halo_width;         /* HALO_PACKING halo width; <= 0 = 1             */
  long halo_num_vars;      /* HALO_PACKING variables; <= 0 = 3              */
} oracle_opts;

typedef struct oracle_result {
  double checksum;           /* long double checksum rounded to double      */
  double checksum_residual;  /* checksum - (double)checksum                  */
  long long actual_size;
  long long reps;
  long long its_per_rep;
  long long kernels_per_rep;
  long long bytes_per_rep;
  long long flops_per_rep;
  double time_s;             /* rep-loop wall time                           */
  int status;                /* 0 ok, 1 unknown kernel, 2 bad args, 3 alloc */
} oracle_result;

/* Runs one kernel with the suite's semantics. */
int oracle_run(const char* kernel, const oracle_opts* opts, oracle_result* out);

/* ---- building blocks, exposed for element-wise tests ---- */

/* common/DataUtils.cpp:504-513 */
void oracle_init_reference(double* p, int64_t n, double factor);
/* seeded uniform values, identical to the device generator */
double oracle_uniform_value(uint64_t seed, uint64_t stream, uint64_t i,
                            double lo, double hi);
void oracle_init_uniform(double* p, int64_t n, uint64_t seed, uint64_t stream,
                         double lo, double hi);
void oracle_init_uniform_i64(int64_t* p, int64_t n, uint64_t seed,
                             uint64_t stream, int64_t lo, int64_t hi);
/* common/DataUtils.cpp:600-621; returns the checksum rounded to double and
 * the rounding residual in *residual (may be NULL). */
double oracle_checksum(const double* p, int64_t n, double scale,
                       double* residual);
double oracle_checksum_i64(const int64_t* p, int64_t n, double scale,
                           double* residual);

/* One rep of a kernel body on caller arrays (Base_Seq loop order). */
void oracle_hydro_2d_rep(double* za, double* zb, const double* zm,
                         const double* zp, const double* zq, const double* zr,
                         double* zu, double* zv, const double* zz,
                         double* zrout, double* zzout, double s, double t,
                         int64_t kn, int64_t jn);
void oracle_del_dot_vec_2d_rep(const double* x, const double* y,
                               const double* xdot, const double* ydot,
                               double* div, const int64_t* real_zones,
                               int64_t nzones, int64_t jp, double ptiny,
                               double half);
void oracle_vol3d_rep(const double* x, const double* y, const double* z,
                      double* vol, double vnormq, int64_t jp, int64_t kp,
                      int64_t ibegin, int64_t iend);
void oracle_energy_rep(double* e_new, const double* e_old, const double* delvc,
                       const double* p_new, const double* p_old, double* q_new,
                       const double* q_old, const double* work,
                       const double* compHalfStep, const double* pHalfStep,
                       const double* bvc, const double* pbvc,
                       const double* ql_old, const double* qq_old,
                       const double* vnewc, double rho0, double e_cut,
                       double emin, double q_cut, int64_t n);
void oracle_jacobi_2d(double* A, double* B, int64_t N, int64_t tsteps);
void oracle_heat_3d(double* A, double* B, int64_t N, int64_t tsteps);
void oracle_fdtd_2d(double* ex, double* ey, double* hz, const double* fict,
                    int64_t nx, int64_t ny, int64_t tsteps);
/* Index of the planted minimum of FIRST_MIN in the uniform mode. */
int64_t oracle_first_min_planted_index(uint64_t seed, int64_t n);
void oracle_scan_f64(const double* x, double* y, int64_t n);
void oracle_scan_i64(const int64_t* x, int64_t* y, int64_t n);
void oracle_gemm(const double* A, const double* B, double* C, int64_t ni,
                 int64_t nj, int64_t nk, double alpha, double beta);

#ifdef __cplusplus
}
#endif

#endif
