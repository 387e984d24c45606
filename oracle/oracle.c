/*
 * oracle.c -- CPU oracle for the Base_GB300 kernels (TEST INFRASTRUCTURE;
 * see oracle.h).  Restates the RAJA Performance Suite's Base_Seq and
 * Base_OpenMP variants; citations are file:line in the suite's src/ tree.
 *
 * Build: cc -O2 -std=c11 -ffp-contract=off -fopenmp -shared -fPIC
 *        oracle.c -o liboracle.so -lm
 * (-ffp-contract=off: the same rounding as the suite's -O2 x86-64 Base_Seq.)
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef long long idx_t;

/* ------------------------------------------------------------------------ */
/* data set-up: common/DataUtils.cpp                                         */
/* ------------------------------------------------------------------------ */

typedef struct ctx {
  const oracle_opts* o;
  int count;           /* data_init_count, DataUtils.cpp:131-147 */
  int nt;              /* OpenMP threads (>= 1) */
  int par;             /* 1 when running the Base_OpenMP loops */
} ctx;

static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

static uint64_t counter_bits(uint64_t seed, uint64_t stream, uint64_t i) {
  uint64_t key = mix64(seed + 0x9e3779b97f4a7c15ULL * (stream + 1));
  return mix64(key + 0x9e3779b97f4a7c15ULL * (i + 1));
}

double oracle_uniform_value(uint64_t seed, uint64_t stream, uint64_t i,
                            double lo, double hi) {
  double u = (double)(counter_bits(seed, stream, i) >> 11) * 0x1.0p-53;
  return lo + (hi - lo) * u;
}

void oracle_init_uniform(double* p, int64_t n, uint64_t seed, uint64_t stream,
                         double lo, double hi) {
  for (int64_t i = 0; i < n; ++i) p[i] = oracle_uniform_value(seed, stream, i, lo, hi);
}

void oracle_init_uniform_i64(int64_t* p, int64_t n, uint64_t seed,
                             uint64_t stream, int64_t lo, int64_t hi) {
  uint64_t range = (uint64_t)(hi - lo);
  for (int64_t i = 0; i < n; ++i)
    p[i] = lo + (int64_t)(counter_bits(seed, stream, i) % range);
}

/* DataUtils.cpp:504-513 */
void oracle_init_reference(double* p, int64_t n, double factor) {
  for (int64_t i = 0; i < n; ++i) p[i] = factor * (i + 1.1) / (i + 1.12345);
}

static double* alloc_raw(int64_t n) {
  double* p = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  return p;
}

/* allocAndInitData (DataUtils.cpp:504-513), or the uniform mode */
static double* alloc_init(ctx* c, int64_t n) {
  double* p = alloc_raw(n);
  if (!p) return NULL;
  if (c->o->init_mode == 1) {
    oracle_init_uniform(p, n, c->o->seed, (uint64_t)c->count, c->o->lo, c->o->hi);
  } else {
    oracle_init_reference(p, n, (c->count % 2 ? 0.1 : 0.2));
  }
  c->count++;
  return p;
}

/* allocAndInitDataConst (DataUtils.cpp:518-536) */
static double* alloc_const(ctx* c, int64_t n, double v) {
  double* p = alloc_raw(n);
  if (!p) return NULL;
  for (int64_t i = 0; i < n; ++i) p[i] = v;
  c->count++;
  return p;
}

static int64_t* alloc_const_idx(ctx* c, int64_t n, int64_t v) {
  int64_t* p = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  if (!p) return NULL;
  for (int64_t i = 0; i < n; ++i) p[i] = v;
  c->count++;
  return p;
}

/* allocAndInitDataRandValue (DataUtils.cpp:560-569) */
static double* alloc_randvalue(ctx* c, int64_t n) {
  if (c->o->init_mode == 1) return alloc_init(c, n);
  double* p = alloc_raw(n);
  if (!p) return NULL;
  srand(4793);
  for (int64_t i = 0; i < n; ++i) p[i] = (double)rand() / RAND_MAX;
  c->count++;
  return p;
}

/* allocAndInitDataRandSign (DataUtils.cpp:542-555), or the uniform mode */
static double* alloc_randsign(ctx* c, int64_t n) {
  if (c->o->init_mode == 1) return alloc_init(c, n);
  double* p = alloc_raw(n);
  if (!p) return NULL;
  double factor = (c->count % 2 ? 0.1 : 0.2);
  srand(4793);
  for (int64_t i = 0; i < n; ++i) {
    double s = (double)rand() / RAND_MAX;
    s = (s < 0.5 ? -1.0 : 1.0);
    p[i] = s * factor * (i + 1.1) / (i + 1.12345);
  }
  c->count++;
  return p;
}

/* allocAndInitData(Int_ptr) (DataUtils.cpp:477-497), in either mode; an
 * index equal to n (rand() == RAND_MAX) is skipped. */
static int* alloc_int(ctx* c, int64_t n) {
  int* p = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  if (!p) return NULL;
  srand(4793);
  for (int64_t i = 0; i < n; ++i) p[i] = ((double)rand() / RAND_MAX < 0.5 ? -1 : 1);
  double f = (double)rand() / RAND_MAX;
  size_t ilo = (size_t)(n * f);
  if ((int64_t)ilo < n) p[ilo] = -58;
  f = (double)rand() / RAND_MAX;
  size_t ihi = (size_t)(n * f);
  if ((int64_t)ihi < n) p[ihi] = 19;
  c->count++;
  return p;
}

/* rand()/RAND_MAX values (DataUtils.cpp:560-569) in either mode; bumps the
 * init count like allocAndInitDataRandValue. */
static double* rand_values(ctx* c, int64_t n) {
  double* p = alloc_raw(n);
  if (!p) return NULL;
  srand(4793);
  for (int64_t i = 0; i < n; ++i) p[i] = (double)rand() / RAND_MAX;
  c->count++;
  return p;
}

static int cmp_double(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* The bins of HISTOGRAM / MULTI_REDUCE (algorithm/HISTOGRAM.cpp:73-131,
 * basic/MULTI_REDUCE.cpp:74-133). */
static int64_t* assign_bins(ctx* c, int64_t n, int64_t num_bins, int algo) {
  int64_t* bins = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  if (!bins) return NULL;
  if (algo == 0) {
    double* d = rand_values(c, n);
    if (!d) { free(bins); return NULL; }
    for (int64_t i = 0; i < n; ++i) {
      int64_t b = (int64_t)(d[i] * num_bins);
      if (b >= num_bins) b = num_bins - 1;
      if (b < 0) b = 0;
      bins[i] = b;
    }
    free(d);
    return bins;
  }
  double* bounds;
  if (algo == 1) {
    bounds = rand_values(c, num_bins);
    if (!bounds) { free(bins); return NULL; }
    qsort(bounds, (size_t)num_bins, sizeof(double), cmp_double);
  } else {
    bounds = alloc_raw(num_bins);
    if (!bounds) { free(bins); return NULL; }
    for (int64_t b = 0; b < num_bins; ++b)
      bounds[b] = (algo == 2) ? (double)(b + 1) / num_bins : 0.0;
  }
  int64_t bin = 0;
  for (int64_t i = 0; i < n; ++i) {
    double pos = (double)i / n;
    while (bin + 1 < num_bins && pos >= bounds[bin]) bin += 1;
    bins[i] = bin;
  }
  free(bounds);
  return bins;
}

/* initData(Real_type&) (DataUtils.cpp:589-595) */
static double init_scalar(ctx* c) {
  double factor = (c->count % 2 ? 0.1 : 0.2);
  double d = factor * 1.1 / 1.12345;
  c->count++;
  return d;
}

static __thread int g_skip_checksum = 0;

/* DataUtils.cpp:600-621 */
static long double checksum_ld(const double* p, int64_t n, double scale) {
  if (g_skip_checksum) return 0.0L;
  long double tchk = 0.0;
  long double ckahan = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    long double x = (fabs(sin(j + 1.0)) + 0.5) * (long double)p[j];
    long double y = x - ckahan;
    volatile long double t = tchk + y;
    volatile long double z = t - tchk;
    ckahan = z - y;
    tchk = t;
  }
  tchk *= scale;
  return tchk;
}

static long double checksum_ld_i64(const int64_t* p, int64_t n, double scale) {
  if (g_skip_checksum) return 0.0L;
  long double tchk = 0.0;
  long double ckahan = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    long double x = (fabs(sin(j + 1.0)) + 0.5) * (long double)p[j];
    long double y = x - ckahan;
    volatile long double t = tchk + y;
    volatile long double z = t - tchk;
    ckahan = z - y;
    tchk = t;
  }
  tchk *= scale;
  return tchk;
}

static long double checksum_ld_int(const int* p, int64_t n, double scale) {
  if (g_skip_checksum) return 0.0L;
  long double tchk = 0.0, ckahan = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    long double x = (fabs(sin(j + 1.0)) + 0.5) * (long double)p[j];
    long double y = x - ckahan;
    volatile long double t = tchk + y;
    volatile long double z = t - tchk;
    ckahan = z - y;
    tchk = t;
  }
  return tchk * scale;
}

static long double checksum_ld_u64(const unsigned long long* p, int64_t n, double scale) {
  if (g_skip_checksum) return 0.0L;
  long double tchk = 0.0, ckahan = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    long double x = (fabs(sin(j + 1.0)) + 0.5) * (long double)p[j];
    long double y = x - ckahan;
    volatile long double t = tchk + y;
    volatile long double z = t - tchk;
    ckahan = z - y;
    tchk = t;
  }
  return tchk * scale;
}

double oracle_checksum(const double* p, int64_t n, double scale, double* residual) {
  g_skip_checksum = 0;
  long double v = checksum_ld(p, n, scale);
  double d = (double)v;
  if (residual) *residual = (double)(v - (long double)d);
  return d;
}

double oracle_checksum_i64(const int64_t* p, int64_t n, double scale, double* residual) {
  g_skip_checksum = 0;
  long double v = checksum_ld_i64(p, n, scale);
  double d = (double)v;
  if (residual) *residual = (double)(v - (long double)d);
  return d;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* KernelBase.cpp:115-125 */
static idx_t target_size(const ctx* c, idx_t default_size) {
  if (c->o->size >= 0) return (idx_t)c->o->size;
  return (idx_t)(default_size * 1.0);
}

static void set_result(oracle_result* r, long double ck, idx_t size, idx_t reps,
                       idx_t its, idx_t kernels, idx_t bytes, idx_t flops, double t) {
  r->checksum = (double)ck;
  r->checksum_residual = (double)(ck - (long double)r->checksum);
  r->actual_size = size;
  r->reps = reps;
  r->its_per_rep = its;
  r->kernels_per_rep = kernels;
  r->bytes_per_rep = bytes;
  r->flops_per_rep = flops;
  r->time_s = t;
  r->status = 0;
}

#define NT (c->nt)
#define PAR (c->par)
#define OMP_FOR _Pragma("omp parallel for num_threads(NT) if(PAR)")
#define OMP_FOR2 _Pragma("omp parallel for collapse(2) num_threads(NT) if(PAR)")
#define CHECK_ALLOC(p) do { if (!(p)) { r->status = 3; goto done; } } while (0)

/* ------------------------------------------------------------------------ */
/* Stream: stream/{COPY,MUL,ADD,TRIAD,DOT}.cpp and -Seq.cpp / -OMP.cpp       */
/* ------------------------------------------------------------------------ */

/* COPY.cpp:21-69, COPY-Seq.cpp:37 */
static void run_copy(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *a = alloc_init(c, n), *cc = alloc_const(c, n, 0.0);
  double t0;
  CHECK_ALLOC(a); CHECK_ALLOC(cc);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) cc[i] = a[i];
  }
  set_result(r, checksum_ld(cc, n, 1.0), n, reps, n, 1, 16 * n, 0, now_s() - t0);
done:
  free(a); free(cc);
}

/* MUL.cpp:21-75, MUL.hpp:25 */
static void run_mul(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *b = alloc_const(c, n, 0.0), *cc = alloc_init(c, n);
  double alpha = init_scalar(c), t0;
  CHECK_ALLOC(b); CHECK_ALLOC(cc);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) b[i] = alpha * cc[i];
  }
  set_result(r, checksum_ld(b, n, 1.0), n, reps, n, 1, 16 * n, n, now_s() - t0);
done:
  free(b); free(cc);
}

/* ADD.cpp:21-76, ADD.hpp:25 */
static void run_add(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *a = alloc_init(c, n), *b = alloc_init(c, n), *cc = alloc_const(c, n, 0.0);
  double t0;
  CHECK_ALLOC(a); CHECK_ALLOC(b); CHECK_ALLOC(cc);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) cc[i] = a[i] + b[i];
  }
  set_result(r, checksum_ld(cc, n, 1.0), n, reps, n, 1, 24 * n, n, now_s() - t0);
done:
  free(a); free(b); free(cc);
}

/* TRIAD.cpp:24-84, TRIAD.hpp:26, TRIAD-Seq.cpp:37-47 */
static void run_triad(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *a = alloc_const(c, n, 0.0), *b = alloc_init(c, n), *cc = alloc_init(c, n);
  double alpha = init_scalar(c), t0;
  long double scale = (long double)0.001 * ((long double)1000000 / n);
  CHECK_ALLOC(a); CHECK_ALLOC(b); CHECK_ALLOC(cc);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) a[i] = b[i] + alpha * cc[i];
  }
  set_result(r, checksum_ld(a, n, (double)scale), n, reps, n, 1, 24 * n, 2 * n,
             now_s() - t0);
done:
  free(a); free(b); free(cc);
}

/* DOT.cpp:21-81, DOT-Seq.cpp:34-47, DOT-OMP.cpp:33-45 */
static void run_dot(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *a = alloc_init(c, n), *b = alloc_init(c, n);
  double m_dot = 0.0, m_dot_init = 0.0, t0;
  CHECK_ALLOC(a); CHECK_ALLOC(b);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    double dot = m_dot_init;
    if (PAR) {
      #pragma omp parallel for reduction(+:dot) num_threads(NT)
      for (idx_t i = 0; i < n; ++i) dot += a[i] * b[i];
    } else {
      for (idx_t i = 0; i < n; ++i) dot += a[i] * b[i];
    }
    m_dot += dot;
  }
  set_result(r, (long double)m_dot, n, reps, n, 1, 8 + 16 * n + 8, 2 * n, now_s() - t0);
done:
  free(a); free(b);
}

/* ------------------------------------------------------------------------ */
/* Basic: basic/{DAXPY,INIT3,MULADDSUB}.cpp                                  */
/* ------------------------------------------------------------------------ */

/* DAXPY.cpp:20-70, DAXPY.hpp: y[i] += a*x[i] */
static void run_daxpy(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *y = alloc_const(c, n, 0.0), *x = alloc_init(c, n);
  double a = init_scalar(c), t0;
  CHECK_ALLOC(x); CHECK_ALLOC(y);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) y[i] += a * x[i];
  }
  set_result(r, checksum_ld(y, n, 1.0), n, reps, n, 1, 24 * n, 2 * n, now_s() - t0);
done:
  free(x); free(y);
}

/* INIT3.cpp, INIT3.hpp: out1 = out2 = out3 = -in1 - in2 */
static void run_init3(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *o1 = alloc_const(c, n, 0.0), *o2 = alloc_const(c, n, 0.0),
         *o3 = alloc_const(c, n, 0.0), *i1 = alloc_init(c, n), *i2 = alloc_init(c, n);
  double t0;
  long double ck;
  CHECK_ALLOC(o1); CHECK_ALLOC(o2); CHECK_ALLOC(o3); CHECK_ALLOC(i1); CHECK_ALLOC(i2);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) o1[i] = o2[i] = o3[i] = -i1[i] - i2[i];
  }
  t0 = now_s() - t0;
  ck = checksum_ld(o1, n, 1.0);
  ck += checksum_ld(o2, n, 1.0);
  ck += checksum_ld(o3, n, 1.0);
  set_result(r, ck, n, reps, n, 1, 40 * n, n, t0);
done:
  free(o1); free(o2); free(o3); free(i1); free(i2);
}

/* MULADDSUB.cpp, MULADDSUB.hpp */
static void run_muladdsub(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *o1 = alloc_const(c, n, 0.0), *o2 = alloc_const(c, n, 0.0),
         *o3 = alloc_const(c, n, 0.0), *i1 = alloc_init(c, n), *i2 = alloc_init(c, n);
  double t0;
  long double ck;
  CHECK_ALLOC(o1); CHECK_ALLOC(o2); CHECK_ALLOC(o3); CHECK_ALLOC(i1); CHECK_ALLOC(i2);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) {
      o1[i] = i1[i] * i2[i];
      o2[i] = i1[i] + i2[i];
      o3[i] = i1[i] - i2[i];
    }
  }
  t0 = now_s() - t0;
  ck = checksum_ld(o1, n, 1.0);
  ck += checksum_ld(o2, n, 1.0);
  ck += checksum_ld(o3, n, 1.0);
  set_result(r, ck, n, reps, n, 1, 40 * n, 3 * n, t0);
done:
  free(o1); free(o2); free(o3); free(i1); free(i2);
}

/* ------------------------------------------------------------------------ */
/* Lcals                                                                     */
/* ------------------------------------------------------------------------ */

/* HYDRO_1D.cpp:24-87, HYDRO_1D.hpp:30 */
static void run_hydro_1d(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps, len = n + 12;
  double *x = alloc_const(c, len, 0.0), *y = alloc_init(c, len), *z = alloc_init(c, len);
  double q = init_scalar(c), rr = init_scalar(c), t = init_scalar(c), t0;
  long double scale = (long double)0.001 * ((long double)1000000 / n);
  CHECK_ALLOC(x); CHECK_ALLOC(y); CHECK_ALLOC(z);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) x[i] = q + y[i] * (rr * z[i + 10] + t * z[i + 11]);
  }
  set_result(r, checksum_ld(x, n, (double)scale), n, reps, n, 1,
             8 * n + 8 * (n + 1) + 8 * n, 5 * n, now_s() - t0);
done:
  free(x); free(y); free(z);
}

/* HYDRO_2D.hpp:66-90 (BODY1..3), HYDRO_2D-Seq.cpp:24-66 */
void oracle_hydro_2d_rep(double* za, double* zb, const double* zm,
                         const double* zp, const double* zq, const double* zr,
                         double* zu, double* zv, const double* zz,
                         double* zrout, double* zzout, double s, double t,
                         int64_t kn, int64_t jn) {
  for (idx_t k = 1; k < kn - 1; ++k)
    for (idx_t j = 1; j < jn - 1; ++j) {
      za[j + k * jn] = (zp[j - 1 + (k + 1) * jn] + zq[j - 1 + (k + 1) * jn] -
                        zp[j - 1 + k * jn] - zq[j - 1 + k * jn]) *
                       (zr[j + k * jn] + zr[j - 1 + k * jn]) /
                       (zm[j - 1 + k * jn] + zm[j - 1 + (k + 1) * jn]);
      zb[j + k * jn] = (zp[j - 1 + k * jn] + zq[j - 1 + k * jn] - zp[j + k * jn] -
                        zq[j + k * jn]) *
                       (zr[j + k * jn] + zr[j + (k - 1) * jn]) /
                       (zm[j + k * jn] + zm[j - 1 + k * jn]);
    }
  for (idx_t k = 1; k < kn - 1; ++k)
    for (idx_t j = 1; j < jn - 1; ++j) {
      zu[j + k * jn] += s * (za[j + k * jn] * (zz[j + k * jn] - zz[j + 1 + k * jn]) -
                             za[j - 1 + k * jn] * (zz[j + k * jn] - zz[j - 1 + k * jn]) -
                             zb[j + k * jn] * (zz[j + k * jn] - zz[j + (k - 1) * jn]) +
                             zb[j + (k + 1) * jn] * (zz[j + k * jn] - zz[j + (k + 1) * jn]));
      zv[j + k * jn] += s * (za[j + k * jn] * (zr[j + k * jn] - zr[j + 1 + k * jn]) -
                             za[j - 1 + k * jn] * (zr[j + k * jn] - zr[j - 1 + k * jn]) -
                             zb[j + k * jn] * (zr[j + k * jn] - zr[j + (k - 1) * jn]) +
                             zb[j + (k + 1) * jn] * (zr[j + k * jn] - zr[j + (k + 1) * jn]));
    }
  for (idx_t k = 1; k < kn - 1; ++k)
    for (idx_t j = 1; j < jn - 1; ++j) {
      zrout[j + k * jn] = zr[j + k * jn] + t * zu[j + k * jn];
      zzout[j + k * jn] = zz[j + k * jn] + t * zv[j + k * jn];
    }
}

/* HYDRO_2D.cpp:27-107 */
static void run_hydro_2d(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 1000 * 1000);
  idx_t jn = (idx_t)(sqrt((double)target) + sqrt(2.0) - 1), kn = jn;
  idx_t len = kn * jn;
  double s = 0.0041, t = 0.0037, t0;
  double *zrout = alloc_const(c, len, 0.0), *zzout = alloc_const(c, len, 0.0);
  double *za = alloc_init(c, len), *zb = alloc_init(c, len), *zm = alloc_init(c, len),
         *zp = alloc_init(c, len), *zq = alloc_init(c, len), *zr = alloc_init(c, len),
         *zu = alloc_init(c, len), *zv = alloc_init(c, len), *zz = alloc_init(c, len);
  long double scale = (long double)0.001 * ((long double)1000000 / target), ck;
  CHECK_ALLOC(zrout); CHECK_ALLOC(zzout); CHECK_ALLOC(za); CHECK_ALLOC(zb);
  CHECK_ALLOC(zm); CHECK_ALLOC(zp); CHECK_ALLOC(zq); CHECK_ALLOC(zr);
  CHECK_ALLOC(zu); CHECK_ALLOC(zv); CHECK_ALLOC(zz);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    if (!PAR) {
      oracle_hydro_2d_rep(za, zb, zm, zp, zq, zr, zu, zv, zz, zrout, zzout, s, t, kn, jn);
      continue;
    }
    OMP_FOR
    for (idx_t k = 1; k < kn - 1; ++k)
      for (idx_t j = 1; j < jn - 1; ++j) {
        za[j + k * jn] = (zp[j - 1 + (k + 1) * jn] + zq[j - 1 + (k + 1) * jn] -
                          zp[j - 1 + k * jn] - zq[j - 1 + k * jn]) *
                         (zr[j + k * jn] + zr[j - 1 + k * jn]) /
                         (zm[j - 1 + k * jn] + zm[j - 1 + (k + 1) * jn]);
        zb[j + k * jn] = (zp[j - 1 + k * jn] + zq[j - 1 + k * jn] - zp[j + k * jn] -
                          zq[j + k * jn]) *
                         (zr[j + k * jn] + zr[j + (k - 1) * jn]) /
                         (zm[j + k * jn] + zm[j - 1 + k * jn]);
      }
    OMP_FOR
    for (idx_t k = 1; k < kn - 1; ++k)
      for (idx_t j = 1; j < jn - 1; ++j) {
        zu[j + k * jn] += s * (za[j + k * jn] * (zz[j + k * jn] - zz[j + 1 + k * jn]) -
                               za[j - 1 + k * jn] * (zz[j + k * jn] - zz[j - 1 + k * jn]) -
                               zb[j + k * jn] * (zz[j + k * jn] - zz[j + (k - 1) * jn]) +
                               zb[j + (k + 1) * jn] * (zz[j + k * jn] - zz[j + (k + 1) * jn]));
        zv[j + k * jn] += s * (za[j + k * jn] * (zr[j + k * jn] - zr[j + 1 + k * jn]) -
                               za[j - 1 + k * jn] * (zr[j + k * jn] - zr[j - 1 + k * jn]) -
                               zb[j + k * jn] * (zr[j + k * jn] - zr[j + (k - 1) * jn]) +
                               zb[j + (k + 1) * jn] * (zr[j + k * jn] - zr[j + (k + 1) * jn]));
      }
    OMP_FOR
    for (idx_t k = 1; k < kn - 1; ++k)
      for (idx_t j = 1; j < jn - 1; ++j) {
        zrout[j + k * jn] = zr[j + k * jn] + t * zu[j + k * jn];
        zzout[j + k * jn] = zz[j + k * jn] + t * zv[j + k * jn];
      }
  }
  t0 = now_s() - t0;
  ck = checksum_ld(zzout, len, (double)scale);
  ck += checksum_ld(zrout, len, (double)scale);
  set_result(r, ck, target, reps, 3 * target, 3,
             (4 * 8 * len + 4 * 8 * len + 4 * 8 * (kn - 2) * (jn - 2)) +
                 (2 + 2 + 2) * 8 * (kn - 2) * (jn - 2),
             (14 + 26 + 4) * (jn - 2) * (kn - 2), t0);
done:
  free(zrout); free(zzout); free(za); free(zb); free(zm); free(zp);
  free(zq); free(zr); free(zu); free(zv); free(zz);
}

/* EOS.cpp:24-89, EOS.hpp:33 */
static void run_eos(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps, len = n + 7;
  double *x = alloc_const(c, len, 0.0), *y = alloc_init(c, len), *z = alloc_init(c, len),
         *u = alloc_init(c, len);
  double q = init_scalar(c), rr = init_scalar(c), t = init_scalar(c), t0;
  long double scale = (long double)0.0001 * ((long double)1000000 / n);
  CHECK_ALLOC(x); CHECK_ALLOC(y); CHECK_ALLOC(z); CHECK_ALLOC(u);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i)
      x[i] = u[i] + rr * (z[i] + rr * y[i]) +
             t * (u[i + 3] + rr * (u[i + 2] + rr * u[i + 1]) +
                  t * (u[i + 6] + q * (u[i + 5] + q * u[i + 4])));
  }
  set_result(r, checksum_ld(x, n, (double)scale), n, reps, n, 1,
             16 * n + 8 * len + 8 * n, 16 * n, now_s() - t0);
done:
  free(x); free(y); free(z); free(u);
}

/* FIRST_DIFF.cpp:24-77, FIRST_DIFF.hpp:25 */
static void run_first_diff(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps, N = n + 1;
  double *x = alloc_const(c, N, 0.0), *y = alloc_init(c, N), t0;
  CHECK_ALLOC(x); CHECK_ALLOC(y);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) x[i] = y[i + 1] - y[i];
  }
  set_result(r, checksum_ld(x, n, 1.0), n, reps, n, 1, 8 * N + 8 * n, n, now_s() - t0);
done:
  free(x); free(y);
}

/* INT_PREDICT.cpp:24-93, INT_PREDICT.hpp:40 */
static void run_int_predict(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  idx_t len = n * 13, offset = n;
  double initval = 1.0;
  double* px = alloc_const(c, len, initval);
  double dm22 = init_scalar(c), dm23 = init_scalar(c), dm24 = init_scalar(c),
         dm25 = init_scalar(c), dm26 = init_scalar(c), dm27 = init_scalar(c),
         dm28 = init_scalar(c), c0 = init_scalar(c), t0;
  CHECK_ALLOC(px);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i)
      px[i] = dm28 * px[i + offset * 12] + dm27 * px[i + offset * 11] +
              dm26 * px[i + offset * 10] + dm25 * px[i + offset * 9] +
              dm24 * px[i + offset * 8] + dm23 * px[i + offset * 7] +
              dm22 * px[i + offset * 6] +
              c0 * (px[i + offset * 4] + px[i + offset * 5]) + px[i + offset * 2];
  }
  t0 = now_s() - t0;
  /* INT_PREDICT.cpp:80-88: subtract the initial value before the checksum */
  for (idx_t i = 0; i < n; ++i) px[i] -= initval;
  set_result(r, checksum_ld(px, n, 1.0), n, reps, n, 1, 88 * n, 17 * n, t0);
done:
  free(px);
}

/* FIRST_MIN.cpp:24-94, FIRST_MIN.hpp:29-54, FIRST_MIN-Seq.cpp:34-48.
 * Uniform mode: x uniform in [lo, hi) with one planted minimum lo - 1 at a
 * seeded index. */
int64_t oracle_first_min_planted_index(uint64_t seed, int64_t n) {
  double u = oracle_uniform_value(seed, 0xF1257ULL, 0, 0.0, 1.0);
  int64_t idx = (int64_t)(u * (double)n);
  return idx >= n ? n - 1 : idx;
}

static void run_first_min(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *x, xmin_init, t0;
  idx_t initloc = 0, minloc = -1;
  if (c->o->init_mode == 1) {
    x = alloc_init(c, n);
    CHECK_ALLOC(x);
    x[oracle_first_min_planted_index(c->o->seed, n)] = c->o->lo - 1.0;
  } else {
    x = alloc_const(c, n, 0.0);
    CHECK_ALLOC(x);
    x[n / 2] = -1.0e+10;
  }
  xmin_init = x[0];
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    double mval = xmin_init;
    idx_t mloc = initloc;
    if (PAR) {
      /* FIRST_MIN-OMP.cpp Base_OpenMP: per-thread min-loc, then combine
       * (a.val < b.val ? a : b). */
      int nth = NT;
      double* tv = (double*)malloc(sizeof(double) * nth);
      idx_t* tl = (idx_t*)malloc(sizeof(idx_t) * nth);
      for (int k = 0; k < nth; ++k) { tv[k] = mval; tl[k] = mloc; }
      #pragma omp parallel num_threads(NT)
      {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double v = mval;
        idx_t l = mloc;
        #pragma omp for
        for (idx_t i = 0; i < n; ++i)
          if (x[i] < v) { v = x[i]; l = i; }
        tv[tid] = v;
        tl[tid] = l;
      }
      for (int k = 0; k < nth; ++k)
        if (!(mval < tv[k])) { mval = tv[k]; mloc = tl[k]; }
      free(tv); free(tl);
    } else {
      for (idx_t i = 0; i < n; ++i)
        if (x[i] < mval) { mval = x[i]; mloc = i; }
    }
    minloc = mloc;
  }
  set_result(r, (long double)minloc, n, reps, n, 1, 8 + 8 + 8 * n + 8 + 8, 0,
             now_s() - t0);
done:
  free(x);
}

/* DIFF_PREDICT.cpp, DIFF_PREDICT.hpp */
static void run_diff_predict(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  idx_t len = n * 14, o = n;
  double *px = alloc_const(c, len, 0.0), *cx = alloc_init(c, len), t0;
  CHECK_ALLOC(px); CHECK_ALLOC(cx);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) {
      double ar, br, cr;
      ar = cx[i + o * 4];
      br = ar - px[i + o * 4];
      px[i + o * 4] = ar;
      cr = br - px[i + o * 5];
      px[i + o * 5] = br;
      ar = cr - px[i + o * 6];
      px[i + o * 6] = cr;
      br = ar - px[i + o * 7];
      px[i + o * 7] = ar;
      cr = br - px[i + o * 8];
      px[i + o * 8] = br;
      ar = cr - px[i + o * 9];
      px[i + o * 9] = cr;
      br = ar - px[i + o * 10];
      px[i + o * 10] = ar;
      cr = br - px[i + o * 11];
      px[i + o * 11] = br;
      px[i + o * 13] = cr - px[i + o * 12];
      px[i + o * 12] = cr;
    }
  }
  set_result(r, checksum_ld(px, len, 1.0), n, reps, n, 1, 160 * n, 9 * n, now_s() - t0);
done:
  free(px); free(cx);
}

/* PLANCKIAN.cpp, PLANCKIAN.hpp */
static void run_planckian(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *x = alloc_init(c, n), *y = alloc_init(c, n), *u = alloc_init(c, n),
         *v = alloc_init(c, n), *w = alloc_const(c, n, 0.0), t0;
  CHECK_ALLOC(x); CHECK_ALLOC(y); CHECK_ALLOC(u); CHECK_ALLOC(v); CHECK_ALLOC(w);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) {
      y[i] = u[i] / v[i];
      w[i] = x[i] / (exp(y[i]) - 1.0);
    }
  }
  set_result(r, checksum_ld(w, n, 1.0), n, reps, n, 1, 40 * n, 4 * n, now_s() - t0);
done:
  free(x); free(y); free(u); free(v); free(w);
}

/* ------------------------------------------------------------------------ */
/* Apps: apps/AppsData.{hpp,cpp} mesh helpers                                */
/* ------------------------------------------------------------------------ */

typedef struct adomain {
  idx_t ndims, NPNL, NPNR, imin, jmin, kmin, imax, jmax, kmax, jp, kp, nnalls;
  idx_t fpn, lpn, frn, lrn, fpz, lpz, n_real_zones, n_real_nodes;
} adomain;

/* AppsData.hpp ADomain constructor */
static adomain make_domain(idx_t rnpd, idx_t ndims) {
  adomain d;
  memset(&d, 0, sizeof(d));
  d.ndims = ndims;
  d.NPNL = 2;
  d.NPNR = 1;
  idx_t NPZL = d.NPNL - 1, NPZR = d.NPNR + 1 - 1;
  d.imin = d.NPNL;
  d.imax = d.NPNL + rnpd - 1;
  d.nnalls = (d.imax + 1 - d.imin + d.NPNL + d.NPNR);
  d.n_real_zones = (d.imax - d.imin);
  d.n_real_nodes = (d.imax + 1 - d.imin);
  if (ndims >= 2) {
    d.jmin = d.NPNL;
    d.jmax = d.NPNL + rnpd - 1;
    d.jp = d.nnalls;
    d.nnalls *= (d.jmax + 1 - d.jmin + d.NPNL + d.NPNR);
    d.n_real_zones *= (d.jmax - d.jmin);
    d.n_real_nodes *= (d.jmax + 1 - d.jmin);
  }
  if (ndims >= 3) {
    d.kmin = d.NPNL;
    d.kmax = d.NPNL + rnpd - 1;
    d.kp = d.nnalls;
    d.nnalls *= (d.kmax + 1 - d.kmin + d.NPNL + d.NPNR);
    d.n_real_zones *= (d.kmax - d.kmin);
    d.n_real_nodes *= (d.kmax + 1 - d.kmin);
  }
  d.frn = d.kmin * d.kp + d.jmin * d.jp + d.imin;
  d.lrn = d.kmax * d.kp + d.jmax * d.jp + d.imax;
  d.fpn = (d.kmin - d.NPNL) * d.kp + (d.jmin - d.NPNL) * d.jp + (d.imin - d.NPNL);
  d.lpn = (d.kmax + d.NPNR) * d.kp + (d.jmax + d.NPNR) * d.jp + (d.imax + d.NPNR);
  d.fpz = (d.kmin - NPZL) * d.kp + (d.jmin - NPZL) * d.jp + (d.imin - NPZL);
  d.lpz = (d.kmax - 1 + NPZR) * d.kp + (d.jmax - 1 + NPZR) * d.jp + (d.imax - 1 + NPZR);
  return d;
}

/* AppsData.cpp:56-81 setRealZones_2d */
static void set_real_zones_2d(int64_t* rz, const adomain* d) {
  idx_t j_stride = d->imax - d->imin;
  for (idx_t j = d->jmin; j < d->jmax; j++)
    for (idx_t i = d->imin; i < d->imax; i++)
      rz[(i - d->imin) + (j - d->jmin) * j_stride] = i + j * d->jp;
}

/* AppsData.cpp:122-151 setMeshPositions_2d; uniform mode jitters each node
 * by up to 0.1 cell in x and y. */
static void set_mesh_2d(double* x, double dx, double* y, double dy,
                        const adomain* d, const oracle_opts* o) {
  for (idx_t j = d->jmin - d->NPNL; j < d->jmax + 1 + d->NPNR; j++)
    for (idx_t i = d->imin - d->NPNL; i < d->imax + 1 + d->NPNR; i++) {
      idx_t in = i + j * d->jp;
      x[in] = i * dx;
      y[in] = j * dy;
      if (o->init_mode == 1) {
        x[in] += dx * oracle_uniform_value(o->seed, 0x2D0001ULL, (uint64_t)in, -0.1, 0.1);
        y[in] += dy * oracle_uniform_value(o->seed, 0x2D0002ULL, (uint64_t)in, -0.1, 0.1);
      }
    }
}

/* AppsData.cpp:153-180 setMeshPositions_3d */
static void set_mesh_3d(double* x, double dx, double* y, double dy, double* z,
                        double dz, const adomain* d) {
  for (idx_t k = d->kmin - d->NPNL; k < d->kmax + 1 + d->NPNR; k++)
    for (idx_t j = d->jmin - d->NPNL; j < d->jmax + 1 + d->NPNR; j++)
      for (idx_t i = d->imin - d->NPNL; i < d->imax + 1 + d->NPNR; i++) {
        idx_t in = i + j * d->jp + k * d->kp;
        x[in] = i * dx;
        y[in] = j * dy;
        z[in] = k * dz;
      }
}

/* DEL_DOT_VEC_2D.hpp:65-90 (NDSET2D corners v4=v, v1=v+1, v2=v1+jp, v3=v+jp) */
#define DDV_BODY(ii)                                                            \
  do {                                                                          \
    idx_t i = real_zones[ii];                                                   \
    const double *x4 = x, *x1 = x + 1, *x2 = x1 + jp, *x3 = x + jp;             \
    const double *y4 = y, *y1 = y + 1, *y2 = y1 + jp, *y3 = y + jp;             \
    const double *fx4 = xdot, *fx1 = xdot + 1, *fx2 = fx1 + jp, *fx3 = xdot + jp; \
    const double *fy4 = ydot, *fy1 = ydot + 1, *fy2 = fy1 + jp, *fy3 = ydot + jp; \
    double xi = half * (x1[i] + x2[i] - x3[i] - x4[i]);                        \
    double xj = half * (x2[i] + x3[i] - x4[i] - x1[i]);                        \
    double yi = half * (y1[i] + y2[i] - y3[i] - y4[i]);                        \
    double yj = half * (y2[i] + y3[i] - y4[i] - y1[i]);                        \
    double fxi = half * (fx1[i] + fx2[i] - fx3[i] - fx4[i]);                   \
    double fxj = half * (fx2[i] + fx3[i] - fx4[i] - fx1[i]);                   \
    double fyi = half * (fy1[i] + fy2[i] - fy3[i] - fy4[i]);                   \
    double fyj = half * (fy2[i] + fy3[i] - fy4[i] - fy1[i]);                   \
    double rarea = 1.0 / (xi * yj - xj * yi + ptiny);                          \
    double dfxdx = rarea * (fxi * yj - fxj * yi);                              \
    double dfydy = rarea * (fyj * xi - fyi * xj);                              \
    double affine = (fy1[i] + fy2[i] + fy3[i] + fy4[i]) /                      \
                    (y1[i] + y2[i] + y3[i] + y4[i]);                           \
    div[i] = dfxdx + dfydy + affine;                                           \
  } while (0)

void oracle_del_dot_vec_2d_rep(const double* x, const double* y,
                               const double* xdot, const double* ydot,
                               double* div, const int64_t* real_zones,
                               int64_t nzones, int64_t jp, double ptiny,
                               double half) {
  for (idx_t ii = 0; ii < nzones; ++ii) DDV_BODY(ii);
}

/* DEL_DOT_VEC_2D.cpp:28-107, DEL_DOT_VEC_2D-Seq.cpp:24-45 */
static void run_del_dot_vec_2d(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 1000 * 1000);
  idx_t rzmax = (idx_t)(sqrt((double)target) + 1 + sqrt(2.0) - 1);
  adomain d = make_domain(rzmax, 2);
  idx_t len = d.nnalls, nz = d.n_real_zones, jp = d.jp;
  double ptiny = 1.0e-20, half = 0.5, t0;
  double *x = alloc_const(c, len, 0.0), *y = alloc_const(c, len, 0.0);
  int64_t* real_zones = alloc_const_idx(c, nz, -1);
  double *xdot = NULL, *ydot = NULL, *div = NULL;
  CHECK_ALLOC(x); CHECK_ALLOC(y); CHECK_ALLOC(real_zones);
  set_mesh_2d(x, 0.2, y, 0.1, &d, c->o);
  set_real_zones_2d(real_zones, &d);
  xdot = alloc_init(c, len);
  ydot = alloc_init(c, len);
  div = alloc_const(c, len, 0.0);
  CHECK_ALLOC(xdot); CHECK_ALLOC(ydot); CHECK_ALLOC(div);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t ii = 0; ii < nz; ++ii) DDV_BODY(ii);
  }
  set_result(r, checksum_ld(div, len, 1.0), nz, reps, nz, 1,
             8 * nz + 4 * 8 * d.n_real_nodes + 8 * nz, 54 * nz, now_s() - t0);
done:
  free(x); free(y); free(real_zones); free(xdot); free(ydot); free(div);
}

/* VOL3D.hpp:88-146 -- the macro body, with its four accumulation blocks. */
#define VOL3D_BODY(i)                                                           \
  do {                                                                          \
    const double *x0 = x, *x1 = x0 + 1, *x2 = x0 + jp, *x3 = x1 + jp,           \
                 *x4 = x0 + kp, *x5 = x1 + kp, *x6 = x2 + kp, *x7 = x3 + kp;     \
    const double *y0 = y, *y1 = y0 + 1, *y2 = y0 + jp, *y3 = y1 + jp,           \
                 *y4 = y0 + kp, *y5 = y1 + kp, *y6 = y2 + kp, *y7 = y3 + kp;     \
    const double *z0 = z, *z1 = z0 + 1, *z2 = z0 + jp, *z3 = z1 + jp,           \
                 *z4 = z0 + kp, *z5 = z1 + kp, *z6 = z2 + kp, *z7 = z3 + kp;     \
    double x71 = x7[i] - x1[i], x72 = x7[i] - x2[i], x74 = x7[i] - x4[i];      \
    double x30 = x3[i] - x0[i], x50 = x5[i] - x0[i], x60 = x6[i] - x0[i];      \
    double y71 = y7[i] - y1[i], y72 = y7[i] - y2[i], y74 = y7[i] - y4[i];      \
    double y30 = y3[i] - y0[i], y50 = y5[i] - y0[i], y60 = y6[i] - y0[i];      \
    double z71 = z7[i] - z1[i], z72 = z7[i] - z2[i], z74 = z7[i] - z4[i];      \
    double z30 = z3[i] - z0[i], z50 = z5[i] - z0[i], z60 = z6[i] - z0[i];      \
    double xps = x71 + x60, yps = y71 + y60, zps = z71 + z60;                  \
    double cyz = y72 * z30 - z72 * y30;                                         \
    double czx = z72 * x30 - x72 * z30;                                         \
    double cxy = x72 * y30 - y72 * x30;                                         \
    vol[i] = xps * cyz + yps * czx + zps * cxy;                                 \
    xps = x72 + x50; yps = y72 + y50; zps = z72 + z50;                          \
    cyz = y74 * z60 - z74 * y60;                                                \
    czx = z74 * x60 - x74 * z60;                                                \
    cxy = x74 * y60 - y74 * x60;                                                \
    vol[i] += xps * cyz + yps * czx + zps * cxy;                                \
    xps = x74 + x30; yps = y74 + y30; zps = z74 + z30;                          \
    cyz = y74 * z60 - z74 * y60;                                                \
    czx = z74 * x60 - x74 * z60;                                                \
    cxy = x74 * y60 - y74 * x60;                                                \
    vol[i] += xps * cyz + yps * czx + zps * cxy;                                \
    xps = x74 + x30; yps = y74 + y30; zps = z74 + z30;                          \
    cyz = y71 * z50 - z71 * y50;                                                \
    czx = z71 * x50 - x71 * z50;                                                \
    cxy = x71 * y50 - y71 * x50;                                                \
    vol[i] += xps * cyz + yps * czx + zps * cxy;                                \
    vol[i] *= vnormq;                                                           \
  } while (0)

void oracle_vol3d_rep(const double* x, const double* y, const double* z,
                      double* vol, double vnormq, int64_t jp, int64_t kp,
                      int64_t ibegin, int64_t iend) {
  for (idx_t i = ibegin; i < iend; ++i) VOL3D_BODY(i);
}

/* VOL3D.cpp:28-104, VOL3D-Seq.cpp:23-39 */
static void run_vol3d(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 100 * 100 * 100);
  idx_t rzmax = (idx_t)(cbrt((double)target) + 1 + cbrt(3.0) - 1);
  adomain d = make_domain(rzmax, 3);
  idx_t len = d.nnalls, jp = d.jp, kp = d.kp, ib = d.fpz, ie = d.lpz + 1;
  double vnormq = 0.083333333333333333, t0;
  long double scale;
  double *x = alloc_const(c, len, 0.0), *y = alloc_const(c, len, 0.0),
         *z = alloc_const(c, len, 0.0), *vol = NULL;
  CHECK_ALLOC(x); CHECK_ALLOC(y); CHECK_ALLOC(z);
  set_mesh_3d(x, 0.3, y, 0.2, z, 0.1, &d);
  vol = alloc_const(c, len, 0.0);
  CHECK_ALLOC(vol);
  scale = (long double)0.001 * ((long double)1000000 / d.n_real_zones);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = ib; i < ie; ++i) VOL3D_BODY(i);
  }
  set_result(r, checksum_ld(vol, len, (double)scale), d.n_real_zones, reps, ie - ib, 1,
             3 * 8 * ((ie - ib) + 1 + jp + kp) + 8 * (ie - ib), 72 * (ie - ib),
             now_s() - t0);
done:
  free(x); free(y); free(z); free(vol);
}

/* ENERGY.hpp:111-178 (BODY1..6) */
void oracle_energy_rep(double* e_new, const double* e_old, const double* delvc,
                       const double* p_new, const double* p_old, double* q_new,
                       const double* q_old, const double* work,
                       const double* compHalfStep, const double* pHalfStep,
                       const double* bvc, const double* pbvc,
                       const double* ql_old, const double* qq_old,
                       const double* vnewc, double rho0, double e_cut,
                       double emin, double q_cut, int64_t n) {
  for (idx_t i = 0; i < n; ++i)
    e_new[i] = e_old[i] - 0.5 * delvc[i] * (p_old[i] + q_old[i]) + 0.5 * work[i];
  for (idx_t i = 0; i < n; ++i) {
    if (delvc[i] > 0.0) {
      q_new[i] = 0.0;
    } else {
      double vhalf = 1.0 / (1.0 + compHalfStep[i]);
      double ssc = (pbvc[i] * e_new[i] + vhalf * vhalf * bvc[i] * pHalfStep[i]) / rho0;
      if (ssc <= 0.1111111e-36) ssc = 0.3333333e-18;
      else ssc = sqrt(ssc);
      q_new[i] = (ssc * ql_old[i] + qq_old[i]);
    }
  }
  for (idx_t i = 0; i < n; ++i)
    e_new[i] = e_new[i] + 0.5 * delvc[i] *
                              (3.0 * (p_old[i] + q_old[i]) - 4.0 * (pHalfStep[i] + q_new[i]));
  for (idx_t i = 0; i < n; ++i) {
    e_new[i] += 0.5 * work[i];
    if (fabs(e_new[i]) < e_cut) e_new[i] = 0.0;
    if (e_new[i] < emin) e_new[i] = emin;
  }
  for (idx_t i = 0; i < n; ++i) {
    double q_tilde;
    if (delvc[i] > 0.0) {
      q_tilde = 0.;
    } else {
      double ssc = (pbvc[i] * e_new[i] + vnewc[i] * vnewc[i] * bvc[i] * p_new[i]) / rho0;
      if (ssc <= 0.1111111e-36) ssc = 0.3333333e-18;
      else ssc = sqrt(ssc);
      q_tilde = (ssc * ql_old[i] + qq_old[i]);
    }
    e_new[i] = e_new[i] - (7.0 * (p_old[i] + q_old[i]) - 8.0 * (pHalfStep[i] + q_new[i]) +
                           (p_new[i] + q_tilde)) * delvc[i] / 6.0;
    if (fabs(e_new[i]) < e_cut) e_new[i] = 0.0;
    if (e_new[i] < emin) e_new[i] = emin;
  }
  for (idx_t i = 0; i < n; ++i) {
    if (delvc[i] <= 0.0) {
      double ssc = (pbvc[i] * e_new[i] + vnewc[i] * vnewc[i] * bvc[i] * p_new[i]) / rho0;
      if (ssc <= 0.1111111e-36) ssc = 0.3333333e-18;
      else ssc = sqrt(ssc);
      q_new[i] = (ssc * ql_old[i] + qq_old[i]);
      if (fabs(q_new[i]) < q_cut) q_new[i] = 0.0;
    }
  }
}

/* ENERGY.cpp:24-112, ENERGY-Seq.cpp:24-76 */
static void run_energy(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *e_new = alloc_const(c, n, 0.0), *e_old = alloc_init(c, n),
         *delvc = alloc_init(c, n), *p_new = alloc_init(c, n), *p_old = alloc_init(c, n),
         *q_new = alloc_const(c, n, 0.0), *q_old = alloc_init(c, n),
         *work = alloc_init(c, n), *compHalfStep = alloc_init(c, n),
         *pHalfStep = alloc_init(c, n), *bvc = alloc_init(c, n), *pbvc = alloc_init(c, n),
         *ql_old = alloc_init(c, n), *qq_old = alloc_init(c, n), *vnewc = alloc_init(c, n);
  double rho0 = init_scalar(c), e_cut = init_scalar(c), emin = init_scalar(c),
         q_cut = init_scalar(c), t0;
  long double ck;
  CHECK_ALLOC(e_new); CHECK_ALLOC(e_old); CHECK_ALLOC(delvc); CHECK_ALLOC(p_new);
  CHECK_ALLOC(p_old); CHECK_ALLOC(q_new); CHECK_ALLOC(q_old); CHECK_ALLOC(work);
  CHECK_ALLOC(compHalfStep); CHECK_ALLOC(pHalfStep); CHECK_ALLOC(bvc);
  CHECK_ALLOC(pbvc); CHECK_ALLOC(ql_old); CHECK_ALLOC(qq_old); CHECK_ALLOC(vnewc);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    if (!PAR) {
      oracle_energy_rep(e_new, e_old, delvc, p_new, p_old, q_new, q_old, work,
                        compHalfStep, pHalfStep, bvc, pbvc, ql_old, qq_old, vnewc,
                        rho0, e_cut, emin, q_cut, n);
      continue;
    }
    /* Base_OpenMP: the same six loops, each parallel (ENERGY-OMP.cpp). */
    #pragma omp parallel num_threads(NT)
    {
      #pragma omp for
      for (idx_t i = 0; i < n; ++i)
        e_new[i] = e_old[i] - 0.5 * delvc[i] * (p_old[i] + q_old[i]) + 0.5 * work[i];
      #pragma omp for
      for (idx_t i = 0; i < n; ++i) {
        if (delvc[i] > 0.0) {
          q_new[i] = 0.0;
        } else {
          double vhalf = 1.0 / (1.0 + compHalfStep[i]);
          double ssc = (pbvc[i] * e_new[i] + vhalf * vhalf * bvc[i] * pHalfStep[i]) / rho0;
          if (ssc <= 0.1111111e-36) ssc = 0.3333333e-18;
          else ssc = sqrt(ssc);
          q_new[i] = (ssc * ql_old[i] + qq_old[i]);
        }
      }
      #pragma omp for
      for (idx_t i = 0; i < n; ++i)
        e_new[i] = e_new[i] + 0.5 * delvc[i] *
                                  (3.0 * (p_old[i] + q_old[i]) - 4.0 * (pHalfStep[i] + q_new[i]));
      #pragma omp for
      for (idx_t i = 0; i < n; ++i) {
        e_new[i] += 0.5 * work[i];
        if (fabs(e_new[i]) < e_cut) e_new[i] = 0.0;
        if (e_new[i] < emin) e_new[i] = emin;
      }
      #pragma omp for
      for (idx_t i = 0; i < n; ++i) {
        double q_tilde;
        if (delvc[i] > 0.0) {
          q_tilde = 0.;
        } else {
          double ssc = (pbvc[i] * e_new[i] + vnewc[i] * vnewc[i] * bvc[i] * p_new[i]) / rho0;
          if (ssc <= 0.1111111e-36) ssc = 0.3333333e-18;
          else ssc = sqrt(ssc);
          q_tilde = (ssc * ql_old[i] + qq_old[i]);
        }
        e_new[i] = e_new[i] - (7.0 * (p_old[i] + q_old[i]) - 8.0 * (pHalfStep[i] + q_new[i]) +
                               (p_new[i] + q_tilde)) * delvc[i] / 6.0;
        if (fabs(e_new[i]) < e_cut) e_new[i] = 0.0;
        if (e_new[i] < emin) e_new[i] = emin;
      }
      #pragma omp for
      for (idx_t i = 0; i < n; ++i) {
        if (delvc[i] <= 0.0) {
          double ssc = (pbvc[i] * e_new[i] + vnewc[i] * vnewc[i] * bvc[i] * p_new[i]) / rho0;
          if (ssc <= 0.1111111e-36) ssc = 0.3333333e-18;
          else ssc = sqrt(ssc);
          q_new[i] = (ssc * ql_old[i] + qq_old[i]);
          if (fabs(q_new[i]) < q_cut) q_new[i] = 0.0;
        }
      }
    }
  }
  t0 = now_s() - t0;
  ck = checksum_ld(e_new, n, 1.0);
  ck += checksum_ld(q_new, n, 1.0);
  set_result(r, ck, n, reps, 6 * n, 6, (5 + 1 + 6 + 2 + 7 + 1) * 8 * n + 5 * 8 * n,
             (6 + 11 + 8 + 2 + 19 + 9) * n, t0);
done:
  free(e_new); free(e_old); free(delvc); free(p_new); free(p_old); free(q_new);
  free(q_old); free(work); free(compHalfStep); free(pHalfStep); free(bvc);
  free(pbvc); free(ql_old); free(qq_old); free(vnewc);
}

/* PRESSURE.cpp:24-86, PRESSURE.hpp:39-46 */
static void run_pressure(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *compression = alloc_init(c, n), *bvc = alloc_init(c, n),
         *p_new = alloc_const(c, n, 0.0), *e_old = alloc_init(c, n), *vnewc = alloc_init(c, n);
  double cls = init_scalar(c), p_cut = init_scalar(c), pmin = init_scalar(c),
         eosvmax = init_scalar(c), t0;
  CHECK_ALLOC(compression); CHECK_ALLOC(bvc); CHECK_ALLOC(p_new); CHECK_ALLOC(e_old);
  CHECK_ALLOC(vnewc);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) bvc[i] = cls * (compression[i] + 1.0);
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) {
      p_new[i] = bvc[i] * e_old[i];
      if (fabs(p_new[i]) < p_cut) p_new[i] = 0.0;
      if (vnewc[i] >= eosvmax) p_new[i] = 0.0;
      if (p_new[i] < pmin) p_new[i] = pmin;
    }
  }
  set_result(r, checksum_ld(p_new, n, 1.0), n, reps, 2 * n, 2, 32 * n + 16 * n, 3 * n,
             now_s() - t0);
done:
  free(compression); free(bvc); free(p_new); free(e_old); free(vnewc);
}

/* ------------------------------------------------------------------------ */
/* Polybench                                                                 */
/* ------------------------------------------------------------------------ */

/* POLYBENCH_JACOBI_2D.hpp:38-44, -Seq.cpp:20-45 */
void oracle_jacobi_2d(double* A, double* B, int64_t N, int64_t tsteps) {
  for (idx_t t = 0; t < tsteps; ++t) {
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        B[j + i * N] = 0.2 * (A[j + i * N] + A[j - 1 + i * N] + A[j + 1 + i * N] +
                              A[j + (i + 1) * N] + A[j + (i - 1) * N]);
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        A[j + i * N] = 0.2 * (B[j + i * N] + B[j - 1 + i * N] + B[j + 1 + i * N] +
                              B[j + (i + 1) * N] + B[j + (i - 1) * N]);
  }
}

static void jacobi_2d_par(ctx* c, double* A, double* B, idx_t N, idx_t tsteps) {
  for (idx_t t = 0; t < tsteps; ++t) {
    OMP_FOR
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        B[j + i * N] = 0.2 * (A[j + i * N] + A[j - 1 + i * N] + A[j + 1 + i * N] +
                              A[j + (i + 1) * N] + A[j + (i - 1) * N]);
    OMP_FOR
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        A[j + i * N] = 0.2 * (B[j + i * N] + B[j - 1 + i * N] + B[j + 1 + i * N] +
                              B[j + (i + 1) * N] + B[j + (i - 1) * N]);
  }
}

/* POLYBENCH_JACOBI_2D.cpp:26-94 */
static void run_jacobi_2d(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 1000 * 1000);
  idx_t N = (idx_t)(sqrt((double)target) + 2 + sqrt(2.0) - 1);
  idx_t tsteps = c->o->tsteps >= 0 ? c->o->tsteps : 40;
  idx_t NN = N * N;
  long double scale = (long double)0.0001 * ((long double)1000000 / ((N - 2) * (N - 2))), ck;
  double *Ainit = alloc_init(c, NN), *Binit = alloc_init(c, NN);
  double *A = alloc_raw(NN), *B = alloc_raw(NN), t0;
  CHECK_ALLOC(Ainit); CHECK_ALLOC(Binit); CHECK_ALLOC(A); CHECK_ALLOC(B);
  memcpy(A, Ainit, sizeof(double) * NN);
  memcpy(B, Binit, sizeof(double) * NN);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    if (PAR) jacobi_2d_par(c, A, B, N, tsteps);
    else oracle_jacobi_2d(A, B, N, tsteps);
  }
  t0 = now_s() - t0;
  ck = checksum_ld(A, NN, (double)scale);
  ck += checksum_ld(B, NN, (double)scale);
  set_result(r, ck, (N - 2) * (N - 2), reps, tsteps * 2 * (N - 2) * (N - 2), 2,
             (8 * (NN - 4) * 2 + 8 * (N - 2) * (N - 2) * 2) * tsteps,
             tsteps * 10 * (N - 2) * (N - 2), t0);
done:
  free(Ainit); free(Binit); free(A); free(B);
}

/* POLYBENCH_HEAT_3D.hpp:47-82, -Seq.cpp */
#define HEAT_BODY(D, S)                                                         \
  D[k + N * (j + N * i)] =                                                      \
      0.125 * (S[k + N * (j + N * (i + 1))] - 2.0 * S[k + N * (j + N * i)] +    \
               S[k + N * (j + N * (i - 1))]) +                                  \
      0.125 * (S[k + N * (j + 1 + N * i)] - 2.0 * S[k + N * (j + N * i)] +      \
               S[k + N * (j - 1 + N * i)]) +                                    \
      0.125 * (S[k + 1 + N * (j + N * i)] - 2.0 * S[k + N * (j + N * i)] +      \
               S[k - 1 + N * (j + N * i)]) +                                    \
      S[k + N * (j + N * i)]

void oracle_heat_3d(double* A, double* B, int64_t N, int64_t tsteps) {
  for (idx_t t = 0; t < tsteps; ++t) {
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        for (idx_t k = 1; k < N - 1; ++k) HEAT_BODY(B, A);
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        for (idx_t k = 1; k < N - 1; ++k) HEAT_BODY(A, B);
  }
}

static void heat_3d_par(ctx* c, double* A, double* B, idx_t N, idx_t tsteps) {
  for (idx_t t = 0; t < tsteps; ++t) {
    OMP_FOR
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        for (idx_t k = 1; k < N - 1; ++k) HEAT_BODY(B, A);
    OMP_FOR
    for (idx_t i = 1; i < N - 1; ++i)
      for (idx_t j = 1; j < N - 1; ++j)
        for (idx_t k = 1; k < N - 1; ++k) HEAT_BODY(A, B);
  }
}

/* POLYBENCH_HEAT_3D.cpp:27-95 */
static void run_heat_3d(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 100 * 100 * 100);
  idx_t N = (idx_t)(cbrt((double)target) + 2 + cbrt(3.0) - 1);
  idx_t tsteps = c->o->tsteps >= 0 ? c->o->tsteps : 20;
  idx_t NNN = N * N * N, inner = (N - 2) * (N - 2) * (N - 2);
  long double scale = (long double)0.0001 * ((long double)1000000 / inner), ck;
  double *Ainit = alloc_init(c, NNN), *Binit = alloc_init(c, NNN);
  double *A = alloc_raw(NNN), *B = alloc_raw(NNN), t0;
  CHECK_ALLOC(Ainit); CHECK_ALLOC(Binit); CHECK_ALLOC(A); CHECK_ALLOC(B);
  memcpy(A, Ainit, sizeof(double) * NNN);
  memcpy(B, Binit, sizeof(double) * NNN);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    if (PAR) heat_3d_par(c, A, B, N, tsteps);
    else oracle_heat_3d(A, B, N, tsteps);
  }
  t0 = now_s() - t0;
  ck = checksum_ld(A, NNN, (double)scale);
  ck += checksum_ld(B, NNN, (double)scale);
  set_result(r, ck, inner, reps, tsteps * 2 * inner, tsteps * 2,
             (8 * (NNN - 12 * (N - 2) - 8) * 2 + 8 * inner * 2) * tsteps,
             tsteps * 30 * inner, t0);
done:
  free(Ainit); free(Binit); free(A); free(B);
}

/* POLYBENCH_FDTD_2D.hpp:52-69, -Seq.cpp:20-57 */
void oracle_fdtd_2d(double* ex, double* ey, double* hz, const double* fict,
                    int64_t nx, int64_t ny, int64_t tsteps) {
  for (idx_t t = 0; t < tsteps; ++t) {
    for (idx_t j = 0; j < ny; j++) ey[j + 0 * ny] = fict[t];
    for (idx_t i = 1; i < nx; i++)
      for (idx_t j = 0; j < ny; j++)
        ey[j + i * ny] = ey[j + i * ny] - 0.5 * (hz[j + i * ny] - hz[j + (i - 1) * ny]);
    for (idx_t i = 0; i < nx; i++)
      for (idx_t j = 1; j < ny; j++)
        ex[j + i * ny] = ex[j + i * ny] - 0.5 * (hz[j + i * ny] - hz[j - 1 + i * ny]);
    for (idx_t i = 0; i < nx - 1; i++)
      for (idx_t j = 0; j < ny - 1; j++)
        hz[j + i * ny] = hz[j + i * ny] - 0.7 * (ex[j + 1 + i * ny] - ex[j + i * ny] +
                                                 ey[j + (i + 1) * ny] - ey[j + i * ny]);
  }
}

static void fdtd_2d_par(ctx* c, double* ex, double* ey, double* hz, const double* fict,
                        idx_t nx, idx_t ny, idx_t tsteps) {
  for (idx_t t = 0; t < tsteps; ++t) {
    OMP_FOR
    for (idx_t j = 0; j < ny; j++) ey[j + 0 * ny] = fict[t];
    OMP_FOR
    for (idx_t i = 1; i < nx; i++)
      for (idx_t j = 0; j < ny; j++)
        ey[j + i * ny] = ey[j + i * ny] - 0.5 * (hz[j + i * ny] - hz[j + (i - 1) * ny]);
    OMP_FOR
    for (idx_t i = 0; i < nx; i++)
      for (idx_t j = 1; j < ny; j++)
        ex[j + i * ny] = ex[j + i * ny] - 0.5 * (hz[j + i * ny] - hz[j - 1 + i * ny]);
    OMP_FOR
    for (idx_t i = 0; i < nx - 1; i++)
      for (idx_t j = 0; j < ny - 1; j++)
        hz[j + i * ny] = hz[j + i * ny] - 0.7 * (ex[j + 1 + i * ny] - ex[j + i * ny] +
                                                 ey[j + (i + 1) * ny] - ey[j + i * ny]);
  }
}

/* POLYBENCH_FDTD_2D.cpp:30-116 */
static void run_fdtd_2d(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 999 * 1000);
  idx_t nx = (idx_t)(sqrt((double)target) + 1 + sqrt(2.0) - 1), ny = nx;
  idx_t tsteps = c->o->tsteps >= 0 ? c->o->tsteps : 40;
  idx_t actual = (nx - 1) * ny > nx * (ny - 1) ? (nx - 1) * ny : nx * (ny - 1);
  long double scale = (long double)0.001 * ((long double)999000 / actual);
  double *hz = alloc_const(c, nx * ny, 0.0), *ex = alloc_init(c, nx * ny),
         *ey = alloc_init(c, nx * ny), *fict = alloc_init(c, tsteps), t0;
  CHECK_ALLOC(hz); CHECK_ALLOC(ex); CHECK_ALLOC(ey); CHECK_ALLOC(fict);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    if (PAR) fdtd_2d_par(c, ex, ey, hz, fict, nx, ny, tsteps);
    else oracle_fdtd_2d(ex, ey, hz, fict, nx, ny, tsteps);
  }
  set_result(r, checksum_ld(hz, nx * ny, (double)scale), actual, reps,
             tsteps * (ny + (nx - 1) * ny + nx * (ny - 1) + (nx - 1) * (ny - 1)), tsteps * 4,
             (8 + 8 * (nx - 1) * ny + 8 * nx * ny + 8 * nx * (ny - 1) + 8 * nx * ny +
              8 * (nx - 1) * (ny - 1) + 8 * (nx - 1) * ny + 8 * nx * (ny - 1)) * tsteps +
                 (8 * ny + 8 * (nx - 1) * ny + 8 * nx * (ny - 1) + 8 * (nx - 1) * (ny - 1)) *
                     tsteps,
             tsteps * (3 * (nx - 1) * ny + 3 * nx * (ny - 1) + 5 * (nx - 1) * (ny - 1)),
             now_s() - t0);
done:
  free(hz); free(ex); free(ey); free(fict);
}

/* C = alpha * A * B + beta * C, plain FP64 (the split-precision reference). */
void oracle_gemm(const double* A, const double* B, double* C, int64_t ni,
                 int64_t nj, int64_t nk, double alpha, double beta) {
  for (idx_t i = 0; i < ni; ++i)
    for (idx_t j = 0; j < nj; ++j) {
      double dot = 0.0;
      for (idx_t k = 0; k < nk; ++k) dot += A[k + i * nk] * B[j + k * nj];
      C[j + i * nj] = alpha * dot + beta * C[j + i * nj];
    }
}

/* POLYBENCH_GEMM.hpp:40-56, .cpp:24-95, -Seq.cpp:20-45 (beta is dead: BODY2
 * scales C, BODY4 overwrites it) */
static void run_gemm(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 1000 * 1000);
  idx_t ni = (idx_t)(sqrt((double)target) + sqrt(2.0) - 1), nj = ni;
  idx_t nk = (idx_t)((double)1200 / 1000 * ni);
  double alpha = 0.62, beta = 1.002, t0;
  long double scale = (long double)0.001 * ((long double)1000000 / (ni * nj));
  double *A = alloc_init(c, ni * nk), *B = alloc_init(c, nk * nj),
         *C = alloc_const(c, ni * nj, 0.0);
  CHECK_ALLOC(A); CHECK_ALLOC(B); CHECK_ALLOC(C);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < ni; ++i)
      for (idx_t j = 0; j < nj; ++j) {
        double dot = 0.0;
        C[j + i * nj] *= beta;
        for (idx_t k = 0; k < nk; ++k) dot += alpha * A[k + i * nk] * B[j + k * nj];
        C[j + i * nj] = dot;
      }
  }
  set_result(r, checksum_ld(C, ni * nj, (double)scale), ni * nj, reps, ni * nj, 1,
             8 * ni * nk + 8 * nj * nk + 8 * ni * nj, (1 + 3 * nk) * ni * nj, now_s() - t0);
done:
  free(A); free(B); free(C);
}

/* POLYBENCH_3MM.hpp:61-86, .cpp:28-117, -Seq.cpp:31-64 */
static void run_3mm(ctx* c, oracle_result* r) {
  idx_t reps = c->o->reps;
  idx_t target = target_size(c, 1000 * 1000);
  idx_t ni = (idx_t)(sqrt((double)target) + sqrt(2.0) - 1), nj = ni, nl = ni;
  idx_t nk = (idx_t)((double)1010 / 1000 * ni), nm = (idx_t)((double)1200 / 1000 * ni);
  idx_t actual = ni * nj;
  long double scale;
  double *A = alloc_init(c, ni * nk), *B = alloc_init(c, nk * nj), *C = alloc_init(c, nj * nm),
         *D = alloc_init(c, nm * nl), *E = alloc_const(c, ni * nj, 0.0),
         *F = alloc_const(c, nj * nl, 0.0), *G = alloc_const(c, ni * nl, 0.0), t0;
  if (nj * nl > actual) actual = nj * nl;
  if (ni * nl > actual) actual = ni * nl;
  scale = (long double)0.000000001 * ((long double)1000000 / actual);
  CHECK_ALLOC(A); CHECK_ALLOC(B); CHECK_ALLOC(C); CHECK_ALLOC(D);
  CHECK_ALLOC(E); CHECK_ALLOC(F); CHECK_ALLOC(G);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < ni; i++)
      for (idx_t j = 0; j < nj; j++) {
        double dot = 0.0;
        for (idx_t k = 0; k < nk; k++) dot += A[k + i * nk] * B[j + k * nj];
        E[j + i * nj] = dot;
      }
    OMP_FOR
    for (idx_t j = 0; j < nj; j++)
      for (idx_t l = 0; l < nl; l++) {
        double dot = 0.0;
        for (idx_t m = 0; m < nm; m++) dot += C[m + j * nm] * D[l + m * nl];
        F[l + j * nl] = dot;
      }
    OMP_FOR
    for (idx_t i = 0; i < ni; i++)
      for (idx_t l = 0; l < nl; l++) {
        double dot = 0.0;
        for (idx_t j = 0; j < nj; j++) dot += E[j + i * nj] * F[l + j * nl];
        G[l + i * nl] = dot;
      }
  }
  set_result(r, checksum_ld(G, ni * nl, (double)scale), actual, reps,
             ni * nj + nj * nl + ni * nl, 3,
             8 * (ni * nk + nj * nk + nj * nm + nl * nm + ni * nj + nj * nl) +
                 8 * (ni * nj + nj * nl + ni * nl),
             2 * ni * nj * nk + 2 * nj * nl * nm + 2 * ni * nj * nl, now_s() - t0);
done:
  free(A); free(B); free(C); free(D); free(E); free(F); free(G);
}

/* ------------------------------------------------------------------------ */
/* Algorithm                                                                 */
/* ------------------------------------------------------------------------ */

/* SCAN.hpp:23-36 (exclusive scan), SCAN-Seq.cpp:31-42 */
void oracle_scan_f64(const double* x, double* y, int64_t n) {
  double scan_var = 0.0;
  for (idx_t i = 0; i < n; ++i) {
    y[i] = scan_var;
    scan_var += x[i];
  }
}

void oracle_scan_i64(const int64_t* x, int64_t* y, int64_t n) {
  int64_t scan_var = 0;
  for (idx_t i = 0; i < n; ++i) {
    y[i] = scan_var;
    scan_var += x[i];
  }
}

/* SCAN-OMP.cpp Base_OpenMP: per-thread chunk scans, then offsets. */
static void scan_f64_par(ctx* c, const double* x, double* y, idx_t n) {
  int p0 = NT < n ? NT : (int)(n > 0 ? n : 1);
  double* sums = (double*)calloc((size_t)p0, sizeof(double));
  #pragma omp parallel num_threads(p0)
  {
    int p = 1, pid = 0;
#ifdef _OPENMP
    p = omp_get_num_threads();
    pid = omp_get_thread_num();
#endif
    idx_t step = n / p;
    idx_t lb = pid * step, le = (pid == p - 1) ? n : (pid + 1) * step;
    double local = 0.0;
    for (idx_t i = lb; i < le; ++i) { y[i] = local; local += x[i]; }
    sums[pid] = local;
    #pragma omp barrier
    if (pid != 0) {
      double prev = 0;
      for (int ip = 0; ip < pid; ++ip) prev += sums[ip];
      for (idx_t i = lb; i < le; ++i) y[i] += prev;
    }
  }
  free(sums);
}

static void scan_i64_par(ctx* c, const int64_t* x, int64_t* y, idx_t n) {
  int p0 = NT < n ? NT : (int)(n > 0 ? n : 1);
  int64_t* sums = (int64_t*)calloc((size_t)p0, sizeof(int64_t));
  #pragma omp parallel num_threads(p0)
  {
    int p = 1, pid = 0;
#ifdef _OPENMP
    p = omp_get_num_threads();
    pid = omp_get_thread_num();
#endif
    idx_t step = n / p;
    idx_t lb = pid * step, le = (pid == p - 1) ? n : (pid + 1) * step;
    int64_t local = 0;
    for (idx_t i = lb; i < le; ++i) { y[i] = local; local += x[i]; }
    sums[pid] = local;
    #pragma omp barrier
    if (pid != 0) {
      int64_t prev = 0;
      for (int ip = 0; ip < pid; ++ip) prev += sums[ip];
      for (idx_t i = lb; i < le; ++i) y[i] += prev;
    }
  }
  free(sums);
}

/* SCAN.cpp:24-77.  variant 1: int64 values uniform in [0,100) from the
 * seed, exact prefix sums (not in the suite; the integer form of the scan). */
static void run_scan(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  long double scale = (long double)1e-2 * ((long double)1000000 / n) / n;
  double t0;
  if (c->o->variant == 1) {
    int64_t* x = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t* y = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!x || !y) { free(x); free(y); r->status = 3; return; }
    oracle_init_uniform_i64(x, n, c->o->seed, (uint64_t)c->count, 0, 100);
    c->count++;
    for (idx_t i = 0; i < n; ++i) y[i] = 0;
    c->count++;
    t0 = now_s();
    for (idx_t irep = 0; irep < reps; ++irep) {
      if (PAR) scan_i64_par(c, x, y, n);
      else oracle_scan_i64(x, y, n);
    }
    t0 = now_s() - t0;
    set_result(r, checksum_ld_i64(y, n, (double)scale), n, reps, n, 1, 16 * n, n, t0);
    free(x); free(y);
    return;
  }
  {
    double *x = alloc_randvalue(c, n), *y = alloc_const(c, n, 0.0);
    CHECK_ALLOC(x); CHECK_ALLOC(y);
    t0 = now_s();
    for (idx_t irep = 0; irep < reps; ++irep) {
      if (PAR) scan_f64_par(c, x, y, n);
      else oracle_scan_f64(x, y, n);
    }
    set_result(r, checksum_ld(y, n, (double)scale), n, reps, n, 1, 16 * n, n, now_s() - t0);
  done:
    free(x); free(y);
  }
}

/* REDUCE_SUM.cpp:24-76, REDUCE_SUM-Seq.cpp:34-48 */
static void run_reduce_sum(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double* x = alloc_init(c, n);
  double m_sum = 0.0, m_sum_init = 0.0, t0;
  CHECK_ALLOC(x);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    double sum = m_sum_init;
    if (PAR) {
      #pragma omp parallel for reduction(+:sum) num_threads(NT)
      for (idx_t i = 0; i < n; ++i) sum += x[i];
    } else {
      for (idx_t i = 0; i < n; ++i) sum += x[i];
    }
    m_sum = sum;
  }
  t0 = now_s() - t0;
  set_result(r, checksum_ld(&m_sum, 1, 1.0), n, reps, n, 1, 8 * (1 + n) + 8, n, t0);
done:
  free(x);
}

/* ------------------------------------------------------------------------ */
/* Algorithm MEMSET / MEMCPY / HISTOGRAM, Basic INDEXLIST / MULTI_REDUCE      */
/* ------------------------------------------------------------------------ */

/* MEMSET.cpp:22-75, MEMSET.hpp:27-28 */
static void run_memset(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double* x = alloc_const(c, n, -1.234567e89);
  double val = 0.0, t0;
  CHECK_ALLOC(x);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) x[i] = val;
  }
  set_result(r, checksum_ld(x, n, 1.0), n, reps, n, 1, 8 * n, 0, now_s() - t0);
done:
  free(x);
}

/* MEMCPY.cpp:22-75, MEMCPY.hpp:27-28 */
static void run_memcpy(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double *x = alloc_const(c, n, 0.0), *y = alloc_const(c, n, -1.234567e89), t0;
  CHECK_ALLOC(x); CHECK_ALLOC(y);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    OMP_FOR
    for (idx_t i = 0; i < n; ++i) y[i] = x[i];
  }
  set_result(r, checksum_ld(y, n, 1.0), n, reps, n, 1, 16 * n, 0, now_s() - t0);
done:
  free(x); free(y);
}

/* INDEXLIST.cpp:22-80, INDEXLIST.hpp:28-34, INDEXLIST-Seq.cpp; with
 * three_loop, INDEXLIST_3LOOP.cpp:22-92 (counts, their exclusive scan and the
 * list from count changes: the same list and length). */
static void run_indexlist_any(ctx* c, oracle_result* r, int three_loop) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  double* x = alloc_randsign(c, n);
  int* list = alloc_int(c, n);
  idx_t* counts = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n + 1));
  idx_t len = -1;
  double t0;
  CHECK_ALLOC(x); CHECK_ALLOC(list); CHECK_ALLOC(counts);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    if (!three_loop) {
      idx_t count = 0;
      for (idx_t i = 0; i < n; ++i)
        if (x[i] < 0.0) list[count++] = (int)i;
      len = count;
    } else {
      for (idx_t i = 0; i < n; ++i) counts[i] = (x[i] < 0.0) ? 1 : 0;
      idx_t count = 0;
      for (idx_t i = 0; i < n + 1; ++i) {
        idx_t inc = (i < n) ? counts[i] : 0;
        counts[i] = count;
        count += inc;
      }
      for (idx_t i = 0; i < n; ++i)
        if (counts[i] != counts[i + 1]) list[counts[i]] = (int)i;
      len = counts[n];
    }
  }
  t0 = now_s() - t0;
  if (!three_loop) {
    set_result(r, checksum_ld_int(list, n, 1.0) + (long double)len, n, reps, n, 1,
               8 + 8 * n + 8 + 4 * n / 2, 0, t0);
  } else {
    set_result(r, checksum_ld_int(list, n, 1.0) + (long double)len, n, reps, 3 * n + 1, 3,
               8 * n + 8 + 8 * (n + 1) + 8 * (n + 1) +
                   (8 * n + 8 + 8 * (n + 1) + 4 * (n + 1) / 2),
               0, t0);
  }
done:
  free(x); free(list); free(counts);
}

static void run_indexlist(ctx* c, oracle_result* r) { run_indexlist_any(c, r, 0); }
static void run_indexlist_3loop(ctx* c, oracle_result* r) { run_indexlist_any(c, r, 1); }

static int64_t bins_of(const ctx* c) { return c->o->num_bins > 0 ? c->o->num_bins : 10; }
static int bin_algo_of(const ctx* c) {
  return (c->o->bin_algo >= 0 && c->o->bin_algo <= 3) ? c->o->bin_algo : 1;
}

/* HISTOGRAM.cpp:24-149, HISTOGRAM.hpp:37-64, HISTOGRAM-Seq.cpp */
static void run_histogram(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  int64_t nb = bins_of(c);
  int64_t* bins = assign_bins(c, n, nb, bin_algo_of(c));
  unsigned long long* counts = (unsigned long long*)calloc((size_t)nb, sizeof(unsigned long long));
  double t0;
  CHECK_ALLOC(bins); CHECK_ALLOC(counts);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    for (int64_t b = 0; b < nb; ++b) counts[b] = 0ull;  /* counts_init */
    for (idx_t i = 0; i < n; ++i) counts[bins[i]] += 1ull;
  }
  set_result(r, checksum_ld_u64(counts, nb, 1.0), n, reps, n, 1, 8 * nb + 8 * n + 8 * nb, n,
             now_s() - t0);
done:
  free(bins); free(counts);
}

/* MULTI_REDUCE.cpp:24-153, MULTI_REDUCE.hpp:38-65, MULTI_REDUCE-Seq.cpp */
static void run_multi_reduce(ctx* c, oracle_result* r) {
  idx_t n = target_size(c, 1000000), reps = c->o->reps;
  int64_t nb = bins_of(c);
  double* data = alloc_randvalue(c, n);
  int64_t* bins = assign_bins(c, n, nb, bin_algo_of(c));
  double* values = (double*)calloc((size_t)nb, sizeof(double));
  double t0;
  CHECK_ALLOC(data); CHECK_ALLOC(bins); CHECK_ALLOC(values);
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    for (int64_t b = 0; b < nb; ++b) values[b] = 0.0;  /* values_init */
    for (idx_t i = 0; i < n; ++i) values[bins[i]] += data[i];
  }
  set_result(r, checksum_ld(values, nb, 1.0), n, reps, n, 1, 8 * nb + 8 * n + 8 * n + 8 * nb,
             n, now_s() - t0);
done:
  free(data); free(bins); free(values);
}

/* ------------------------------------------------------------------------ */
/* Comm HALO_PACKING / HALO_PACKING_FUSED (one rank)                           */
/* ------------------------------------------------------------------------ */

/* comm/HALO_base.cpp:80-116 */
static const int kHaloOffsets[26][3] = {
    {-1, 0, 0},   {1, 0, 0},   {0, -1, 0},  {0, 1, 0},   {0, 0, -1},  {0, 0, 1},
    {-1, -1, 0},  {-1, 1, 0},  {1, -1, 0},  {1, 1, 0},   {-1, 0, -1}, {-1, 0, 1},
    {1, 0, -1},   {1, 0, 1},   {0, -1, -1}, {0, -1, 1},  {0, 1, -1},  {0, 1, 1},
    {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},
    {1, 1, -1},   {1, 1, 1}};

/* comm/HALO_base.cpp:118-162 (send: the boundary layer; recv: the halo) */
static void halo_bounds(int off, int send, idx_t w, idx_t dim, idx_t* lo, idx_t* hi) {
  if (off == -1) { *lo = send ? w : 0; *hi = send ? 2 * w : w; }
  else if (off == 0) { *lo = w; *hi = w + dim; }
  else { *lo = send ? dim : w + dim; *hi = send ? w + dim : w + dim + w; }
}

/* comm/HALO_base.cpp:164-276: the list of one neighbour and direction */
static int* halo_list(const idx_t* gd, idx_t w, int l, int send, idx_t* len) {
  idx_t lo[3], hi[3];
  for (int d = 0; d < 3; ++d) halo_bounds(kHaloOffsets[l][d], send, w, gd[d], &lo[d], &hi[d]);
  idx_t js = gd[0] + 2 * w, ks = js * (gd[1] + 2 * w);
  *len = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
  int* list = (int*)malloc(sizeof(int) * (size_t)(*len > 0 ? *len : 1));
  if (!list) return NULL;
  idx_t k = 0;
  for (idx_t kk = lo[2]; kk < hi[2]; ++kk)
    for (idx_t jj = lo[1]; jj < hi[1]; ++jj)
      for (idx_t ii = lo[0]; ii < hi[0]; ++ii) list[k++] = (int)(ii + jj * js + kk * ks);
  return list;
}

/* HALO_PACKING.cpp:18-170, HALO_PACKING-Seq.cpp (Base_Seq, one rank, pack
 * and unpack buffers in the same space: no separate send/recv copies);
 * HALO_PACKING_FUSED only differs in its kernel count. */
static void run_halo_packing_any(ctx* c, oracle_result* r, int fused) {
  idx_t reps = c->o->reps;
  double target = c->o->size >= 0 ? c->o->size : 1000000.0;
  idx_t w = c->o->halo_width > 0 ? c->o->halo_width : 1;
  idx_t nv = c->o->halo_num_vars > 0 ? c->o->halo_num_vars : 3;
  double cbrt_run = cbrt(target) + cbrt(3.0) - 1.0;
  idx_t gd[3] = {(idx_t)cbrt_run, (idx_t)cbrt_run, (idx_t)cbrt_run};
  idx_t var_size = (gd[0] + 2 * w) * (gd[1] + 2 * w) * (gd[2] + 2 * w);
  idx_t actual = gd[0] * gd[1] * gd[1];
  int* plist[26] = {0};
  int* ulist[26] = {0};
  idx_t plen[26], ulen[26];
  double* vars[16] = {0};
  double* pbuf[26] = {0};
  double* ubuf[26] = {0};
  long double ck = 0.0L;
  double t0;
  int ok = nv <= 16;
  for (int l = 0; ok && l < 26; ++l) {
    plist[l] = halo_list(gd, w, l, 1, &plen[l]);
    c->count++;  /* allocAndInitData of the list, then overwritten */
    ulist[l] = halo_list(gd, w, l, 0, &ulen[l]);
    c->count++;
    ok = plist[l] && ulist[l];
  }
  for (idx_t v = 0; ok && v < nv; ++v) {
    vars[v] = alloc_raw(var_size);
    c->count++;  /* allocAndInitData, then var[i] = i + v */
    ok = vars[v] != NULL;
    for (idx_t i = 0; ok && i < var_size; ++i) vars[v][i] = (double)(i + v);
  }
  for (int l = 0; ok && l < 26; ++l) ok = (pbuf[l] = alloc_init(c, nv * plen[l])) != NULL;
  for (int l = 0; ok && l < 26; ++l) ok = (ubuf[l] = alloc_init(c, nv * ulen[l])) != NULL;
  if (!ok) { r->status = 3; goto done; }
  t0 = now_s();
  for (idx_t irep = 0; irep < reps; ++irep) {
    for (int l = 0; l < 26; ++l) {
      double* buffer = pbuf[l];
      for (idx_t v = 0; v < nv; ++v) {
        for (idx_t i = 0; i < plen[l]; ++i) buffer[i] = vars[v][plist[l][i]];
        buffer += plen[l];
      }
    }
    for (int l = 0; l < 26; ++l) {
      double* buffer = ubuf[l];
      for (idx_t v = 0; v < nv; ++v) {
        for (idx_t i = 0; i < ulen[l]; ++i) vars[v][ulist[l][i]] = buffer[i];
        buffer += ulen[l];
      }
    }
  }
  t0 = now_s() - t0;
  for (idx_t v = 0; v < nv; ++v) ck += checksum_ld(vars[v], var_size, 1.0);
  for (int l = 0; l < 26; ++l) ck += checksum_ld(pbuf[l], nv * plen[l], 1.0);
  {
    idx_t its = nv * (var_size - actual);
    set_result(r, ck, actual, reps, its, fused ? 2 : 2 * 26 * nv, 4 * its + 8 * its + 4 * its +
               8 * its + 8 * its + 8 * its, 0, t0);
  }
done:
  for (int l = 0; l < 26; ++l) { free(plist[l]); free(ulist[l]); free(pbuf[l]); free(ubuf[l]); }
  for (int v = 0; v < 16; ++v) free(vars[v]);
}

static void run_halo_packing(ctx* c, oracle_result* r) { run_halo_packing_any(c, r, 0); }
static void run_halo_packing_fused(ctx* c, oracle_result* r) { run_halo_packing_any(c, r, 1); }

/* ------------------------------------------------------------------------ */

typedef void (*runner_fn)(ctx*, oracle_result*);

static const struct {
  const char* name;
  runner_fn fn;
} kRunners[] = {
    {"Stream_COPY", run_copy},         {"Stream_MUL", run_mul},
    {"Stream_ADD", run_add},           {"Stream_TRIAD", run_triad},
    {"Stream_DOT", run_dot},           {"Basic_DAXPY", run_daxpy},
    {"Basic_INIT3", run_init3},        {"Basic_MULADDSUB", run_muladdsub},
    {"Lcals_HYDRO_1D", run_hydro_1d},  {"Lcals_HYDRO_2D", run_hydro_2d},
    {"Lcals_EOS", run_eos},            {"Lcals_FIRST_DIFF", run_first_diff},
    {"Lcals_INT_PREDICT", run_int_predict}, {"Lcals_FIRST_MIN", run_first_min},
    {"Lcals_DIFF_PREDICT", run_diff_predict}, {"Lcals_PLANCKIAN", run_planckian},
    {"Apps_DEL_DOT_VEC_2D", run_del_dot_vec_2d}, {"Apps_VOL3D", run_vol3d},
    {"Apps_ENERGY", run_energy},       {"Apps_PRESSURE", run_pressure},
    {"Polybench_JACOBI_2D", run_jacobi_2d}, {"Polybench_HEAT_3D", run_heat_3d},
    {"Polybench_FDTD_2D", run_fdtd_2d}, {"Polybench_GEMM", run_gemm},
    {"Polybench_3MM", run_3mm},        {"Algorithm_SCAN", run_scan},
    {"Algorithm_REDUCE_SUM", run_reduce_sum}, {"Algorithm_MEMSET", run_memset},
    {"Algorithm_MEMCPY", run_memcpy},   {"Algorithm_HISTOGRAM", run_histogram},
    {"Basic_INDEXLIST", run_indexlist}, {"Basic_INDEXLIST_3LOOP", run_indexlist_3loop},
    {"Basic_MULTI_REDUCE", run_multi_reduce},
    {"Comm_HALO_PACKING", run_halo_packing}, {"Comm_HALO_PACKING_FUSED", run_halo_packing_fused},
};

int oracle_run(const char* kernel, const oracle_opts* opts, oracle_result* out) {
  ctx c;
  if (!kernel || !opts || !out) return 2;
  memset(out, 0, sizeof(*out));
  if (opts->reps < 0) { out->status = 2; return 2; }
  c.o = opts;
  c.count = 0;
  c.par = opts->threads > 0;
  c.nt = opts->threads > 0 ? opts->threads : 1;
  g_skip_checksum = opts->skip_checksum;
  for (size_t k = 0; k < sizeof(kRunners) / sizeof(kRunners[0]); ++k) {
    if (strcmp(kernel, kRunners[k].name) == 0) {
      kRunners[k].fn(&c, out);
      return out->status;
    }
  }
  out->status = 1;
  return 1;
}
