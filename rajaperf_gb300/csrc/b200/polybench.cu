// Polybench group: JACOBI_2D, HEAT_3D, FDTD_2D, GEMM, 3MM (native FP64).
//
// On GB300 the FP64 pipe (about 0.53 T FP64 instructions/s) bounds these
// stencils well before HBM does, so the kernels keep the suite's per-point
// arithmetic exactly (the same operation order, no extra FP64 work) and rely
// on L1/L2 for neighbour reuse.  A library call runs all time steps of one
// rep; each half-step is one launch.
//
// GEMM is a shared-memory-tiled DFMA kernel: a 64x64 C tile per CTA, 4x4
// accumulators per thread, K in steps of 16 with the next K slice prefetched
// into registers while the current one is consumed.  Each C element's dot
// product runs over k in increasing order, as the suite's loop does.
#include "b200_internal.cuh"

using namespace b200;

namespace {

template <typename T>
__device__ __forceinline__ T ld(const T* p) { return __ldg(p); }

// ---- JACOBI_2D: polybench/POLYBENCH_JACOBI_2D.hpp:38-44 ---------------------
template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
jacobi2d_step(const double* __restrict__ src, double* __restrict__ dst, int64_t N) {
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= N - 1) return;
  for (int64_t i = 1 + static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < N - 1;
       i += static_cast<int64_t>(gridDim.y) * BY) {
    const int64_t c = j + i * N;
    dst[c] = 0.2 * (ld(src + c) + ld(src + c - 1) + ld(src + c + 1) + ld(src + c + N) +
                    ld(src + c - N));
  }
}

// ---- HEAT_3D: polybench/POLYBENCH_HEAT_3D.hpp:47-82 -------------------------
// Index k + N*(j + N*i); threads run along k (contiguous).
template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
heat3d_step(const double* __restrict__ S, double* __restrict__ D, int64_t N) {
  const int64_t k = 1 + static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y;
  if (k >= N - 1 || j >= N - 1) return;
  const int64_t NN = N * N;
  for (int64_t i = 1 + blockIdx.z; i < N - 1; i += gridDim.z) {
    const int64_t c = k + N * (j + N * i);
    const double a = ld(S + c);
    D[c] = 0.125 * (ld(S + c + NN) - 2.0 * a + ld(S + c - NN)) +
           0.125 * (ld(S + c + N) - 2.0 * a + ld(S + c - N)) +
           0.125 * (ld(S + c + 1) - 2.0 * a + ld(S + c - 1)) + a;
  }
}

// ---- FDTD_2D: polybench/POLYBENCH_FDTD_2D.hpp:52-69 -------------------------
// Launch 1 fuses BODY1..BODY3 (they read only hz, which none of them write):
// row 0 of ey takes fict[t], rows >= 1 of ey and columns >= 1 of ex update.
// Launch 2 is BODY4 (hz from the new ex, ey).
template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
fdtd2d_e(double* __restrict__ ex, double* __restrict__ ey, const double* __restrict__ hz,
         const double* __restrict__ fict, int64_t t, int64_t nx, int64_t ny) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= ny) return;
  const double f = ld(fict + t);
  for (int64_t i = static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < nx;
       i += static_cast<int64_t>(gridDim.y) * BY) {
    const int64_t c = j + i * ny;
    const double h = ld(hz + c);
    if (i == 0) ey[c] = f;
    else ey[c] = ey[c] - 0.5 * (h - ld(hz + c - ny));
    if (j >= 1) ex[c] = ex[c] - 0.5 * (h - ld(hz + c - 1));
  }
}

template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
fdtd2d_h(const double* __restrict__ ex, const double* __restrict__ ey,
         double* __restrict__ hz, int64_t nx, int64_t ny) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= ny - 1) return;
  for (int64_t i = static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < nx - 1;
       i += static_cast<int64_t>(gridDim.y) * BY) {
    const int64_t c = j + i * ny;
    hz[c] = hz[c] - 0.7 * (ld(ex + c + 1) - ld(ex + c) + ld(ey + c + ny) - ld(ey + c));
  }
}

// ---- GEMM (FP64, DFMA) -------------------------------------------------------
// C[i][j] = sum_k (alpha*A[i][k]) * B[k][j]   (row-major A: ni x nk, B: nk x nj)
// When beta_mode is set: C = alpha*sum_k A*B + beta*C (the classic form).
constexpr int GT = 64;   // C tile edge
constexpr int GK = 16;   // K slice
constexpr int GTH = 16;  // threads per tile edge (16x16 = 256 threads, 4x4 each)

__global__ void __launch_bounds__(256)
dgemm_kernel(const double* __restrict__ A, const double* __restrict__ B,
             double* __restrict__ C, int64_t ni, int64_t nj, int64_t nk, double alpha,
             double beta, int mode) {
  __shared__ double As[GK][GT + 1];  // As[k][i]
  __shared__ double Bs[GK][GT];      // Bs[k][j]
  const int tx = threadIdx.x % GTH, ty = threadIdx.x / GTH;
  const int64_t i0 = static_cast<int64_t>(blockIdx.y) * GT;
  const int64_t j0 = static_cast<int64_t>(blockIdx.x) * GT;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

  // loader mapping: 256 threads load a 64x16 A slice and a 16x64 B slice,
  // 4 elements each
  const int la_k = threadIdx.x % GK, la_i = threadIdx.x / GK;   // A: k fastest
  const int lb_j = threadIdx.x % GT, lb_k = threadIdx.x / GT;   // B: j fastest
  double ra[4], rb[4];
  auto load = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int64_t gi = i0 + la_i + r * 16, gk = k0 + la_k;
      ra[r] = (gi < ni && gk < nk) ? ld(A + gk + gi * nk) : 0.0;
      int64_t gk2 = k0 + lb_k + r * 4, gj = j0 + lb_j;
      rb[r] = (gk2 < nk && gj < nj) ? ld(B + gj + gk2 * nj) : 0.0;
    }
  };
  load(0);
  for (int64_t k0 = 0; k0 < nk; k0 += GK) {
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      As[la_k][la_i + r * 16] = (mode == 0) ? alpha * ra[r] : ra[r];
      Bs[lb_k + r * 4][lb_j] = rb[r];
    }
    __syncthreads();
    if (k0 + GK < nk) load(k0 + GK);
    const int kmax = (nk - k0 < GK) ? static_cast<int>(nk - k0) : GK;
    for (int kk = 0; kk < kmax; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + r * GTH];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx + c * GTH];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int64_t gi = i0 + ty + r * GTH;
    if (gi >= ni) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int64_t gj = j0 + tx + c * GTH;
      if (gj >= nj) continue;
      double* p = C + gj + gi * nj;
      if (mode == 0) *p = acc[r][c];
      else *p = alpha * acc[r][c] + beta * (*p);
    }
  }
}

int launch_dgemm(const double* A, const double* B, double* C, int64_t ni, int64_t nj,
                 int64_t nk, double alpha, double beta, int mode, cudaStream_t st) {
  if (ni <= 0 || nj <= 0) return B200_OK;
  int64_t gx = ceil_div(nj, GT), gy = ceil_div(ni, GT);
  if (gx > 0x7fffffff || gy > 65535) return invalid("gemm: matrix too large");
  dgemm_kernel<<<dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy)), 256, 0, st>>>(
      A, B, C, ni, nj, nk, alpha, beta, mode);
  return B200_OK;
}

dim3 grid2(int64_t nxthreads, int64_t nrows, int bx, int by) {
  int64_t gx = ceil_div(nxthreads > 0 ? nxthreads : 1, bx);
  int64_t gy = ceil_div(nrows > 0 ? nrows : 1, by);
  if (gy > 65535) gy = 65535;
  return dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy), 1);
}

}  // namespace

extern "C" {

int b200_polybench_jacobi_2d(double* A, double* B, int64_t N, int64_t tsteps,
                             const b200_tune* tune, b200_stream_t stream) {
  if (!A || !B || N < 0 || tsteps < 0) return invalid("b200_polybench_jacobi_2d: bad args");
  if (N < 3 || tsteps == 0) return B200_OK;
  (void)tune;
  cudaStream_t st = as_stream(stream);
  constexpr int BX = 64, BY = 4;
  dim3 g = grid2(N - 2, N - 2, BX, BY);
  for (int64_t t = 0; t < tsteps; ++t) {
    jacobi2d_step<BX, BY><<<g, dim3(BX, BY), 0, st>>>(A, B, N);
    jacobi2d_step<BX, BY><<<g, dim3(BX, BY), 0, st>>>(B, A, N);
  }
  return after_launch("b200_polybench_jacobi_2d", static_cast<int>(2 * tsteps));
}

int b200_polybench_heat_3d(double* A, double* B, int64_t N, int64_t tsteps,
                           const b200_tune* tune, b200_stream_t stream) {
  if (!A || !B || N < 0 || tsteps < 0) return invalid("b200_polybench_heat_3d: bad args");
  if (N < 3 || tsteps == 0) return B200_OK;
  (void)tune;
  cudaStream_t st = as_stream(stream);
  constexpr int BX = 32, BY = 8;
  int64_t gz = N - 2;
  if (gz > 65535) gz = 65535;
  dim3 g(static_cast<unsigned>(ceil_div(N - 2, BX)), static_cast<unsigned>(ceil_div(N - 2, BY)),
         static_cast<unsigned>(gz));
  if (ceil_div(N - 2, BY) > 65535) return invalid("b200_polybench_heat_3d: N too large");
  for (int64_t t = 0; t < tsteps; ++t) {
    heat3d_step<BX, BY><<<g, dim3(BX, BY), 0, st>>>(A, B, N);
    heat3d_step<BX, BY><<<g, dim3(BX, BY), 0, st>>>(B, A, N);
  }
  return after_launch("b200_polybench_heat_3d", static_cast<int>(2 * tsteps));
}

int b200_polybench_fdtd_2d(double* ex, double* ey, double* hz, const double* fict,
                           int64_t nx, int64_t ny, int64_t tsteps, const b200_tune* tune,
                           b200_stream_t stream) {
  if (!ex || !ey || !hz || !fict || nx < 0 || ny < 0 || tsteps < 0)
    return invalid("b200_polybench_fdtd_2d: bad args");
  if (nx == 0 || ny == 0 || tsteps == 0) return B200_OK;
  (void)tune;
  cudaStream_t st = as_stream(stream);
  constexpr int BX = 64, BY = 4;
  dim3 ge = grid2(ny, nx, BX, BY);
  dim3 gh = grid2(ny - 1, nx - 1, BX, BY);
  for (int64_t t = 0; t < tsteps; ++t) {
    fdtd2d_e<BX, BY><<<ge, dim3(BX, BY), 0, st>>>(ex, ey, hz, fict, t, nx, ny);
    if (nx > 1 && ny > 1) fdtd2d_h<BX, BY><<<gh, dim3(BX, BY), 0, st>>>(ex, ey, hz, nx, ny);
  }
  int per = (nx > 1 && ny > 1) ? 2 : 1;
  return after_launch("b200_polybench_fdtd_2d", static_cast<int>(per * tsteps));
}

int b200_polybench_gemm(const double* A, const double* B, double* C, int64_t ni,
                        int64_t nj, int64_t nk, double alpha, const b200_tune* tune,
                        b200_stream_t stream) {
  if (!A || !B || !C || ni < 0 || nj < 0 || nk < 0)
    return invalid("b200_polybench_gemm: bad args");
  (void)tune;
  int st = launch_dgemm(A, B, C, ni, nj, nk, alpha, 0.0, 0, as_stream(stream));
  if (st != B200_OK) return st;
  return after_launch("b200_polybench_gemm", (ni > 0 && nj > 0) ? 1 : 0);
}

int b200_gemm_f64(const double* A, const double* B, double* C, int64_t m, int64_t n,
                  int64_t k, double alpha, double beta, const b200_tune* tune,
                  b200_stream_t stream) {
  if (!A || !B || !C || m < 0 || n < 0 || k < 0) return invalid("b200_gemm_f64: bad args");
  (void)tune;
  int st = launch_dgemm(A, B, C, m, n, k, alpha, beta, 1, as_stream(stream));
  if (st != B200_OK) return st;
  return after_launch("b200_gemm_f64", (m > 0 && n > 0) ? 1 : 0);
}

int b200_polybench_3mm(const double* A, const double* B, const double* C,
                       const double* D, double* E, double* F, double* G, int64_t ni,
                       int64_t nj, int64_t nk, int64_t nl, int64_t nm,
                       const b200_tune* tune, b200_stream_t stream) {
  if (!A || !B || !C || !D || !E || !F || !G || ni < 0 || nj < 0 || nk < 0 || nl < 0 ||
      nm < 0)
    return invalid("b200_polybench_3mm: bad args");
  (void)tune;
  cudaStream_t st = as_stream(stream);
  int s = launch_dgemm(A, B, E, ni, nj, nk, 1.0, 0.0, 0, st);   // E = A*B
  if (s == B200_OK) s = launch_dgemm(C, D, F, nj, nl, nm, 1.0, 0.0, 0, st);  // F = C*D
  if (s == B200_OK) s = launch_dgemm(E, F, G, ni, nl, nj, 1.0, 0.0, 0, st);  // G = E*F
  if (s != B200_OK) return s;
  return after_launch("b200_polybench_3mm", 3);
}

}  // extern "C"
