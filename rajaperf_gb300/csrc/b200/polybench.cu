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
#include "b200_f64emu.cuh"
#include "b200_fma_form.cuh"
#include "b200_internal.cuh"

#include <type_traits>

using namespace b200;

namespace {

template <typename T>
__device__ __forceinline__ T ld(const T* p) { return __ldg(p); }

// ---- JACOBI_2D: polybench/POLYBENCH_JACOBI_2D.hpp:38-44 ---------------------
// One point per thread (tune->items 1).  The four adds stay on the FP64 pipe;
// the product by 0.2 runs on the integer pipe (f64emu::mul_fast, correctly
// rounded, bit-identical), leaving the FP64 pipe 4 instructions per point
// instead of 5.  A thread that met a zero, subnormal or non-finite sum
// rewrites its points natively after the loop.
template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
jacobi2d_step(const double* __restrict__ src, double* __restrict__ dst, int64_t N) {
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= N - 1) return;
  bool slow = false;
  for (int64_t i = 1 + static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < N - 1;
       i += static_cast<int64_t>(gridDim.y) * BY) {
    const int64_t c = j + i * N;
    dst[c] = f64emu::mul_fast(
        ld(src + c) + ld(src + c - 1) + ld(src + c + 1) + ld(src + c + N) + ld(src + c - N),
        0.2, slow);
  }
  if (__any_sync(__activemask(), slow) && slow) {
    for (int64_t i = 1 + static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < N - 1;
         i += static_cast<int64_t>(gridDim.y) * BY) {
      const int64_t c = j + i * N;
      dst[c] = 0.2 * (ld(src + c) + ld(src + c - 1) + ld(src + c + 1) + ld(src + c + N) +
                      ld(src + c - N));
    }
  }
}

// The default: column segments.  Thread j of CTA (bx, by) computes rows
// i0 .. i0+R-1 of column j with all loads issued first (vertical neighbours
// shared between consecutive rows) and R independent sums, each multiplied by
// 0.2 on the integer pipe; out-of-range sums are redone natively as in
// jacobi2d_step.  With the multiply off the FP64 pipe, the independent rows
// hide its integer latency: 165 -> 133 us per half-step at 4096^2 (one point
// per thread with the FP64 multiply: 165 us; with the integer multiply: 158).
// The four adds are register-operand FMAs (fform::add, bit-identical), which
// the FP64 pipe issues at its full rate where DADD gets 5/6 of it: 133 ->
// 115 us.  With 4 rows per thread and the first add of each point on the
// integer pipes (KQ = 4 below): 92 us.  `zero` is 0 at run time.
// KQ adds in every four consecutive points (the first ones of each point, in
// the suite's order; row r of a group of four takes (KQ(r+1))/4 - (KQ r)/4)
// run on the integer pipes (f64emu::add_close_fast, bit-identical; its
// operands here are sums of one sign and similar size), the rest on the FP64
// pipe, and the product by 0.2 on the integer pipe (MULINT) or the FP64 pipe
// (an FMA with -0, bit-identical to the product): the two pipes then share
// the point's work instead of the FP64 pipe carrying all of it.
template <int BX, int R, int KQ = 0, bool MULINT = true>
__global__ void __launch_bounds__(BX)
jacobi2d_rows(const double* __restrict__ src, double* __restrict__ dst, int64_t N, int zero) {
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= N - 1) return;
  const int64_t i0 = 1 + static_cast<int64_t>(blockIdx.y) * R;
  const int64_t rows = (N - 1 - i0 < R) ? (N - 1 - i0) : R;
  const double* p = src + (i0 - 1) * N + j;
  double* q = dst + i0 * N + j;
  bool slow = false;
  if (rows == R) {
    double col[R + 2], lft[R], rgt[R];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) col[r] = ld(p + r * N);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      lft[r] = ld(p + (r + 1) * N - 1);
      rgt[r] = ld(p + (r + 1) * N + 1);
    }
    const fform::Regs fr = fform::regs(zero);
    const double fifth = fform::reg(0.2, zero);  // a per-thread register
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int ki = (KQ * (r % 4 + 1)) / 4 - (KQ * (r % 4)) / 4;
      auto add = [&](int k, double a, double b) {
        return (k < ki) ? f64emu::add_close_fast(a, b, slow) : fform::add(a, b, fr);
      };
      const double sum =
          add(3, add(2, add(1, add(0, col[r + 1], lft[r]), rgt[r]), col[r + 2]), col[r]);
      q[r * N] = MULINT ? f64emu::mul_fast(sum, 0.2, slow) : fform::mul(sum, fifth, fr);
    }
  } else {
    for (int64_t r = 0; r < rows; ++r) {
      const double* c = p + (r + 1) * N;
      q[r * N] = f64emu::mul_fast(c[0] + c[-1] + c[1] + c[N] + c[-N], 0.2, slow);
    }
  }
  if (__any_sync(__activemask(), slow) && slow) {
    for (int64_t r = 0; r < rows; ++r) {
      const double* c = p + (r + 1) * N;
      q[r * N] = 0.2 * (ld(c) + ld(c - 1) + ld(c + 1) + ld(c + N) + ld(c - N));
    }
  }
}

// ---- HEAT_3D: polybench/POLYBENCH_HEAT_3D.hpp:47-82 -------------------------
// Index k + N*(j + N*i); threads run along k (contiguous), and each thread
// walks PL consecutive planes i, keeping b(i-1), a and b(i+1) in registers
// (five loads a point instead of seven, one index step).  KS2 of the six
// differences b(+1) - 2a of two consecutive planes (directions i, j, k in that
// order; an odd KS2 gives the second plane the larger share) run on the
// integer pipes (f64emu::sub_near_fast, bit-identical); the rest stay on the
// FP64 pipe.
template <int BX, int BY, int PL, int KS2>
__global__ void __launch_bounds__(BX * BY)
heat3d_step(const double* __restrict__ S, double* __restrict__ D, int64_t N, int zero) {
  static_assert(PL % 2 == 0 && KS2 >= 0 && KS2 <= 6, "planes in pairs, 0..6 integer differences");
  const int64_t k = 1 + static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y;
  if (k >= N - 1 || j >= N - 1) return;
  const unsigned live = __activemask();
  const int64_t NN = N * N;
  const int64_t i0 = 1 + static_cast<int64_t>(blockIdx.z) * PL;
  const int np = static_cast<int>((N - 1 - i0) < PL ? (N - 1 - i0) : PL);
  // 2.0 * a and 0.125 * v are exact: exponent moves on the integer pipe, so
  // the FP64 pipe keeps at most the 9 adds of a point, issued as
  // register-operand FMAs (fform, bit-identical; full rate where DADD gets 5/6
  // of it).  A thread that met a zero, subnormal or non-finite value (or
  // differences too far apart for the integer-pipe form) rewrites its points
  // with the FP64 products after the loop (the same results, bit for bit).
  // `zero` is 0 at run time.
  const fform::Regs fr = fform::regs(zero);
  bool slow = false;
  const double* p = S + k + N * (j + N * i0);
  double* q = D + k + N * (j + N * i0);
  double im = ld(p - NN), a = ld(p);
#pragma unroll
  for (int r = 0; r < PL; ++r) {
    if (r >= np) break;
    const int ks = (KS2 * (r % 2 + 1)) / 2 - (KS2 * (r % 2)) / 2;  // this plane's share
    const double ip = ld(p + NN);
    const double a2 = f64emu::mul_pow2_fast<1>(a, slow);
    auto dir = [&](int m, double hi, double lo) {
      const double d = (m < ks) ? f64emu::sub_near_fast(hi, a2, slow) : fform::sub(hi, a2, fr);
      return f64emu::mul_pow2_fast<-3>(fform::add(d, lo, fr), slow);
    };
    const double ti = dir(0, ip, im);
    const double tj = dir(1, ld(p + N), ld(p - N));
    const double tk = dir(2, ld(p + 1), ld(p - 1));
    *q = fform::add(fform::add(fform::add(ti, tj, fr), tk, fr), a, fr);
    im = a;
    a = ip;
    p += NN;
    q += NN;
  }
  if (__any_sync(live, slow) && slow) {
    for (int r = 0; r < np; ++r) {
      const int64_t c = k + N * (j + N * (i0 + r));
      const double a0 = ld(S + c);
      D[c] = 0.125 * (ld(S + c + NN) - 2.0 * a0 + ld(S + c - NN)) +
             0.125 * (ld(S + c + N) - 2.0 * a0 + ld(S + c - N)) +
             0.125 * (ld(S + c + 1) - 2.0 * a0 + ld(S + c - 1)) + a0;
    }
  }
}

// ---- FDTD_2D: polybench/POLYBENCH_FDTD_2D.hpp:52-69 -------------------------
// Launch 1 fuses BODY1..BODY3 (they read only hz, which none of them write):
// row 0 of ey takes fict[t], rows >= 1 of ey and columns >= 1 of ex update.
// Launch 2 is BODY4 (hz from the new ex, ey).
template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
fdtd2d_e(double* __restrict__ ex, double* __restrict__ ey, const double* __restrict__ hz,
         const double* __restrict__ fict, int64_t t, int64_t nx, int64_t ny, int zero) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= ny) return;
  const double f = ld(fict + t);
  // register-operand FMAs (fform: the differences, and e - 0.5 d as the FMA
  // the compiler contracts it to, with -0.5 in a per-thread register), the
  // FP64 pipe's full-rate form; `zero` is 0 at run time
  const fform::Regs fr = fform::regs(zero);
  const double mhalf = fform::reg(-0.5, zero);
  for (int64_t i = static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < nx;
       i += static_cast<int64_t>(gridDim.y) * BY) {
    const int64_t c = j + i * ny;
    const double h = ld(hz + c);
    if (i == 0) ey[c] = f;
    else ey[c] = fma(mhalf, fform::sub(h, ld(hz + c - ny), fr), ey[c]);
    if (j >= 1) ex[c] = fma(mhalf, fform::sub(h, ld(hz + c - 1), fr), ex[c]);
  }
}

template <int BX, int BY>
__global__ void __launch_bounds__(BX * BY)
fdtd2d_h(const double* __restrict__ ex, const double* __restrict__ ey,
         double* __restrict__ hz, int64_t nx, int64_t ny, int zero) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * BX + threadIdx.x;
  if (j >= ny - 1) return;
  const fform::Regs fr = fform::regs(zero);
  const double m07 = fform::reg(-0.7, zero);
  for (int64_t i = static_cast<int64_t>(blockIdx.y) * BY + threadIdx.y; i < nx - 1;
       i += static_cast<int64_t>(gridDim.y) * BY) {
    const int64_t c = j + i * ny;
    // hz - 0.7 (((ex1 - ex0) + ey1) - ey0), left to right as the suite writes it
    hz[c] = fma(m07,
                fform::sub(fform::add(fform::sub(ld(ex + c + 1), ld(ex + c), fr), ld(ey + c + ny), fr),
                           ld(ey + c), fr),
                hz[c]);
  }
}

// ---- FDTD_2D, one launch per time step ------------------------------------------
// A CTA owns a tile of kFdtdRows rows x kFdtdCols columns (one thread per
// column) and runs the whole time step on it in place: phase 1 updates ex
// and ey (BODY1-3) of its points, keeping the new values in shared memory,
// phase 2 updates hz (BODY4) from them.  H at the tile's last column and row
// needs new ex one column to the right and new ey one row below; the tile
// computes those from the neighbours' old values (a right halo column and a
// bottom halo row, 2 FP64 instructions per halo point, issued as full warps).
// Old values across tile edges cannot come from the arrays, since the
// neighbouring tiles update theirs in place during the same launch: they come
// from a snapshot of every tile's edges (its first row's hz and ey, its last
// row's hz, its first column's hz and ex, its last column's hz) as they were
// at the start of the step.  Each tile writes its new edges into the other
// snapshot buffer for the next step, and a small kernel takes the first
// snapshot.  Per point and step the kernel reads hz, ex, ey and writes them
// once (48 bytes; the two-launch form moves 72) and issues the same 8 FP64
// instructions per point in the same forms as fdtd2d_e / fdtd2d_h, so the
// results are bit-identical.
constexpr int kFdtdCols = 128;     // threads per CTA
constexpr int kFdtdMinRows = 8;    // the workspace holds snapshots for tiles this short
// 8192^2, 20 steps (GB300): 8 rows 0.965 ms per step (556 G FP64
// instructions/s, 93% of the pipe), 16 rows 1.017, 32 rows 1.485 (the
// two-launch form: 1.173); shorter tiles leave more CTAs resident per SM.
constexpr int kFdtdDefaultRows = 8;

struct FdtdSnap {
  double* top_hz;    // [tile rows][ny]: hz of each tile's first row
  double* top_ey;    // [tile rows][ny]: ey of each tile's first row
  double* bot_hz;    // [tile rows][ny]: hz of each tile's last row
  double* left_hz;   // [tile cols][nx]: hz of each tile's first column
  double* left_ex;   // [tile cols][nx]: ex of each tile's first column
  double* right_hz;  // [tile cols][nx]: hz of each tile's last column
};

__global__ void fdtd2d_snap_init(const double* __restrict__ ex, const double* __restrict__ ey,
                                 const double* __restrict__ hz, int64_t nx, int64_t ny,
                                 int64_t ntx, int64_t nty, int th, FdtdSnap s) {
  const int64_t nrow = nty * ny, total = nrow + ntx * nx;
  for (int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (idx < nrow) {
      const int64_t by = idx / ny, j = idx - by * ny;
      const int64_t i0 = by * th;
      const int64_t il = (i0 + th < nx ? i0 + th : nx) - 1;
      s.top_hz[idx] = hz[i0 * ny + j];
      s.top_ey[idx] = ey[i0 * ny + j];
      s.bot_hz[idx] = hz[il * ny + j];
    } else {
      const int64_t k = idx - nrow;
      const int64_t bx = k / nx, i = k - bx * nx;
      const int64_t j0 = bx * kFdtdCols;
      const int64_t jl = (j0 + kFdtdCols < ny ? j0 + kFdtdCols : ny) - 1;
      s.left_hz[k] = hz[i * ny + j0];
      s.left_ex[k] = ex[i * ny + j0];
      s.right_hz[k] = hz[i * ny + jl];
    }
  }
}

template <int TH>
__global__ void __launch_bounds__(kFdtdCols, (TH <= 8 ? 8 : TH <= 16 ? 5 : 3))
fdtd2d_step_fused(double* __restrict__ ex, double* __restrict__ ey, double* __restrict__ hz,
                  const double* __restrict__ fict, int64_t t, int64_t nx, int64_t ny,
                  FdtdSnap in, FdtdSnap out, int zero) {
  extern __shared__ __align__(16) double s_fdtd[];
  // new ex [rows][cols + 1] (column kFdtdCols: the right halo), new ey
  // [rows + 1][cols] (row TH: the bottom halo), new hz of the first
  // and last column
  double (*sEx)[kFdtdCols + 1] = reinterpret_cast<double (*)[kFdtdCols + 1]>(s_fdtd);
  double (*sEy)[kFdtdCols] =
      reinterpret_cast<double (*)[kFdtdCols]>(s_fdtd + TH * (kFdtdCols + 1));
  double* sHzFirst = s_fdtd + TH * (kFdtdCols + 1) + (TH + 1) * kFdtdCols;
  double* sHzLast = sHzFirst + TH;

  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t bx = blockIdx.x, by = blockIdx.y;
  const int64_t j0 = bx * kFdtdCols, i0 = by * TH;
  const int64_t j = j0 + tid;
  const int rows = static_cast<int>(nx - i0 < TH ? nx - i0 : TH);
  const int cols = static_cast<int>(ny - j0 < kFdtdCols ? ny - j0 : kFdtdCols);
  const bool col_ok = tid < cols;
  const fform::Regs fr = fform::regs(zero);
  const double mhalf = fform::reg(-0.5, zero);
  const double m07 = fform::reg(-0.7, zero);
  const double f = ld(fict + t);

  // ---- phase 1: BODY1-3 (ex, ey) ----
  double h_old[TH];
  double hup = (i0 > 0 && col_ok) ? in.bot_hz[(by - 1) * ny + j] : 0.0;
#pragma unroll
  for (int r = 0; r < TH; ++r) {
    h_old[r] = 0.0;
    if (r < rows) {
      const int64_t i = i0 + r;
      const int64_t c = i * ny + j;
      double h = 0.0, exo = 0.0, eyo = 0.0;
      if (col_ok) {
        h = hz[c];
        exo = ex[c];
        eyo = ey[c];
      }
      double hl = __shfl_up_sync(0xffffffffu, h, 1);
      if (lane == 0) {
        if (tid == 0) hl = (j0 > 0) ? in.right_hz[(bx - 1) * nx + i] : 0.0;
        else if (col_ok) hl = hz[c - 1];  // this tile's column, not yet rewritten
      }
      const double eyn = (i == 0) ? f : fma(mhalf, fform::sub(h, hup, fr), eyo);
      const double exn = (j == 0) ? exo : fma(mhalf, fform::sub(h, hl, fr), exo);
      if (col_ok) {
        ex[c] = exn;
        ey[c] = eyn;
      }
      sEx[r][tid] = exn;
      sEy[r][tid] = eyn;
      h_old[r] = h;
      hup = h;
    }
  }
  // bottom halo: new ey one row below the tile (needed when that row exists)
  if (i0 + TH < nx && col_ok) {
    const int64_t k = (by + 1) * ny + j;
    sEy[TH][tid] = fma(mhalf, fform::sub(in.top_hz[k], h_old[TH - 1], fr),
                              in.top_ey[k]);
  }
  // right halo: new ex one column right of the tile, one row per lane of the
  // last warp (full-warp FP64 instructions)
  if (tid >= kFdtdCols - 32 && j0 + kFdtdCols < ny && lane < rows) {
    const int64_t i = i0 + lane;
    const int64_t k = (bx + 1) * nx + i;
    const double hl = hz[i * ny + j0 + kFdtdCols - 1];  // old: read before phase 2
    sEx[lane][kFdtdCols] = fma(mhalf, fform::sub(in.left_hz[k], hl, fr), in.left_ex[k]);
  }
  __syncthreads();

  // ---- phase 2: BODY4 (hz) and the tile's new edges ----
#pragma unroll
  for (int r = 0; r < TH; ++r) {
    if (r < rows) {
      const int64_t i = i0 + r;
      double hn = h_old[r];
      if (col_ok && i < nx - 1 && j < ny - 1) {
        // hz - 0.7 (((ex1 - ex0) + ey1) - ey0), left to right as the suite writes it
        hn = fma(m07,
                 fform::sub(fform::add(fform::sub(sEx[r][tid + 1], sEx[r][tid], fr),
                                       sEy[r + 1][tid], fr),
                            sEy[r][tid], fr),
                 h_old[r]);
        hz[i * ny + j] = hn;
      }
      if (col_ok) {
        if (r == 0) {
          out.top_hz[by * ny + j] = hn;
          out.top_ey[by * ny + j] = sEy[0][tid];
        }
        if (r == rows - 1) out.bot_hz[by * ny + j] = hn;
        if (tid == 0) sHzFirst[r] = hn;
        if (tid == cols - 1) sHzLast[r] = hn;
      }
    }
  }
  __syncthreads();
  if (tid < 32 && lane < rows) {
    const int64_t k = bx * nx + i0 + lane;
    out.left_hz[k] = sHzFirst[lane];
    out.left_ex[k] = sEx[lane][0];
  } else if (tid >= 32 && tid < 64 && lane < rows) {
    out.right_hz[bx * nx + i0 + lane] = sHzLast[lane];
  }
}

constexpr size_t fdtd_smem(int th) {
  return sizeof(double) * (th * (kFdtdCols + 1) + (th + 1) * kFdtdCols + 2 * th);
}

int64_t fdtd_tile_rows(int64_t nx, int th) { return (nx + th - 1) / th; }
int64_t fdtd_tile_cols(int64_t ny) { return (ny + kFdtdCols - 1) / kFdtdCols; }
// doubles of one snapshot for tiles of th rows
int64_t fdtd_snap_doubles(int64_t nx, int64_t ny, int th) {
  return 3 * fdtd_tile_rows(nx, th) * ny + 3 * fdtd_tile_cols(ny) * nx;
}

FdtdSnap fdtd_snap_at(double* base, int64_t nx, int64_t ny, int th) {
  const int64_t rowv = fdtd_tile_rows(nx, th) * ny, colv = fdtd_tile_cols(ny) * nx;
  FdtdSnap s;
  s.top_hz = base;
  s.top_ey = base + rowv;
  s.bot_hz = base + 2 * rowv;
  s.left_hz = base + 3 * rowv;
  s.left_ex = base + 3 * rowv + colv;
  s.right_hz = base + 3 * rowv + 2 * colv;
  return s;
}

template <int TH>
int launch_fdtd_fused(double* ex, double* ey, double* hz, const double* fict, int64_t nx,
                      int64_t ny, int64_t tsteps, double* w, cudaStream_t st) {
  const int rc = allow_dynamic_smem(reinterpret_cast<const void*>(fdtd2d_step_fused<TH>),
                                    fdtd_smem(TH), "b200_polybench_fdtd_2d_ws");
  if (rc != B200_OK) return rc;
  const FdtdSnap snap[2] = {fdtd_snap_at(w, nx, ny, TH),
                            fdtd_snap_at(w + fdtd_snap_doubles(nx, ny, TH), nx, ny, TH)};
  const int64_t ntx = fdtd_tile_cols(ny), nty = fdtd_tile_rows(nx, TH);
  const int64_t total = nty * ny + ntx * nx;
  const unsigned ig = static_cast<unsigned>(std::min<int64_t>(ceil_div(total, 256), 4096));
  fdtd2d_snap_init<<<ig, 256, 0, st>>>(ex, ey, hz, nx, ny, ntx, nty, TH, snap[0]);
  const dim3 g(static_cast<unsigned>(ntx), static_cast<unsigned>(nty));
  for (int64_t t = 0; t < tsteps; ++t)
    fdtd2d_step_fused<TH><<<g, kFdtdCols, fdtd_smem(TH), st>>>(ex, ey, hz, fict, t, nx, ny,
                                                               snap[t & 1], snap[(t + 1) & 1], 0);
  return B200_OK;
}

// ---- mixed FP64-pipe / integer-pipe stencils ----------------------------------
// A CTA of 8 warps owns a tile of 32 contiguous columns.  Warps [0, E) compute
// their rows with the integer-pipe emulation (b200_f64emu.cuh), warps [E, 8)
// with the FP64 pipe; emulated warps take `he` rows each and native warps `hn`,
// so both pipes finish together.  Each thread walks down its rows keeping the
// vertical neighbours in registers.  The emulated arithmetic is bit-identical
// to the FP64 pipe's, so the split never changes a result.
struct MixShape {
  int E, he, hn;
  __host__ __device__ int rows() const { return E * he + (8 - E) * hn; }
};

template <bool EMU>
__device__ __forceinline__ double jacobi_pt(double c, double l, double r, double d, double u) {
  if (EMU) {
    using namespace f64emu;
    return mul(0.2, add(add(add(add(c, l), r), d), u));
  }
  return 0.2 * (c + l + r + d + u);
}

template <bool EMU>
__device__ __forceinline__ void jacobi_rows(const double* __restrict__ S, double* __restrict__ D,
                                            int64_t N, int64_t j, int64_t i_first, int rows) {
  if (i_first >= N - 1) return;  // this warp's rows lie past the interior
  int64_t c = j + i_first * N;
  double up = ld(S + c - N), mid = ld(S + c);
  for (int r = 0; r < rows; ++r, c += N) {
    if (i_first + r >= N - 1) break;
    const double down = ld(S + c + N);
    D[c] = jacobi_pt<EMU>(mid, ld(S + c - 1), ld(S + c + 1), down, up);
    up = mid;
    mid = down;
  }
}

__global__ void __launch_bounds__(256)
jacobi2d_mixed(const double* __restrict__ S, double* __restrict__ D, int64_t N, MixShape m) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.x) * 32 + lane;
  if (j >= N - 1) return;
  const bool emu = warp < m.E;
  const int r0 = emu ? warp * m.he : m.E * m.he + (warp - m.E) * m.hn;
  const int rows = emu ? m.he : m.hn;
  for (int64_t tile = blockIdx.y; tile * m.rows() < N - 2; tile += gridDim.y) {
    const int64_t i_first = 1 + tile * m.rows() + r0;
    if (emu) jacobi_rows<true>(S, D, N, j, i_first, rows);
    else jacobi_rows<false>(S, D, N, j, i_first, rows);
  }
}

// HEAT_3D point: the suite's body, with 2.0*a and 0.125*u as exact
// power-of-two scalings on the emulated path.
template <bool EMU>
__device__ __forceinline__ double heat_pt(double a, double ip, double im, double jp, double jm,
                                          double kp, double km) {
  if (EMU) {
    using namespace f64emu;
    const double a2 = scale2(a, 1);
    const double t1 = scale2(add(sub(ip, a2), im), -3);
    const double t2 = scale2(add(sub(jp, a2), jm), -3);
    const double t3 = scale2(add(sub(kp, a2), km), -3);
    return add(add(add(t1, t2), t3), a);
  }
  return 0.125 * (ip - 2.0 * a + im) + 0.125 * (jp - 2.0 * a + jm) +
         0.125 * (kp - 2.0 * a + km) + a;
}

// Thread (j, k) walks planes i in [i0, i0 + ni): the i-neighbours stay in
// registers.  Index k + N*(j + N*i).
template <bool EMU>
__device__ __forceinline__ void heat_rows(const double* __restrict__ S, double* __restrict__ D,
                                          int64_t N, int64_t k, int64_t j_first, int rows,
                                          int64_t i0, int64_t ni) {
  const int64_t NN = N * N;
  for (int r = 0; r < rows; ++r) {
    const int64_t j = j_first + r;
    if (j >= N - 1) break;
    int64_t c = k + N * (j + N * i0);
    double im = ld(S + c - NN), a = ld(S + c);
    for (int64_t i = i0; i < i0 + ni && i < N - 1; ++i, c += NN) {
      const double ip = ld(S + c + NN);
      D[c] = heat_pt<EMU>(a, ip, im, ld(S + c + N), ld(S + c - N), ld(S + c + 1), ld(S + c - 1));
      im = a;
      a = ip;
    }
  }
}

__global__ void __launch_bounds__(256)
heat3d_mixed(const double* __restrict__ S, double* __restrict__ D, int64_t N, MixShape m,
             int64_t chunk) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k = 1 + static_cast<int64_t>(blockIdx.x) * 32 + lane;
  if (k >= N - 1) return;
  const bool emu = warp < m.E;
  const int r0 = emu ? warp * m.he : m.E * m.he + (warp - m.E) * m.hn;
  const int rows = emu ? m.he : m.hn;
  const int64_t j_first = 1 + static_cast<int64_t>(blockIdx.y) * m.rows() + r0;
  const int64_t i0 = 1 + static_cast<int64_t>(blockIdx.z) * chunk;
  if (emu) heat_rows<true>(S, D, N, k, j_first, rows, i0, chunk);
  else heat_rows<false>(S, D, N, k, j_first, rows, i0, chunk);
}

MixShape mix_shape(const b200_tune* t, MixShape def) {
  MixShape m = def;
  if (t && t->algo > 0) m.E = t->algo - 1;   // algo = 1 + emulated warps (0..8)
  if (t && t->tile_y > 0) m.he = t->tile_y;
  if (t && t->tile_z > 0) m.hn = t->tile_z;
  if (m.E < 0) m.E = 0;
  if (m.E > 8) m.E = 8;
  if (m.he < 1) m.he = 1;
  if (m.hn < 1) m.hn = 1;
  return m;
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

// JACOBI_2D's split between the pipes by default: integer-pipe adds per
// four points and where the product by 0.2 runs.  Measured on GB300 (4 rows
// per thread, us per half-step at 4096^2): FP64 adds only 114.7; one add per
// point on the integer pipe 92.3; two 125.1; with the product on the FP64
// pipe, two adds per point 94.2, one 114.8.  One integer-pipe add costs
// about 33 us of the integer pipes' time per half-step here (some 40
// instructions), the integer product about 59.  With both integer forms rounding in
// one add (90.1 us at one add per point), five and six adds per four points
// measured 94.4 and 102.5 us.
constexpr int kJacobiIntAdds4 = 4;
constexpr bool kJacobiMulInt = true;

// HEAT_3D by default: planes per thread and integer-pipe differences
// b(+1) - 2a per two planes.  Measured on GB300 (us per half-step at 256^3,
// 4 planes): 0 of 6 on the integer pipes 243.9, 2: 219.2, 4: 194.7,
// 5: 184.8, 6: 217.2 (the integer ALU 88% busy: each such difference costs
// some 65 integer instructions); 2 planes per thread, 5 of 6: 192.6.  Sums
// (b(+1) - 2a) + b(-1) on the integer pipes measured slower at every count
// (the ALU is already the co-bound, and a second difference that nearly
// cancels leaves the close-exponent form).
constexpr int kHeatPlanes = 4;
constexpr int kHeatIntSubs2 = 5;

int b200_polybench_jacobi_2d(double* A, double* B, int64_t N, int64_t tsteps,
                             const b200_tune* tune, b200_stream_t stream) {
  if (!A || !B || N < 0 || tsteps < 0) return invalid("b200_polybench_jacobi_2d: bad args");
  if (N < 3 || tsteps == 0) return B200_OK;
  cudaStream_t st = as_stream(stream);
  if (tune && tune->algo > 0) {
    // mixed FP64 / integer pipes (algo = 1 + emulated warps of 8)
    const MixShape m = mix_shape(tune, MixShape{4, 4, 10});
    int64_t gy = ceil_div(N - 2, m.rows());
    if (gy > 65535) gy = 65535;
    dim3 g(static_cast<unsigned>(ceil_div(N - 2, 32)), static_cast<unsigned>(gy));
    for (int64_t t = 0; t < tsteps; ++t) {
      jacobi2d_mixed<<<g, 256, 0, st>>>(A, B, N, m);
      jacobi2d_mixed<<<g, 256, 0, st>>>(B, A, N, m);
    }
    return after_launch("b200_polybench_jacobi_2d", static_cast<int>(2 * tsteps));
  }
  // default: column segments of 4 rows per thread (tune->items 2, 4 or 8);
  // tune->items 1: one point per thread with rows strided over the grid
  const int rows = (tune && tune->items) ? tune->items : 4;
  if (rows != 1 && rows != 2 && rows != 4 && rows != 8)
    return invalid("b200_polybench_jacobi_2d: items %d (1, 2, 4 or 8)", rows);
  if (rows != 1) {
    constexpr int BX = 128;
    const int64_t gy = ceil_div(N - 2, rows);
    if (gy > 65535) return invalid("b200_polybench_jacobi_2d: N too large for %d rows", rows);
    const dim3 g(static_cast<unsigned>(ceil_div(N - 2, BX)), static_cast<unsigned>(gy));
    auto run = [&](auto kernel) {
      for (int64_t t = 0; t < tsteps; ++t) {
        kernel<<<g, BX, 0, st>>>(A, B, N, 0);
        kernel<<<g, BX, 0, st>>>(B, A, N, 0);
      }
    };
    // tune->tile_z = 1 + integer-pipe adds per four points (0, 4, 8, 9, 10,
    // 12); tune->tile_y 2: the product by 0.2 on the FP64 pipe
    const int kq = (tune && tune->tile_z) ? tune->tile_z - 1 : kJacobiIntAdds4;
    const bool mulint = (tune && tune->tile_y) ? tune->tile_y != 2 : kJacobiMulInt;
    auto pick = [&](auto r_tag) -> int {
      constexpr int R = decltype(r_tag)::value;
      switch (kq * 2 + (mulint ? 1 : 0)) {
        case 1: run(jacobi2d_rows<BX, R, 0, true>); break;
        case 0: run(jacobi2d_rows<BX, R, 0, false>); break;
        case 9: run(jacobi2d_rows<BX, R, 4, true>); break;
        case 8: run(jacobi2d_rows<BX, R, 4, false>); break;
        case 17: run(jacobi2d_rows<BX, R, 8, true>); break;
        case 16: run(jacobi2d_rows<BX, R, 8, false>); break;
        case 19: run(jacobi2d_rows<BX, R, 9, true>); break;
        case 18: run(jacobi2d_rows<BX, R, 9, false>); break;
        case 21: run(jacobi2d_rows<BX, R, 10, true>); break;
        case 20: run(jacobi2d_rows<BX, R, 10, false>); break;
        case 25: run(jacobi2d_rows<BX, R, 12, true>); break;
        case 24: run(jacobi2d_rows<BX, R, 12, false>); break;
        default:
          return invalid("b200_polybench_jacobi_2d: tile_z %d (1, 5, 9, 10, 11 or 13)", kq + 1);
      }
      return B200_OK;
    };
    int rc;
    if (rows == 2) rc = pick(std::integral_constant<int, 2>{});
    else if (rows == 4) rc = pick(std::integral_constant<int, 4>{});
    else rc = pick(std::integral_constant<int, 8>{});
    if (rc != B200_OK) return rc;
    return after_launch("b200_polybench_jacobi_2d", static_cast<int>(2 * tsteps));
  }
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
  cudaStream_t st = as_stream(stream);
  if (tune && tune->algo > 0) {
    const MixShape m = mix_shape(tune, MixShape{4, 2, 5});
    const int64_t chunk = (tune->tile_x > 0) ? tune->tile_x : 32;
    const int64_t gy = ceil_div(N - 2, m.rows()), gz = ceil_div(N - 2, chunk);
    if (gy > 65535 || gz > 65535) return invalid("b200_polybench_heat_3d: N too large");
    dim3 g(static_cast<unsigned>(ceil_div(N - 2, 32)), static_cast<unsigned>(gy),
           static_cast<unsigned>(gz));
    for (int64_t t = 0; t < tsteps; ++t) {
      heat3d_mixed<<<g, 256, 0, st>>>(A, B, N, m, chunk);
      heat3d_mixed<<<g, 256, 0, st>>>(B, A, N, m, chunk);
    }
    return after_launch("b200_polybench_heat_3d", static_cast<int>(2 * tsteps));
  }
  constexpr int BX = 32, BY = 8;
  // tile_x = planes per thread (2 or 4), tile_z = 1 + differences on the
  // integer pipes per two planes (0..6); 0 keeps the defaults
  const int pl = (tune && tune->tile_x > 0) ? tune->tile_x : kHeatPlanes;
  const int ks2 = (tune && tune->tile_z > 0) ? tune->tile_z - 1 : kHeatIntSubs2;
  if ((pl != 2 && pl != 4) || ks2 < 0 || ks2 > 6)
    return invalid("b200_polybench_heat_3d: bad tile_x/tile_z");
  const int64_t gz = ceil_div(N - 2, pl);
  if (ceil_div(N - 2, BY) > 65535 || gz > 65535) return invalid("b200_polybench_heat_3d: N too large");
  dim3 g(static_cast<unsigned>(ceil_div(N - 2, BX)), static_cast<unsigned>(ceil_div(N - 2, BY)),
         static_cast<unsigned>(gz));
  auto run = [&](auto kernel) {
    for (int64_t t = 0; t < tsteps; ++t) {
      kernel<<<g, dim3(BX, BY), 0, st>>>(A, B, N, 0);
      kernel<<<g, dim3(BX, BY), 0, st>>>(B, A, N, 0);
    }
  };
  auto by_ks = [&](auto P) {
    constexpr int kP = decltype(P)::value;
    switch (ks2) {
      case 0: run(heat3d_step<BX, BY, kP, 0>); break;
      case 1: run(heat3d_step<BX, BY, kP, 1>); break;
      case 2: run(heat3d_step<BX, BY, kP, 2>); break;
      case 3: run(heat3d_step<BX, BY, kP, 3>); break;
      case 4: run(heat3d_step<BX, BY, kP, 4>); break;
      case 5: run(heat3d_step<BX, BY, kP, 5>); break;
      default: run(heat3d_step<BX, BY, kP, 6>); break;
    }
  };
  if (pl == 2) by_ks(std::integral_constant<int, 2>{});
  else by_ks(std::integral_constant<int, 4>{});
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
    fdtd2d_e<BX, BY><<<ge, dim3(BX, BY), 0, st>>>(ex, ey, hz, fict, t, nx, ny, 0);
    if (nx > 1 && ny > 1) fdtd2d_h<BX, BY><<<gh, dim3(BX, BY), 0, st>>>(ex, ey, hz, nx, ny, 0);
  }
  int per = (nx > 1 && ny > 1) ? 2 : 1;
  return after_launch("b200_polybench_fdtd_2d", static_cast<int>(per * tsteps));
}

size_t b200_fdtd_2d_workspace_bytes(int64_t nx, int64_t ny) {
  if (nx <= 0 || ny <= 0) return 0;
  return 2 * static_cast<size_t>(fdtd_snap_doubles(nx, ny, kFdtdMinRows)) * sizeof(double);
}

int b200_polybench_fdtd_2d_ws(double* ex, double* ey, double* hz, const double* fict,
                              int64_t nx, int64_t ny, int64_t tsteps, void* workspace,
                              size_t workspace_bytes, const b200_tune* tune,
                              b200_stream_t stream) {
  if (!ex || !ey || !hz || !fict || nx < 0 || ny < 0 || tsteps < 0)
    return invalid("b200_polybench_fdtd_2d_ws: bad args");
  const int algo = tune ? tune->algo : 0;
  if (algo != 0 && algo != 1) return invalid("b200_polybench_fdtd_2d_ws: algo %d (0 or 1)", algo);
  if (algo == 1) return b200_polybench_fdtd_2d(ex, ey, hz, fict, nx, ny, tsteps, tune, stream);
  const int th = (tune && tune->tile_y) ? tune->tile_y : kFdtdDefaultRows;
  if (th != 8 && th != 16 && th != 32)
    return invalid("b200_polybench_fdtd_2d_ws: tile_y %d (8, 16 or 32 rows)", th);
  if (nx == 0 || ny == 0 || tsteps == 0) return B200_OK;
  if (fdtd_tile_rows(nx, th) > 65535) return invalid("b200_polybench_fdtd_2d_ws: nx too large");
  const size_t need = b200_fdtd_2d_workspace_bytes(nx, ny);
  if (!workspace || workspace_bytes < need) {
    set_error("b200_polybench_fdtd_2d_ws: workspace %zu bytes, need %zu", workspace_bytes, need);
    return B200_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  double* w = static_cast<double*>(workspace);
  const int rc = th == 8    ? launch_fdtd_fused<8>(ex, ey, hz, fict, nx, ny, tsteps, w, st)
                 : th == 16 ? launch_fdtd_fused<16>(ex, ey, hz, fict, nx, ny, tsteps, w, st)
                            : launch_fdtd_fused<32>(ex, ey, hz, fict, nx, ny, tsteps, w, st);
  if (rc != B200_OK) return rc;
  return after_launch("b200_polybench_fdtd_2d_ws", static_cast<int>(1 + tsteps));
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
