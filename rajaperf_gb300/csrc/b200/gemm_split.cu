// Split-precision FP64 GEMM: C = alpha*A*B + beta*C on bf16 tensor cores.
//
// Ozaki-style splitting with exact integer slices:
//  1. Every row i of A gets a power-of-two scale 2^Ea(i) with
//     |A(i,k)| < 2^(Ea(i)-1); every column j of B likewise 2^Eb(j).
//  2. q = round(A(i,k) * 2^(5S - Ea(i))) is an integer with |q| <= 2^(5S-1)
//     (S slices of 5 bits); its base-32 digits d_1..d_S (d_1 most
//     significant; d_2..d_S balanced in [-16, 15], |d_1| <= 17) are stored as
//     bf16, which holds them exactly.  B is cut the same way and stored
//     transposed (N x K).
//  3. For every digit weight w = s + t the products A_s * B_t are summed over
//     k on the tensor cores in one FP32 accumulator.  Each product is an
//     integer of magnitude <= 289 and K <= kMaxK, so every partial sum is an
//     integer below 2^24 whenever at most 7 slice pairs share a weight: the
//     tensor-core accumulation is exact for the weights that carry the result
//     (larger weights contribute below 2^-45 of it).
//  4. The epilogue adds 2^(-5w) * acc_w into an FP64 accumulator, and finally
//     C = alpha * 2^(Ea+Eb-10S) * acc64 + beta * C in FP64.
// Only weights w <= S + 1 are formed (the dropped products lie below the
// slicing error).  The error against an FP64 GEMM is measured per size by the
// tests and bench.
//
// Engine: mma.sync.m16n8k16 bf16 -> fp32, 128x128 C tile per CTA (8 warps of
// 64x32), 32-wide K stages double-buffered through shared memory with cp.async.
#include "b200_internal.cuh"

#include <cuda_bf16.h>

using namespace b200;

namespace {

constexpr int kSliceBits = 5;
constexpr int kMaxSlices = 12;
constexpr int kDefaultSlices = 11;
constexpr int64_t kMaxK = 8192;  // exactness bound of the FP32 accumulation
constexpr int TM = 128, TN = 128, TK = 32;
constexpr int kLds = TK + 8;     // padded smem row (80 bytes): conflict-free ldmatrix

inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// ---- scaling -----------------------------------------------------------------
// Exponent E with max|row| < 2^(E-1), i.e. E = frexp exponent of the max + 1.
__device__ __forceinline__ int scale_exponent(double amax) {
  if (amax == 0.0 || !isfinite(amax)) return 0;
  int e;
  frexp(amax, &e);
  return e + 1;
}

__global__ void row_scale_kernel(const double* __restrict__ A, int64_t M, int64_t K,
                                 int* __restrict__ E) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (i >= M) return;
  double m = 0.0;
  for (int64_t k = lane; k < K; k += 32) m = fmax(m, fabs(__ldg(A + i * K + k)));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if (lane == 0) E[i] = scale_exponent(m);
}

__global__ void col_scale_kernel(const double* __restrict__ B, int64_t K, int64_t N,
                                 int* __restrict__ E) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= N) return;
  double m = 0.0;
  for (int64_t k = 0; k < K; ++k) m = fmax(m, fabs(__ldg(B + k * N + j)));
  E[j] = scale_exponent(m);
}

// Base-32 digits of q = round(v * 2^shift), |q| <= 2^(5S-1): the S-1 low
// digits are balanced (in [-16, 15]); the top digit takes what is left,
// |d_0| <= 17 (balanced digits alone only reach 0.484 * 32^S).
__device__ __forceinline__ void digits_of(double v, int shift, int S, float* d) {
  long long q = __double2ll_rn(scalbn(v, shift));
  for (int s = S - 1; s >= 1; --s) {
    long long r = ((q + 16) & 31) - 16;   // in [-16, 15]
    d[s] = static_cast<float>(r);
    q = (q - r) >> kSliceBits;
  }
  d[0] = static_cast<float>(q);
}

// As[s][i][k] (Mp x Kp, zero padded) from A (M x K).
__global__ void slice_a_kernel(const double* __restrict__ A, int64_t M, int64_t K,
                               const int* __restrict__ E, int S, int64_t Mp, int64_t Kp,
                               __nv_bfloat16* __restrict__ As) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t i = blockIdx.y;
  if (k >= Kp) return;
  float d[kMaxSlices];
  if (i < M && k < K) {
    digits_of(__ldg(A + i * K + k), kSliceBits * S - E[i], S, d);
  } else {
    for (int s = 0; s < S; ++s) d[s] = 0.f;
  }
  for (int s = 0; s < S; ++s) As[(s * Mp + i) * Kp + k] = __float2bfloat16_rn(d[s]);
}

// Bt[t][j][k] (Np x Kp) from B (K x N): a 32x32 tile transpose through smem.
__global__ void slice_b_kernel(const double* __restrict__ B, int64_t K, int64_t N,
                               const int* __restrict__ E, int S, int64_t Np, int64_t Kp,
                               __nv_bfloat16* __restrict__ Bt) {
  __shared__ signed char tile[kMaxSlices][32][33];  // digits are in [-16, 15]
  const int64_t j0 = static_cast<int64_t>(blockIdx.x) * 32, k0 = static_cast<int64_t>(blockIdx.y) * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int64_t k = k0 + r, j = j0 + tx;
    float d[kMaxSlices];
    if (k < K && j < N) {
      digits_of(__ldg(B + k * N + j), kSliceBits * S - E[j], S, d);
    } else {
      for (int s = 0; s < S; ++s) d[s] = 0.f;
    }
    for (int s = 0; s < S; ++s) tile[s][r][tx] = static_cast<signed char>(d[s]);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t j = j0 + r, k = k0 + tx;
    if (j < Np && k < Kp)
      for (int s = 0; s < S; ++s)
        Bt[(s * Np + j) * Kp + k] = __float2bfloat16_rn(static_cast<float>(tile[s][tx][r]));
  }
}

// ---- mma.sync engine -----------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void ldmatrix_x4(unsigned& r0, unsigned& r1, unsigned& r2,
                                            unsigned& r3, const void* p) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(p));
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(s));
}

__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct SplitArgs {
  const __nv_bfloat16* As;  // [S][Mp][Kp]
  const __nv_bfloat16* Bt;  // [S][Np][Kp]
  const int* Ea;
  const int* Eb;
  double* C;
  int64_t M, N, Mp, Np, Kp;
  double alpha, beta;
  int S;
};

__global__ void __launch_bounds__(256, 1) ozaki_mma_kernel(SplitArgs g) {
  __shared__ __align__(16) __nv_bfloat16 sA[2][TM][kLds];
  __shared__ __align__(16) __nv_bfloat16 sB[2][TN][kLds];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps, 64 x 32 each
  const int64_t i0 = static_cast<int64_t>(blockIdx.y) * TM;
  const int64_t j0 = static_cast<int64_t>(blockIdx.x) * TN;
  const int64_t ksteps = g.Kp / TK;

  double acc64[4][4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc64[a][b][c] = 0.0;

  // stage loader: 128 rows x 32 bf16 = 512 chunks of 16 B per operand
  auto load_stage = [&](int buf, int s, int t, int64_t k0) {
    const __nv_bfloat16* a = g.As + (static_cast<int64_t>(s) * g.Mp + i0) * g.Kp + k0;
    const __nv_bfloat16* b = g.Bt + (static_cast<int64_t>(t) * g.Np + j0) * g.Kp + k0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int c = tid + r * 256;
      const int row = c >> 2, col = (c & 3) * 8;
      cp_async16(&sA[buf][row][col], a + row * g.Kp + col);
      cp_async16(&sB[buf][row][col], b + row * g.Kp + col);
    }
    cp_async_commit();
  };

  for (int w = 2; w <= g.S + 1; ++w) {
    const int s_lo = (w - g.S > 1) ? w - g.S : 1;
    const int s_hi = (w - 1 < g.S) ? w - 1 : g.S;
    const int64_t iters = static_cast<int64_t>(s_hi - s_lo + 1) * ksteps;
    float acc[4][4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;

    load_stage(0, s_lo - 1, w - s_lo - 1, 0);
    for (int64_t it = 0; it < iters; ++it) {
      const int buf = static_cast<int>(it & 1);
      cp_async_wait0();
      __syncthreads();
      if (it + 1 < iters) {
        const int64_t nx = it + 1;
        const int s = s_lo + static_cast<int>(nx / ksteps);
        load_stage(buf ^ 1, s - 1, w - s - 1, (nx % ksteps) * TK);
      }
#pragma unroll
      for (int kk = 0; kk < TK; kk += 16) {
        unsigned af[4][4], bfr[4][2];
#pragma unroll
        for (int mi = 0; mi < 4; ++mi) {
          const int row = wm * 64 + mi * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
          const int col = kk + (lane >> 4) * 8;
          ldmatrix_x4(af[mi][0], af[mi][1], af[mi][2], af[mi][3], &sA[buf][row][col]);
        }
#pragma unroll
        for (int nj = 0; nj < 4; nj += 2) {
          const int row = wn * 32 + nj * 8 + (lane & 7) + (lane >> 4) * 8;
          const int col = kk + ((lane >> 3) & 1) * 8;
          ldmatrix_x4(bfr[nj][0], bfr[nj][1], bfr[nj + 1][0], bfr[nj + 1][1],
                      &sB[buf][row][col]);
        }
#pragma unroll
        for (int mi = 0; mi < 4; ++mi)
#pragma unroll
          for (int nj = 0; nj < 4; ++nj) mma_bf16(acc[mi][nj], af[mi], bfr[nj]);
      }
    }
    __syncthreads();
    // acc64 += 2^(-5w) * acc   (exact scaling; one FP64 add per element)
    const double wscale = scalbn(1.0, -kSliceBits * w);
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
      for (int nj = 0; nj < 4; ++nj)
#pragma unroll
        for (int c = 0; c < 4; ++c)
          acc64[mi][nj][c] = fma(static_cast<double>(acc[mi][nj][c]), wscale, acc64[mi][nj][c]);
  }

  // C = alpha * 2^(Ea+Eb-10S+10S) ... : acc64 holds sum_w 2^(-5w) P_w, and
  // A*B = 2^(Ea+Eb) * 2^(-10S) * sum_w 2^(5(2S-w)) P_w = 2^(Ea+Eb) * acc64.
  const int g4 = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t i = i0 + wm * 64 + mi * 16 + g4 + h * 8;
      if (i >= g.M) continue;
      const int ea = g.Ea[i];
#pragma unroll
      for (int nj = 0; nj < 4; ++nj) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int64_t j = j0 + wn * 32 + nj * 8 + t4 * 2 + e;
          if (j >= g.N) continue;
          const double ab = scalbn(acc64[mi][nj][h * 2 + e], ea + g.Eb[j]);
          double* p = g.C + i * g.N + j;
          *p = (g.beta == 0.0) ? g.alpha * ab : g.alpha * ab + g.beta * (*p);
        }
      }
    }
  }
}

struct SplitLayout {
  int64_t Mp, Np, Kp;
  size_t off_ea, off_eb, off_as, off_bt, total;
};

SplitLayout split_layout(int64_t m, int64_t n, int64_t k, int S) {
  SplitLayout L;
  L.Mp = round_up(m > 0 ? m : 1, TM);
  L.Np = round_up(n > 0 ? n : 1, TN);
  L.Kp = round_up(k > 0 ? k : 1, TK);
  L.off_ea = 0;
  L.off_eb = round_up(L.Mp * 4, 256);
  L.off_as = L.off_eb + round_up(L.Np * 4, 256);
  L.off_bt = L.off_as + round_up(static_cast<int64_t>(S) * L.Mp * L.Kp * 2, 256);
  L.total = L.off_bt + round_up(static_cast<int64_t>(S) * L.Np * L.Kp * 2, 256);
  return L;
}

int slices_of(const b200_tune* t) {
  return (t && t->items) ? t->items : kDefaultSlices;
}

}  // namespace

extern "C" {

size_t b200_gemm_split_workspace_bytes(int64_t m, int64_t n, int64_t k, const b200_tune* tune) {
  return split_layout(m, n, k, slices_of(tune)).total;
}

int b200_gemm_split(const double* A, const double* B, double* C, int64_t m, int64_t n,
                    int64_t k, double alpha, double beta, void* workspace,
                    size_t workspace_bytes, const b200_tune* tune, b200_stream_t stream) {
  if (!A || !B || !C || m < 0 || n < 0 || k < 0) return invalid("b200_gemm_split: bad args");
  const int S = slices_of(tune);
  if (S < 2 || S > kMaxSlices) return invalid("b200_gemm_split: slices %d not in [2, %d]", S, kMaxSlices);
  if (k > kMaxK)
    return invalid("b200_gemm_split: k = %lld exceeds %lld (FP32 exactness bound)",
                   static_cast<long long>(k), static_cast<long long>(kMaxK));
  if (m == 0 || n == 0) return B200_OK;
  SplitLayout L = split_layout(m, n, k, S);
  if (!workspace || workspace_bytes < L.total) {
    set_error("b200_gemm_split: workspace %zu bytes, need %zu", workspace_bytes, L.total);
    return B200_ERR_WORKSPACE;
  }
  if (L.Mp / TM > 65535) return invalid("b200_gemm_split: m too large");
  char* w = static_cast<char*>(workspace);
  int* Ea = reinterpret_cast<int*>(w + L.off_ea);
  int* Eb = reinterpret_cast<int*>(w + L.off_eb);
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(w + L.off_as);
  __nv_bfloat16* Bt = reinterpret_cast<__nv_bfloat16*>(w + L.off_bt);
  cudaStream_t st = as_stream(stream);
  // zero-sized k: C = beta*C through the same epilogue (all digits zero)
  row_scale_kernel<<<static_cast<unsigned>(ceil_div(m, 8)), 256, 0, st>>>(A, m, k, Ea);
  col_scale_kernel<<<static_cast<unsigned>(ceil_div(n, 256)), 256, 0, st>>>(B, k, n, Eb);
  if (L.Mp > 65535) return invalid("b200_gemm_split: m too large");
  slice_a_kernel<<<dim3(static_cast<unsigned>(ceil_div(L.Kp, 256)), static_cast<unsigned>(L.Mp)),
                   256, 0, st>>>(A, m, k, Ea, S, L.Mp, L.Kp, As);
  slice_b_kernel<<<dim3(static_cast<unsigned>(ceil_div(L.Np, 32)), static_cast<unsigned>(ceil_div(L.Kp, 32))),
                   dim3(32, 8), 0, st>>>(B, k, n, Eb, S, L.Np, L.Kp, Bt);
  SplitArgs g{As, Bt, Ea, Eb, C, m, n, L.Mp, L.Np, L.Kp, alpha, beta, S};
  ozaki_mma_kernel<<<dim3(static_cast<unsigned>(L.Np / TN), static_cast<unsigned>(L.Mp / TM)),
                     256, 0, st>>>(g);
  return after_launch("b200_gemm_split", 5);
}

}  // extern "C"
