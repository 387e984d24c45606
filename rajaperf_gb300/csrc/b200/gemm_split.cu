// Split-precision FP64 GEMM: C = alpha*A*B + beta*C on FP8 (or bf16) tensor
// cores.
//
// Ozaki-style splitting with exact integer slices:
//  1. Every row i of A gets a power-of-two scale 2^Ea(i) with
//     |A(i,k)| < 2^(Ea(i)-1); every column j of B likewise 2^Eb(j).
//  2. q = round(A(i,k) * 2^(5S - Ea(i))) is an integer with |q| <= 2^(5S-1)
//     (S slices of 5 bits); its base-32 digits d_1..d_S (d_1 most
//     significant; d_2..d_S balanced in [-16, 15], |d_1| <= 16) are stored as
//     e4m3 bytes (or bf16), which hold every integer of magnitude <= 16
//     exactly.  B is cut the same way and stored transposed (N x K).
//  3. For every digit weight w = s + t the products A_s * B_t are summed over
//     a chunk of k on the tensor cores in one FP32 accumulator.  Each product
//     is an integer of magnitude <= 256 and a chunk holds at most kChunkK = 8192
//     values of k, so every partial sum is an integer of magnitude at most 2^24
//     (exact in FP32) whenever at most 8 slice pairs share a weight: the tensor-core accumulation is exact
//     for the weights that carry the result (larger weights contribute below
//     2^-45 of it).  Longer K is cut into balanced chunks of at most kChunkK.
//  4. The epilogue adds 2^(-5w) * acc_(w,chunk) into an FP64 accumulator after
//     every chunk, and finally C = alpha * 2^(Ea+Eb-10S) * acc64 + beta * C in
//     FP64.
// Only weights w <= S + 1 are formed (the dropped products lie below the
// slicing error).  The error against an FP64 GEMM is measured per size by the
// tests and bench.  The e4m3 and bf16 slices hold the same digits, so the
// engines' results agree bit for bit whenever the accumulation is exact.
//
// Engines (tune->algo; 0 picks 4):
//  4 tcgen05 on e4m3 slices with the digit weights in pairs (128 x 256 MMAs;
//    see the paired-weight engine below): the default.
//  3 tcgen05 on e4m3 slices, 2 the same on bf16 slices: one 128x128 C tile
//    per CTA (CTAs ordered in groups of 8 tile rows, so that resident CTAs
//    share operand tiles in L2).  Warp 0 streams 128 x (128 bytes of k) slice
//    tiles of A and B into a 7-stage shared-memory ring with TMA (128-byte
//    swizzle); warp 1
//    issues tcgen05.mma (kind::f8f6f4: 32 values of k per instruction, or
//    kind::f16: 16; FP32 out) into one of two FP32 accumulators in tensor
//    memory, one per digit weight; warps 2-5 read a finished weight's
//    accumulator with tcgen05.ld and fold it into an FP64 accumulator that
//    also lives in tensor memory (two 32-bit columns per element), so weight
//    w+1's MMAs overlap weight w's FP64 epilogue.  TMEM: 2 x 128 FP32 columns
//    + 256 FP64 columns = 512.  An e4m3 tile carries twice the k of a bf16
//    tile in the same 16 KB, so the shared-memory traffic per MMA flop halves.
//  1 mma.sync.m16n8k16 bf16 -> fp32, 128x128 C tile per CTA (8 warps of
//    64x32), 32-wide K stages double-buffered through shared memory with
//    cp.async (the legacy tensor-core path, kept for comparison).
// Every wait of the tcgen05 engines is bounded (1 s by default,
// b200_tune.wait_limit_us); one that gives up sets the error word at byte
// offset 16 of the workspace and the CTA winds down.
#include "b200_internal.cuh"
#include "b200_async.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <mutex>

using namespace b200;

namespace {

constexpr int kSliceBits = 5;
constexpr int kMaxSlices = 12;
// Default slice count, from the measured relative Frobenius error against an
// FP64 GEMM (uniform [-1, 1) data, rows or columns scaled by 2^[-20, 20],
// all-positive data; K = 1024 .. 20000): about 4.5 * 32^-S, growing like
// K^0.15.  S = 9 gives 0.9-1.3e-13 (above the 1e-13 target at every K
// measured); S = 10 gives 3-5e-15, 20x inside it up to K = 20000, with 55
// slice products per element instead of S = 11's 66.
constexpr int kDefaultSlices = 10;
constexpr int64_t kChunkK = 8192;  // exactness bound of one FP32 accumulation
// Longest K: 64 chunks (the chunk arithmetic and TMA coordinates stay in int).
constexpr int64_t kMaxK = 64 * kChunkK;
constexpr int TM = 128, TN = 128, TK = 32;
constexpr int kLds = TK + 8;     // padded smem row (80 bytes): conflict-free ldmatrix
constexpr int kPadK = 64;        // K padding of the slice arrays (one TMA row = 128 B)

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

// Column maxima of |B| (K x N): 32 columns x kColRows rows per CTA (32 x 8
// threads, coalesced along the row), folded into bmax[j] with one atomicMax
// per column and CTA (the bits of non-negative doubles order as unsigned
// integers).  bmax starts zeroed.
constexpr int kColRows = 256;
__global__ void __launch_bounds__(256)
col_max_kernel(const double* __restrict__ B, int64_t K, int64_t N,
               unsigned long long* __restrict__ bmax) {
  __shared__ double part[8][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t j = static_cast<int64_t>(blockIdx.x) * 32 + tx;
  const int64_t k0 = static_cast<int64_t>(blockIdx.y) * kColRows;
  const int64_t k1 = (k0 + kColRows < K) ? k0 + kColRows : K;
  double m = 0.0;
  if (j < N)
    for (int64_t k = k0 + ty; k < k1; k += 8) m = fmax(m, fabs(__ldg(B + k * N + j)));
  part[ty][tx] = m;
  __syncthreads();
  if (ty == 0 && j < N) {
#pragma unroll
    for (int r = 1; r < 8; ++r) m = fmax(m, part[r][tx]);
    atomicMax(bmax + j, static_cast<unsigned long long>(__double_as_longlong(m)));
  }
}

// Base-32 digits of q = round(v * 2^shift), |q| <= 2^(5S-1) = 16 * 32^(S-1):
// the S-1 low digits are balanced (in [-16, 15], together within
// [-0.52, 0.49] * 32^(S-1)); the top digit takes what is left, an integer of
// magnitude below 16.52, so |d_0| <= 16.

// Digit e (0-based) of a 16-byte word of slice digits in the arrays'
// storage type: e4m3 bytes (exact for the integers |d| <= 16) or bf16.
template <typename T>
__device__ __forceinline__ void pack_digit(uint32_t (&w)[4], int e, int d) {
  if constexpr (sizeof(T) == 1) {
    const uint32_t b = static_cast<uint32_t>(
        __nv_cvt_float_to_fp8(static_cast<float>(d), __NV_SATFINITE, __NV_E4M3));
    w[e >> 2] |= b << (8 * (e & 3));
  } else {
    const uint32_t h = __bfloat16_as_ushort(__float2bfloat16_rn(static_cast<float>(d)));
    w[e >> 1] |= h << (16 * (e & 1));
  }
}

// The S digits of q = round(v * 2^shift) (as digits_of), slice s into w[s]
// at position e; slices are indexed at compile time (kept in registers).
template <typename T>
__device__ __forceinline__ void put_digits(double v, int shift, int S, int e,
                                           uint32_t (&w)[kMaxSlices][4]) {
  long long q = __double2ll_rn(scalbn(v, shift));
#pragma unroll
  for (int s = kMaxSlices - 1; s >= 1; --s) {
    if (s < S) {
      const long long r = ((q + 16) & 31) - 16;   // in [-16, 15]
      pack_digit<T>(w[s], e, static_cast<int>(r));
      q = (q - r) >> kSliceBits;
    }
  }
  pack_digit<T>(w[0], e, static_cast<int>(q));
}

// As[s][i][k] (Mp x Kp, zero padded) from A (M x K): a thread forms the digits
// of 16 bytes' worth of consecutive k of one row (16 e4m3 or 8 bf16 digits
// per slice) and writes one 16-byte word to every slice.
template <typename T>
__global__ void __launch_bounds__(128)
slice_a_kernel(const double* __restrict__ A, int64_t M, int64_t K, const int* __restrict__ E,
               int S, int64_t Mp, int64_t Kp, T* __restrict__ As) {
  constexpr int kPer = 16 / static_cast<int>(sizeof(T));
  const int64_t k0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * kPer;
  const int64_t i = blockIdx.y;
  if (k0 >= Kp) return;
  const bool row = i < M;
  const int shift = row ? kSliceBits * S - E[i] : 0;
  uint32_t w[kMaxSlices][4];
#pragma unroll
  for (int s = 0; s < kMaxSlices; ++s) w[s][0] = w[s][1] = w[s][2] = w[s][3] = 0u;
#pragma unroll
  for (int e = 0; e < kPer; ++e) {
    const int64_t k = k0 + e;
    const double v = (row && k < K) ? __ldg(A + i * K + k) : 0.0;
    put_digits<T>(v, shift, S, e, w);
  }
#pragma unroll
  for (int s = 0; s < kMaxSlices; ++s)
    if (s < S)
      *reinterpret_cast<uint4*>(As + (s * Mp + i) * Kp + k0) =
          make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Bt[t][j][k] (Np x Kp) from B (K x N): a 32 (k) x 64 (j) tile per CTA of
// 256 threads.  Reads run along B's rows (coalesced); the digits go through
// shared memory (row stride 36 bytes: a warp's byte stores hit 32 banks) and
// leave as 16-byte words along Bt's rows.  The CTAs of the first k tile also
// write the column exponents Eb from the column maxima.
constexpr int kBtK = 32, kBtJ = 64;
template <typename T>
__global__ void __launch_bounds__(256)
slice_b_kernel(const double* __restrict__ B, int64_t K, int64_t N,
               const unsigned long long* __restrict__ bmax, int* __restrict__ Eb, int S,
               int64_t Np, int64_t Kp, T* __restrict__ Bt) {
  constexpr int kPer = 16 / static_cast<int>(sizeof(T));
  constexpr int kChunks = kBtK / kPer;  // 16-byte words per Bt row of the tile
  __shared__ __align__(16) signed char dig[kMaxSlices][kBtJ][kBtK + 4];
  __shared__ int sE[kBtJ];
  const int tid = threadIdx.x;
  const int64_t j0 = static_cast<int64_t>(blockIdx.x) * kBtJ;
  const int64_t k0 = static_cast<int64_t>(blockIdx.y) * kBtK;
  if (tid < kBtJ) {
    const int64_t j = j0 + tid;
    int e = 0;
    if (j < N) {
      e = scale_exponent(__longlong_as_double(static_cast<long long>(bmax[j])));
      if (blockIdx.y == 0) Eb[j] = e;
    }
    sE[tid] = e;
  }
  __syncthreads();
  const int jj = tid & (kBtJ - 1);
  const int64_t j = j0 + jj;
  const int shift = kSliceBits * S - sE[jj];
#pragma unroll 2
  for (int r = 0; r < kBtK / 4; ++r) {
    const int kk = (tid >> 6) + 4 * r;
    const int64_t k = k0 + kk;
    const double v = (k < K && j < N) ? __ldg(B + k * N + j) : 0.0;
    long long q = __double2ll_rn(scalbn(v, shift));
#pragma unroll
    for (int s = kMaxSlices - 1; s >= 1; --s) {
      if (s < S) {
        const long long d = ((q + 16) & 31) - 16;
        dig[s][jj][kk] = static_cast<signed char>(d);
        q = (q - d) >> kSliceBits;
      }
    }
    dig[0][jj][kk] = static_cast<signed char>(q);
  }
  __syncthreads();
  for (int c = tid; c < S * kBtJ * kChunks; c += 256) {
    const int s = c / (kBtJ * kChunks), rem = c % (kBtJ * kChunks);
    const int row = rem / kChunks, ch = rem % kChunks;
    uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int e = 0; e < kPer; ++e) pack_digit<T>(w, e, dig[s][row][ch * kPer + e]);
    *reinterpret_cast<uint4*>(Bt + (s * Np + j0 + row) * Kp + k0 + ch * kPer) =
        make_uint4(w[0], w[1], w[2], w[3]);
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

  // K in balanced chunks of at most kChunkK (whole TK steps), each summed
  // exactly in FP32 and folded into the FP64 accumulator
  const int64_t nchunks = (ksteps * TK + kChunkK - 1) / kChunkK;
  const int64_t chunk_steps = (ksteps + nchunks - 1) / nchunks;
  for (int pass = 0; pass < (g.S) * static_cast<int>(nchunks); ++pass) {
    const int w = 2 + pass / static_cast<int>(nchunks);
    const int64_t c0 = (pass % nchunks) * chunk_steps;
    const int64_t csteps = (c0 + chunk_steps < ksteps) ? chunk_steps : ksteps - c0;
    const int s_lo = (w - g.S > 1) ? w - g.S : 1;
    const int s_hi = (w - 1 < g.S) ? w - 1 : g.S;
    const int64_t iters = static_cast<int64_t>(s_hi - s_lo + 1) * csteps;
    float acc[4][4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;

    load_stage(0, s_lo - 1, w - s_lo - 1, c0 * TK);
    for (int64_t it = 0; it < iters; ++it) {
      const int buf = static_cast<int>(it & 1);
      cp_async_wait0();
      __syncthreads();
      if (it + 1 < iters) {
        const int64_t nx = it + 1;
        const int s = s_lo + static_cast<int>(nx / csteps);
        load_stage(buf ^ 1, s - 1, w - s - 1, (c0 + nx % csteps) * TK);
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

// ---- tcgen05 engine ------------------------------------------------------------
namespace tc {

constexpr int BM = 128, BN = 128;
constexpr int kRowBytes = 128;                      // one 128-byte swizzle row of K
// k values per k block: 64 bf16 or 128 e4m3 (one swizzle row either way)
template <bool F8> constexpr int kBK = F8 ? 128 : 64;
constexpr int kStages = 7;                          // 7 x 32 KB of operand tiles in flight
constexpr uint32_t kTileBytes = BM * kRowBytes;     // 16 KB per operand tile
constexpr int kRasterRows = 8;                      // tile rows per raster group
constexpr uint32_t kStageBytes = 2 * kTileBytes;    // A + B
constexpr int kThreads = 192;                       // TMA, MMA, 4 epilogue warps
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kAcc64Col = 2 * BN;              // FP64 accumulator columns 256..511
constexpr uint64_t kWaitLimitNs = 1000000000ull;    // default wait limit: 1 s
constexpr size_t kSmemBytes = 1024 + kStages * kStageBytes + 256;

// Instruction descriptors: D = F32 (bits 4-5 = 1), both operands K-major,
// N >> 3 at bits 17-22, M >> 4 at 24-28; A and B formats at bits 7-9 and
// 10-12: kind::f16 BF16 = 1, kind::f8f6f4 E4M3 = 0 (A and B the same type).
constexpr uint32_t kIdescShape = (1u << 4) | (static_cast<uint32_t>(BN >> 3) << 17) |
                                 (static_cast<uint32_t>(BM >> 4) << 24);
template <bool F8>
constexpr uint32_t kIdesc = F8 ? kIdescShape : (kIdescShape | (1u << 7) | (1u << 10));
static_assert(kSmemBytes <= 232448, "shared memory budget");

// Waits for the phase of parity `parity` to complete.  Gives up after
// limit_ns (setting the CTA's abort flag) or when another role has aborted.
__device__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag,
                          uint64_t limit_ns) {
  if (mbar_try_wait(b, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (;;) {
    if (mbar_try_wait(b, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > limit_ns) {
      *abort_flag = 1;
      return false;
    }
  }
}
// The same wait for the wind-down after an abort: bounded, ignores the flag.
__device__ bool mbar_wait_drain(uint64_t* b, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(b, parity))
    if (globaltimer() - t0 > limit_ns) return false;
  return true;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// K-major operand tile of 8-row x 128-byte swizzle atoms (as TMA's 128-byte
// swizzle writes it): start >> 4, leading offset 16 B (unused for this
// layout), stride 1024 B between 8-row groups, descriptor version 1,
// swizzle mode 2 (128 B).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (1ull << 16) |
         (static_cast<uint64_t>(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}
// One 128 x 128 x (32 bytes of K) MMA: 16 bf16 (kind::f16) or 32 e4m3
// (kind::f8f6f4) values of k, FP32 accumulation in tensor memory.
template <bool F8>
__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                     uint32_t accumulate) {
  if constexpr (F8) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc<true>), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc<false>), "r"(accumulate)
        : "memory");
  }
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// tcgen05.wait::ld, tied to the loaded registers so that no use of them is
// scheduled before the wait.
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}
__device__ __forceinline__ void tmem_keep(uint32_t (&r)[16]) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ double pair_to_double(uint32_t lo, uint32_t hi) {
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

// This CTA's tile row (rows = true) or column under the grouped raster: CTA
// id c = blockIdx.y * gridDim.x + blockIdx.x; group g = c / (G * nx) covers
// tile rows [g G, g G + G) (fewer in the last group), column-major inside.
__device__ __forceinline__ int raster_tile(bool rows) {
  const int nx = static_cast<int>(gridDim.x), ny = static_cast<int>(gridDim.y);
  const int c = static_cast<int>(blockIdx.y) * nx + static_cast<int>(blockIdx.x);
  const int group = kRasterRows * nx;
  const int first = (c / group) * kRasterRows;
  const int rows_in = (ny - first < kRasterRows) ? ny - first : kRasterRows;
  const int r = c % group;
  return rows ? first + r % rows_in : r / rows_in;
}

struct TcArgs {
  const int* Ea;
  const int* Eb;
  double* C;
  unsigned int* error;
  int64_t M, N, Mp, Np, Kp;
  double alpha, beta;
  int S;
  uint64_t limit_ns;  // limit of every bounded wait
};

template <bool F8>
__global__ void __launch_bounds__(kThreads, 1)
ozaki_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                TcArgs g) {
  constexpr int BK = kBK<F8>;
  extern __shared__ unsigned char smem_raw[];
  // stage ring aligned to 1024 B (the 128-byte swizzle atom), then barriers
  unsigned char* ring = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* acc_full = empty + kStages;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int st = 0; st < kStages; ++st) {
      mbar_init(full + st, 1);
      mbar_init(empty + st, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full + b, 1);
      mbar_init(acc_empty + b, 4);  // one arrival per epilogue warp
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    mbar_init_fence();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int S = g.S;
  const int nkb = static_cast<int>(g.Kp / BK);
  // K in balanced chunks of at most kChunkK (whole k blocks); a pass is one
  // (weight, chunk): its slice products accumulate in one FP32 buffer, which
  // the epilogue folds into the FP64 accumulator
  const int nch = static_cast<int>((static_cast<int64_t>(nkb) * BK + kChunkK - 1) / kChunkK);
  const int ckb = (nkb + nch - 1) / nch;
  const int npass = S * nch;
  // Raster: consecutive CTAs walk groups of kRasterRows tile rows column by
  // column, so the CTAs resident together share A rows and B columns in L2.
  const int64_t i0 = static_cast<int64_t>(raster_tile(true)) * BM;
  const int64_t j0 = static_cast<int64_t>(raster_tile(false)) * BN;

  if (warp == 0) {
    if (lane == 0) {
      // producer: (pass, slice pair, k block) in the MMA warp's order
      uint32_t it = 0;
      bool ok = true;
      for (int p = 0; ok && p < npass; ++p) {
        const int w = 2 + p / nch;
        const int kb0 = (p % nch) * ckb;
        const int kb1 = (kb0 + ckb < nkb) ? kb0 + ckb : nkb;
        for (int s = 1; ok && s <= w - 1; ++s) {
          const int t = w - s;
          for (int kb = kb0; kb < kb1; ++kb, ++it) {
            const int st = static_cast<int>(it % kStages);
            const uint32_t ph = (it / kStages) & 1u;
            if (!mbar_wait(empty + st, ph ^ 1u, abort_flag, g.limit_ns)) {
              ok = false;
              break;
            }
            unsigned char* a = ring + st * kStageBytes;
            mbar_arrive_expect_tx(full + st, kStageBytes);
            tma_load_2d(a, &tmA, full + st, kb * BK, static_cast<int>((s - 1) * g.Mp + i0));
            tma_load_2d(a + kTileBytes, &tmB, full + st, kb * BK,
                        static_cast<int>((t - 1) * g.Np + j0));
          }
        }
      }
      if (!ok) {
        // wind-down: let the copies already issued land before the CTA exits
        const uint32_t first = it > static_cast<uint32_t>(kStages) ? it - kStages : 0u;
        for (uint32_t j = first; j < it; ++j)
          mbar_wait_drain(full + (j % kStages), (j / kStages) & 1u, g.limit_ns);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int wi = 0; ok && wi < npass; ++wi) {
        const int w = 2 + wi / nch;
        const int kb0 = (wi % nch) * ckb;
        const int kb1 = (kb0 + ckb < nkb) ? kb0 + ckb : nkb;
        const int buf = wi & 1;
        const uint32_t use = static_cast<uint32_t>(wi >> 1);
        if (!mbar_wait(acc_empty + buf, (use & 1u) ^ 1u, abort_flag, g.limit_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d_acc = tmem + static_cast<uint32_t>(buf * BN);
        uint32_t accumulate = 0u;
        for (int s = 1; ok && s <= w - 1; ++s) {
          for (int kb = kb0; kb < kb1; ++kb, ++it) {
            const int st = static_cast<int>(it % kStages);
            if (!mbar_wait(full + st, (it / kStages) & 1u, abort_flag, g.limit_ns)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a_addr = smem_u32(ring + st * kStageBytes);
            const uint64_t ad = sw128_desc(a_addr), bd = sw128_desc(a_addr + kTileBytes);
#pragma unroll
            for (int kk = 0; kk < kRowBytes / 32; ++kk) {
              // advance 32 bytes along K inside the swizzle atom
              umma<F8>(d_acc, ad + 2u * kk, bd + 2u * kk, accumulate);
              accumulate = 1u;
            }
            umma_commit(empty + st);
          }
        }
        if (ok) umma_commit(acc_full + buf);
      }
      // every MMA issued by this thread completes before teardown
      umma_commit(mma_done);
      mbar_wait_drain(mma_done, 0u, g.limit_ns);
    }
  } else {
    // epilogue warps 2..5 own TMEM lane quadrants (warp % 4): tile row = lane
    const int q = warp & 3;
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;
    bool ok = true;
    for (int wi = 0; wi < npass; ++wi) {
      const int w = 2 + wi / nch;
      const int buf = wi & 1;
      const uint32_t use = static_cast<uint32_t>(wi >> 1);
      if (!mbar_wait(acc_full + buf, use & 1u, abort_flag, g.limit_ns)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const double wscale = scalbn(1.0, -kSliceBits * w);
      for (int c = 0; c < BN; c += 16) {
        uint32_t f[16], d0[16], d1[16];
        tmem_ld16(tmem + lane_base + static_cast<uint32_t>(buf * BN + c), f);
        if (wi > 0) {
          tmem_ld16(tmem + lane_base + kAcc64Col + static_cast<uint32_t>(2 * c), d0);
          tmem_ld16(tmem + lane_base + kAcc64Col + static_cast<uint32_t>(2 * c + 16), d1);
          tmem_ld_wait(d0);
          tmem_keep(d1);
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e) d0[e] = d1[e] = 0u;
        }
        tmem_ld_wait(f);
        tmem_keep(d1);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          double v0 = pair_to_double(d0[2 * e], d0[2 * e + 1]);
          double v1 = pair_to_double(d1[2 * e], d1[2 * e + 1]);
          v0 = fma(static_cast<double>(__uint_as_float(f[e])), wscale, v0);
          v1 = fma(static_cast<double>(__uint_as_float(f[e + 8])), wscale, v1);
          d0[2 * e] = static_cast<uint32_t>(__double2loint(v0));
          d0[2 * e + 1] = static_cast<uint32_t>(__double2hiint(v0));
          d1[2 * e] = static_cast<uint32_t>(__double2loint(v1));
          d1[2 * e + 1] = static_cast<uint32_t>(__double2hiint(v1));
        }
        tmem_st16(tmem + lane_base + kAcc64Col + static_cast<uint32_t>(2 * c), d0);
        tmem_st16(tmem + lane_base + kAcc64Col + static_cast<uint32_t>(2 * c + 16), d1);
      }
      tmem_st_wait();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty + buf);
    }
    if (ok) {
      // C = alpha * 2^(Ea+Eb) * acc64 + beta * C
      const int64_t i = i0 + 32 * q + lane;
      const bool row_ok = i < g.M;
      const int ea = row_ok ? g.Ea[i] : 0;
      for (int c = 0; c < BN; c += 16) {
        uint32_t d0[16], d1[16];
        tmem_ld16(tmem + lane_base + kAcc64Col + static_cast<uint32_t>(2 * c), d0);
        tmem_ld16(tmem + lane_base + kAcc64Col + static_cast<uint32_t>(2 * c + 16), d1);
        tmem_ld_wait(d0);
        tmem_keep(d1);
        if (row_ok) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int64_t j = j0 + c + e;
            if (j < g.N) {
              const double acc = (e < 8) ? pair_to_double(d0[2 * e], d0[2 * e + 1])
                                         : pair_to_double(d1[2 * e - 16], d1[2 * e - 15]);
              const double ab = scalbn(acc, ea + g.Eb[j]);
              double* p = g.C + i * g.N + j;
              *p = (g.beta == 0.0) ? g.alpha * ab : g.alpha * ab + g.beta * (*p);
            }
          }
        }
      }
    }
    tc_fence_before();
  }
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(g.error, 1u);
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// ---- paired-weight engine ------------------------------------------------------
// The same slices and chunks, with the digit weights taken in pairs (w, w+1),
// w = 2, 4, ...: for s = 1 .. w-1 one 128 x 256 MMA multiplies A_s by the
// stacked [B_(w-s); B_(w+1-s)] (256 rows of B in one shared-memory operand),
// so its two 128-column halves accumulate weight w and weight w+1 at once;
// A_w * B_1 (weight w+1 only) follows as a 128 x 128 MMA into the upper half.
// A stage holds A_s and two B tiles (48 KB, 4 stages): 1.5x the bytes of a
// 128 x 128 stage for 2x its MMA work, which lowers the operand bytes each SM
// must receive per tensor cycle by a quarter.  TMEM: the pair's FP32
// accumulator (256 columns) and the FP64 accumulator (256 columns).  Eight
// epilogue warps (two per TMEM lane quadrant, 64 columns each) copy the
// pair's FP32 sums to registers and release the accumulator at once, then
// fold weight w and then weight w+1 into the FP64 accumulator (the order of
// the single-weight engine, so results agree bit for bit when k <= 8192).
constexpr int kPStages = 4;
constexpr uint32_t kPStageBytes = 3 * kTileBytes;   // A, B_lo, B_hi
constexpr int kPThreads = 320;                      // TMA, MMA, 8 epilogue warps
constexpr uint32_t kPAcc64Col = 256;
constexpr size_t kPSmemBytes = 1024 + kPStages * kPStageBytes + 256;
static_assert(kPSmemBytes <= 232448, "shared memory budget");

template <bool F8, int N>
__device__ __forceinline__ void umma_n(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                       uint32_t accumulate) {
  constexpr uint32_t idesc = (1u << 4) | (static_cast<uint32_t>(N >> 3) << 17) |
                             (static_cast<uint32_t>(BM >> 4) << 24) |
                             (F8 ? 0u : ((1u << 7) | (1u << 10)));
  if constexpr (F8) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  }
}

template <bool F8>
__global__ void __launch_bounds__(kPThreads, 1)
ozaki_tc_paired_kernel(const __grid_constant__ CUtensorMap tmA,
                       const __grid_constant__ CUtensorMap tmB, TcArgs g) {
  constexpr int BK = kBK<F8>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* ring = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + kPStages * kPStageBytes);
  uint64_t* empty = full + kPStages;
  uint64_t* acc_full = empty + kPStages;
  uint64_t* acc_empty = acc_full + 1;
  uint64_t* mma_done = acc_empty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int st = 0; st < kPStages; ++st) {
      mbar_init(full + st, 1);
      mbar_init(empty + st, 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 8);  // one arrival per epilogue warp
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    mbar_init_fence();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int S = g.S;
  const int nkb = static_cast<int>(g.Kp / BK);
  const int nch = static_cast<int>((static_cast<int64_t>(nkb) * BK + kChunkK - 1) / kChunkK);
  const int ckb = (nkb + nch - 1) / nch;
  const int npairs = (S + 1) / 2;   // weights 2 .. S+1 in pairs
  const int npass = npairs * nch;
  const int64_t i0 = static_cast<int64_t>(raster_tile(true)) * BM;
  const int64_t j0 = static_cast<int64_t>(raster_tile(false)) * BN;

  if (warp == 0) {
    if (lane == 0) {
      // producer: (pass, slice step, k block) in the MMA warp's order
      uint32_t it = 0;
      bool ok = true;
      for (int p = 0; ok && p < npass; ++p) {
        const int wlo = 2 + 2 * (p / nch);
        const bool hi = wlo + 1 <= S + 1;
        const int kb0 = (p % nch) * ckb;
        const int kb1 = (kb0 + ckb < nkb) ? kb0 + ckb : nkb;
        const int smax = hi ? wlo : wlo - 1;
        for (int sl = 1; ok && sl <= smax; ++sl) {
          const bool extra = sl == wlo;          // A_w * B_1, weight w+1 only
          const bool wide = hi && !extra;        // A_s * [B_(w-s); B_(w+1-s)]
          const int tlo = extra ? 1 : wlo - sl;
          for (int kb = kb0; kb < kb1; ++kb, ++it) {
            const int st = static_cast<int>(it % kPStages);
            const uint32_t ph = (it / kPStages) & 1u;
            if (!mbar_wait(empty + st, ph ^ 1u, abort_flag, g.limit_ns)) {
              ok = false;
              break;
            }
            unsigned char* a = ring + st * kPStageBytes;
            mbar_arrive_expect_tx(full + st, wide ? 3 * kTileBytes : 2 * kTileBytes);
            tma_load_2d(a, &tmA, full + st, kb * BK, static_cast<int>((sl - 1) * g.Mp + i0));
            tma_load_2d(a + kTileBytes, &tmB, full + st, kb * BK,
                        static_cast<int>((tlo - 1) * g.Np + j0));
            if (wide)
              tma_load_2d(a + 2 * kTileBytes, &tmB, full + st, kb * BK,
                          static_cast<int>((tlo) * g.Np + j0));  // B_(w+1-s) = B_(tlo+1)
          }
        }
      }
      if (!ok) {
        const uint32_t first = it > static_cast<uint32_t>(kPStages) ? it - kPStages : 0u;
        for (uint32_t j = first; j < it; ++j)
          mbar_wait_drain(full + (j % kPStages), (j / kPStages) & 1u, g.limit_ns);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int p = 0; ok && p < npass; ++p) {
        const int wlo = 2 + 2 * (p / nch);
        const bool hi = wlo + 1 <= S + 1;
        const int kb0 = (p % nch) * ckb;
        const int kb1 = (kb0 + ckb < nkb) ? kb0 + ckb : nkb;
        const int smax = hi ? wlo : wlo - 1;
        if (!mbar_wait(acc_empty, (static_cast<uint32_t>(p) & 1u) ^ 1u, abort_flag, g.limit_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        uint32_t accumulate = 0u;
        for (int sl = 1; ok && sl <= smax; ++sl) {
          const bool extra = sl == wlo;
          const bool wide = hi && !extra;
          for (int kb = kb0; kb < kb1; ++kb, ++it) {
            const int st = static_cast<int>(it % kPStages);
            if (!mbar_wait(full + st, (it / kPStages) & 1u, abort_flag, g.limit_ns)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a_addr = smem_u32(ring + st * kPStageBytes);
            const uint64_t ad = sw128_desc(a_addr), bd = sw128_desc(a_addr + kTileBytes);
#pragma unroll
            for (int kk = 0; kk < kRowBytes / 32; ++kk) {
              // advance 32 bytes along K inside the swizzle atom
              if (wide) {
                umma_n<F8, 256>(tmem, ad + 2u * kk, bd + 2u * kk, accumulate);
                accumulate = 1u;
              } else if (extra) {
                umma_n<F8, 128>(tmem + 128u, ad + 2u * kk, bd + 2u * kk, 1u);
              } else {
                umma_n<F8, 128>(tmem, ad + 2u * kk, bd + 2u * kk, accumulate);
                accumulate = 1u;
              }
            }
            umma_commit(empty + st);
          }
        }
        if (ok) umma_commit(acc_full);
      }
      umma_commit(mma_done);
      mbar_wait_drain(mma_done, 0u, g.limit_ns);
    }
  } else {
    // epilogue warps 2..9: TMEM lane quadrant q = warp % 4, columns
    // [64 h, 64 h + 64) of each weight of the pair
    const int q = warp & 3, h = (warp - 2) >> 2;
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;
    const uint32_t col0 = static_cast<uint32_t>(64 * h);
    bool ok = true;
    for (int p = 0; p < npass; ++p) {
      const int wlo = 2 + 2 * (p / nch);
      const bool hi = wlo + 1 <= S + 1;
      if (!mbar_wait(acc_full, static_cast<uint32_t>(p) & 1u, abort_flag, g.limit_ns)) {
        ok = false;
        break;
      }
      tc_fence_after();
      uint32_t flo[64], fhi[64];
#pragma unroll
      for (int c = 0; c < 64; c += 16) {
        tmem_ld16(tmem + lane_base + col0 + c, *reinterpret_cast<uint32_t(*)[16]>(flo + c));
        tmem_ld16(tmem + lane_base + 128u + col0 + c,
                  *reinterpret_cast<uint32_t(*)[16]>(fhi + c));
      }
      // wait for the loads, tied to every loaded register (no use of them is
      // scheduled before the wait)
      tmem_ld_wait(*reinterpret_cast<uint32_t(*)[16]>(flo));
#pragma unroll
      for (int c = 16; c < 64; c += 16) tmem_keep(*reinterpret_cast<uint32_t(*)[16]>(flo + c));
#pragma unroll
      for (int c = 0; c < 64; c += 16) tmem_keep(*reinterpret_cast<uint32_t(*)[16]>(fhi + c));
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);  // the MMA warp may start the next pair
      const double slo = scalbn(1.0, -kSliceBits * wlo);
      const double shi = scalbn(1.0, -kSliceBits * (wlo + 1));
#pragma unroll
      for (int c = 0; c < 64; c += 8) {
        uint32_t d[16];
        if (p > 0) {
          tmem_ld16(tmem + lane_base + kPAcc64Col + 2u * (col0 + c), d);
          tmem_ld_wait(d);
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e) d[e] = 0u;
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          double v = pair_to_double(d[2 * e], d[2 * e + 1]);
          v = fma(static_cast<double>(__uint_as_float(flo[c + e])), slo, v);
          if (hi) v = fma(static_cast<double>(__uint_as_float(fhi[c + e])), shi, v);
          d[2 * e] = static_cast<uint32_t>(__double2loint(v));
          d[2 * e + 1] = static_cast<uint32_t>(__double2hiint(v));
        }
        tmem_st16(tmem + lane_base + kPAcc64Col + 2u * (col0 + c), d);
      }
      tmem_st_wait();
    }
    if (ok) {
      // C = alpha * 2^(Ea+Eb) * acc64 + beta * C
      const int64_t i = i0 + 32 * q + lane;
      const bool row_ok = i < g.M;
      const int ea = row_ok ? g.Ea[i] : 0;
      for (int c = 0; c < 64; c += 8) {
        uint32_t d[16];
        tmem_ld16(tmem + lane_base + kPAcc64Col + 2u * (col0 + c), d);
        tmem_ld_wait(d);
        if (row_ok) {
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const int64_t j = j0 + col0 + c + e;
            if (j < g.N) {
              const double ab = scalbn(pair_to_double(d[2 * e], d[2 * e + 1]), ea + g.Eb[j]);
              double* ptr = g.C + i * g.N + j;
              *ptr = (g.beta == 0.0) ? g.alpha * ab : g.alpha * ab + g.beta * (*ptr);
            }
          }
        }
      }
    }
    tc_fence_before();
  }
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(g.error, 1u);
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2-D view [rows][Kp] of the slices (bf16 or e4m3 bytes) with a box of
// 128 bytes of K x 128 rows and 128-byte swizzle.
bool encode_slices(CUtensorMap* map, const void* base, int64_t rows, int64_t Kp, bool f8) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t esize = f8 ? 1u : 2u;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(Kp), static_cast<cuuint64_t>(rows)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(Kp) * esize};
  cuuint32_t box[2] = {static_cast<cuuint32_t>(kRowBytes / esize), static_cast<cuuint32_t>(BM)};
  cuuint32_t estr[2] = {1u, 1u};
  return fn(map, f8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
            const_cast<void*>(base), dims, strides,
            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc

// Engines (tune->algo): 0 the default (4), 1 mma.sync, 2 tcgen05 with bf16
// slices, 3 tcgen05 with e4m3 slices, 4 the same with paired digit weights.
enum Engine {
  kEngineDefault = 0, kEngineMmaSync = 1, kEngineTcBf16 = 2, kEngineTcE4m3 = 3,
  kEngineTcE4m3Paired = 4
};

int engine_of(const b200_tune* t) {
  const int e = (t && t->algo) ? t->algo : kEngineDefault;
  return e == kEngineDefault ? kEngineTcE4m3Paired : e;
}

struct SplitLayout {
  int64_t Mp, Np, Kp;
  int esize;  // bytes per stored digit
  size_t off_err, off_ea, off_eb, off_bmax, off_as, off_bt, total;
};

// The slice arrays' K is padded to one 128-byte TMA row (64 bf16 or 128 e4m3).
SplitLayout split_layout(int64_t m, int64_t n, int64_t k, int S, int engine) {
  SplitLayout L;
  const bool f8 = engine == kEngineTcE4m3 || engine == kEngineTcE4m3Paired;
  L.esize = f8 ? 1 : 2;
  L.Mp = round_up(m > 0 ? m : 1, TM);
  L.Np = round_up(n > 0 ? n : 1, TN);
  L.Kp = round_up(k > 0 ? k : 1, f8 ? 128 : kPadK);
  L.off_err = 16;  // the error word, at the same offset as in the scan workspaces
  L.off_ea = 256;
  L.off_eb = L.off_ea + round_up(L.Mp * 4, 256);
  L.off_bmax = L.off_eb + round_up(L.Np * 4, 256);
  L.off_as = L.off_bmax + round_up(L.Np * 8, 256);
  L.off_bt = L.off_as + round_up(static_cast<int64_t>(S) * L.Mp * L.Kp * L.esize, 256);
  L.total = L.off_bt + round_up(static_cast<int64_t>(S) * L.Np * L.Kp * L.esize, 256);
  return L;
}

int slices_of(const b200_tune* t) {
  return (t && t->items) ? t->items : kDefaultSlices;
}

template <typename T>
int launch_slicing(const double* A, const double* B, int64_t m, int64_t n, int64_t k,
                   const SplitLayout& L, int S, char* w, cudaStream_t st) {
  int* Ea = reinterpret_cast<int*>(w + L.off_ea);
  int* Eb = reinterpret_cast<int*>(w + L.off_eb);
  auto* bmax = reinterpret_cast<unsigned long long*>(w + L.off_bmax);
  const cudaError_t e = cudaMemsetAsync(bmax, 0, static_cast<size_t>(L.Np) * 8, st);
  if (e != cudaSuccess) {
    set_error("b200_gemm_split: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  constexpr int kPer = 16 / static_cast<int>(sizeof(T));
  row_scale_kernel<<<static_cast<unsigned>(ceil_div(m, 8)), 256, 0, st>>>(A, m, k, Ea);
  col_max_kernel<<<dim3(static_cast<unsigned>(ceil_div(n, 32)),
                        static_cast<unsigned>(k > 0 ? ceil_div(k, kColRows) : 1)),
                   dim3(32, 8), 0, st>>>(B, k, n, bmax);
  slice_a_kernel<T><<<dim3(static_cast<unsigned>(ceil_div(L.Kp, 128 * kPer)),
                           static_cast<unsigned>(L.Mp)),
                      128, 0, st>>>(A, m, k, Ea, S, L.Mp, L.Kp,
                                    reinterpret_cast<T*>(w + L.off_as));
  slice_b_kernel<T><<<dim3(static_cast<unsigned>(L.Np / kBtJ), static_cast<unsigned>(L.Kp / kBtK)),
                      256, 0, st>>>(B, k, n, bmax, Eb, S, L.Np, L.Kp,
                                    reinterpret_cast<T*>(w + L.off_bt));
  return B200_OK;
}

}  // namespace

extern "C" {

size_t b200_gemm_split_workspace_bytes(int64_t m, int64_t n, int64_t k, const b200_tune* tune) {
  return split_layout(m, n, k, slices_of(tune), engine_of(tune)).total;
}

int b200_gemm_split(const double* A, const double* B, double* C, int64_t m, int64_t n,
                    int64_t k, double alpha, double beta, void* workspace,
                    size_t workspace_bytes, const b200_tune* tune, b200_stream_t stream) {
  if (!A || !B || !C || m < 0 || n < 0 || k < 0) return invalid("b200_gemm_split: bad args");
  const int S = slices_of(tune);
  if (S < 2 || S > kMaxSlices) return invalid("b200_gemm_split: slices %d not in [2, %d]", S, kMaxSlices);
  const int engine = engine_of(tune);
  if (engine < kEngineMmaSync || engine > kEngineTcE4m3Paired)
    return invalid("b200_gemm_split: engine %d (0 to 4)", engine);
  if (k > kMaxK)
    return invalid("b200_gemm_split: k = %lld exceeds %lld", static_cast<long long>(k),
                   static_cast<long long>(kMaxK));
  if (m == 0 || n == 0) return B200_OK;
  const SplitLayout L = split_layout(m, n, k, S, engine);
  if (!workspace || workspace_bytes < L.total) {
    set_error("b200_gemm_split: workspace %zu bytes, need %zu", workspace_bytes, L.total);
    return B200_ERR_WORKSPACE;
  }
  if (L.Mp > 65535) return invalid("b200_gemm_split: m too large");
  if (engine != kEngineMmaSync && device_info().cc_major < 10)
    return unsupported("b200_gemm_split: the tcgen05 engines need compute capability 10.x");
  char* w = static_cast<char*>(workspace);
  unsigned int* err = reinterpret_cast<unsigned int*>(w + L.off_err);
  int* Ea = reinterpret_cast<int*>(w + L.off_ea);
  int* Eb = reinterpret_cast<int*>(w + L.off_eb);
  cudaStream_t st = as_stream(stream);
  const bool f8 = engine == kEngineTcE4m3 || engine == kEngineTcE4m3Paired;
  // zero-sized k: C = beta*C through the same epilogue (all digits zero)
  const int rc = f8 ? launch_slicing<uint8_t>(A, B, m, n, k, L, S, w, st)
                    : launch_slicing<__nv_bfloat16>(A, B, m, n, k, L, S, w, st);
  if (rc != B200_OK) return rc;
  if (engine == kEngineMmaSync) {
    SplitArgs g{reinterpret_cast<const __nv_bfloat16*>(w + L.off_as),
                reinterpret_cast<const __nv_bfloat16*>(w + L.off_bt),
                Ea, Eb, C, m, n, L.Mp, L.Np, L.Kp, alpha, beta, S};
    ozaki_mma_kernel<<<dim3(static_cast<unsigned>(L.Np / TN), static_cast<unsigned>(L.Mp / TM)),
                       256, 0, st>>>(g);
    return after_launch("b200_gemm_split", 5);
  }
  CUtensorMap tmA, tmB;
  if (!tc::encode_slices(&tmA, w + L.off_as, S * L.Mp, L.Kp, f8) ||
      !tc::encode_slices(&tmB, w + L.off_bt, S * L.Np, L.Kp, f8))
    return unsupported("b200_gemm_split: cuTensorMapEncodeTiled unavailable or rejected the slices");
  const bool paired = engine == kEngineTcE4m3Paired;
  const void* kern = paired ? reinterpret_cast<const void*>(tc::ozaki_tc_paired_kernel<true>)
                     : f8   ? reinterpret_cast<const void*>(tc::ozaki_tc_kernel<true>)
                            : reinterpret_cast<const void*>(tc::ozaki_tc_kernel<false>);
  const size_t smem = paired ? tc::kPSmemBytes : tc::kSmemBytes;
  const int attr = allow_dynamic_smem(kern, smem, "b200_gemm_split");
  if (attr != B200_OK) return attr;
  tc::TcArgs g{Ea, Eb, C, err, m, n, L.Mp, L.Np, L.Kp, alpha, beta, S,
               wait_limit_ns(tune, tc::kWaitLimitNs)};
  const dim3 grid(static_cast<unsigned>(L.Np / tc::BN), static_cast<unsigned>(L.Mp / tc::BM));
  if (paired)
    tc::ozaki_tc_paired_kernel<true><<<grid, tc::kPThreads, smem, st>>>(tmA, tmB, g);
  else if (f8)
    tc::ozaki_tc_kernel<true><<<grid, tc::kThreads, smem, st>>>(tmA, tmB, g);
  else
    tc::ozaki_tc_kernel<false><<<grid, tc::kThreads, smem, st>>>(tmA, tmB, g);
  return after_launch("b200_gemm_split", 5);
}

}  // extern "C"
