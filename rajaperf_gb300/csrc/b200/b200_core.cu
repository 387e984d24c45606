// libb200 core: error state, launch accounting, device properties, tuning
// resolution and the data-initialisation kernels.
#include "b200_f64emu.cuh"
#include "b200_internal.cuh"

#include <map>
#include <mutex>
#include <utility>
#include <vector>

namespace b200 {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};
static std::mutex g_info_mu;
static std::vector<DeviceInfo> g_info;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

int invalid(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return B200_ERR_INVALID_ARG;
}

int unsupported(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return B200_ERR_UNSUPPORTED;
}

int after_launch(const char* what, int nlaunches) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: launch failed: %s", what, cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  g_launches.fetch_add(nlaunches, std::memory_order_relaxed);
  return B200_OK;
}

const DeviceInfo& device_info() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_info_mu);
  if (static_cast<int>(g_info.size()) <= dev) g_info.resize(dev + 1);
  DeviceInfo& d = g_info[dev];
  if (d.device != dev) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) == cudaSuccess) {
      d.sm_count = p.multiProcessorCount;
      d.cc_major = p.major;
      d.cc_minor = p.minor;
      d.global_mem = p.totalGlobalMem;
      d.l2_bytes = p.l2CacheSize;
      d.max_smem_optin = static_cast<int>(p.sharedMemPerBlockOptin);
    } else {
      cudaGetLastError();
      d.sm_count = 152;
    }
    d.device = dev;
  }
  return d;
}

int allow_dynamic_smem(const void* kernel, size_t bytes, const char* what) {
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> granted;  // (kernel, device) -> bytes
  std::lock_guard<std::mutex> lk(mu);
  size_t& have = granted[{kernel, dev}];
  if (bytes <= have) return B200_OK;
  const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(bytes));
  if (e != cudaSuccess) {
    set_error("%s: shared memory attribute (%zu bytes): %s", what, bytes, cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  have = bytes;
  return B200_OK;
}

Shape resolve_1d(const b200_tune* t, int64_t units, int def_block,
                 int def_items, int def_vec, int64_t max_grid) {
  Shape s;
  s.block = (t && t->block_size) ? t->block_size : def_block;
  s.items = (t && t->items) ? t->items : def_items;
  s.vec = (t && t->vec) ? t->vec : def_vec;
  int64_t cap = (t && t->grid_blocks) ? t->grid_blocks : max_grid;
  int64_t tiles = ceil_div(units > 0 ? units : 1,
                           static_cast<int64_t>(s.block) * s.items);
  if (cap > 0 && tiles > cap) tiles = cap;
  if (tiles > 0x7fffffffLL) tiles = 0x7fffffffLL;
  s.grid = static_cast<int>(tiles < 1 ? 1 : tiles);
  return s;
}

}  // namespace b200

using b200::g_last_error;
using b200::g_launches;
using b200::invalid;
using b200::set_error;
using b200::after_launch;
using b200::as_stream;
using b200::device_info;
using b200::ceil_div;
using b200::DeviceInfo;

// ---- initialisation kernels -------------------------------------------------

namespace {

__global__ void init_reference_kernel(double* __restrict__ p, int64_t n,
                                      double factor) {
  int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n; i += stride) {
    // Same operation order as the host formula; __dmul_rn/__ddiv_rn keep the
    // compiler from contracting it, so the values are bit-identical.
    double di = static_cast<double>(i);
    p[i] = __ddiv_rn(__dmul_rn(factor, __dadd_rn(di, 1.1)),
                     __dadd_rn(di, 1.12345));
  }
}

__global__ void init_reference_signed_kernel(double* __restrict__ p,
                                             const int8_t* __restrict__ sign,
                                             int64_t n, double factor) {
  int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n; i += stride) {
    double di = static_cast<double>(i);
    double s = sign[i] < 0 ? -1.0 : 1.0;
    p[i] = __ddiv_rn(__dmul_rn(__dmul_rn(s, factor), __dadd_rn(di, 1.1)),
                     __dadd_rn(di, 1.12345));
  }
}

template <typename T>
__global__ void init_const_kernel(T* __restrict__ p, int64_t n, T v) {
  int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n; i += stride) {
    p[i] = v;
  }
}

// splitmix64 finaliser over (seed, stream, index): a counter-based generator,
// so any element can be produced independently on the host or the device.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

__device__ inline uint64_t counter_bits(uint64_t seed, uint64_t stream,
                                        uint64_t i) {
  uint64_t key = mix64(seed + 0x9e3779b97f4a7c15ULL * (stream + 1));
  return mix64(key + 0x9e3779b97f4a7c15ULL * (i + 1));
}

__global__ void init_uniform_kernel(double* __restrict__ p, int64_t n,
                                    uint64_t seed, uint64_t stream, double lo,
                                    double width) {
  int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n; i += stride) {
    double u = static_cast<double>(counter_bits(seed, stream, i) >> 11) *
               0x1.0p-53;
    p[i] = __dadd_rn(lo, __dmul_rn(width, u));
  }
}

__global__ void init_uniform_i64_kernel(int64_t* __restrict__ p, int64_t n,
                                        uint64_t seed, uint64_t stream,
                                        int64_t lo, uint64_t range) {
  int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n; i += stride) {
    p[i] = lo + static_cast<int64_t>(counter_bits(seed, stream, i) % range);
  }
}

int init_grid(int64_t n) {
  int64_t g = ceil_div(n, 256);
  int64_t cap = static_cast<int64_t>(device_info().sm_count) * 16;
  if (g > cap) g = cap;
  return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

extern "C" {

const char* b200_last_error_string(void) { return g_last_error.c_str(); }

int b200_device_caps(b200_caps* out) {
  if (!out) return invalid("b200_device_caps: null output");
  const DeviceInfo& d = device_info();
  out->device = d.device;
  out->sm_count = d.sm_count;
  out->cc_major = d.cc_major;
  out->cc_minor = d.cc_minor;
  out->global_mem_bytes = static_cast<int64_t>(d.global_mem);
  out->l2_bytes = d.l2_bytes;
  out->max_smem_per_block_optin = d.max_smem_optin;
  out->reserved = 0;
  return B200_OK;
}

int64_t b200_launch_count(void) { return g_launches.load(); }

int b200_workspace_status(void* workspace, size_t workspace_bytes, b200_stream_t stream) {
  // the error word sits at byte 16 of the 256-byte header of every
  // workspace whose kernels wait (scan, index list, split GEMM)
  if (!workspace || workspace_bytes < 256)
    return invalid("b200_workspace_status: workspace of %zu bytes (needs its 256-byte header)",
                   workspace_bytes);
  cudaStream_t st = as_stream(stream);
  unsigned int word = 0;
  cudaError_t e = cudaMemcpyAsync(&word, static_cast<char*>(workspace) + 16, sizeof(word),
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("b200_workspace_status: reading the error word: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  if (word == 0u) return B200_OK;
  // a wait gave up: the tile tickets and statuses may be mid-launch, so the
  // whole workspace starts over from zero
  e = cudaMemsetAsync(workspace, 0, workspace_bytes, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("b200_workspace_status: clearing the workspace: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  set_error("a bounded device-side wait gave up (error word %u): the results of the calls "
            "on this workspace since its last check are invalid; the workspace was cleared",
            word);
  return B200_ERR_TIMEOUT;
}

int b200_init_reference(double* p, int64_t n, double factor,
                        b200_stream_t stream) {
  if (n < 0 || (n > 0 && !p)) return invalid("b200_init_reference: bad args");
  if (n == 0) return B200_OK;
  init_reference_kernel<<<init_grid(n), 256, 0, as_stream(stream)>>>(p, n,
                                                                     factor);
  return after_launch("b200_init_reference");
}

int b200_init_reference_signed(double* p, const int8_t* sign, int64_t n,
                               double factor, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!p || !sign)))
    return invalid("b200_init_reference_signed: bad args");
  if (n == 0) return B200_OK;
  init_reference_signed_kernel<<<init_grid(n), 256, 0, as_stream(stream)>>>(
      p, sign, n, factor);
  return after_launch("b200_init_reference_signed");
}

int b200_init_const(double* p, int64_t n, double value,
                    b200_stream_t stream) {
  if (n < 0 || (n > 0 && !p)) return invalid("b200_init_const: bad args");
  if (n == 0) return B200_OK;
  init_const_kernel<double><<<init_grid(n), 256, 0, as_stream(stream)>>>(
      p, n, value);
  return after_launch("b200_init_const");
}

int b200_init_const_i64(int64_t* p, int64_t n, int64_t value,
                        b200_stream_t stream) {
  if (n < 0 || (n > 0 && !p)) return invalid("b200_init_const_i64: bad args");
  if (n == 0) return B200_OK;
  init_const_kernel<int64_t><<<init_grid(n), 256, 0, as_stream(stream)>>>(
      p, n, value);
  return after_launch("b200_init_const_i64");
}

int b200_init_uniform(double* p, int64_t n, uint64_t seed, uint64_t stream_id,
                      double lo, double hi, b200_stream_t stream) {
  if (n < 0 || (n > 0 && !p) || !(hi >= lo))
    return invalid("b200_init_uniform: bad args");
  if (n == 0) return B200_OK;
  init_uniform_kernel<<<init_grid(n), 256, 0, as_stream(stream)>>>(
      p, n, seed, stream_id, lo, hi - lo);
  return after_launch("b200_init_uniform");
}

int b200_init_uniform_i64(int64_t* p, int64_t n, uint64_t seed,
                          uint64_t stream_id, int64_t lo, int64_t hi,
                          b200_stream_t stream) {
  if (n < 0 || (n > 0 && !p) || hi <= lo)
    return invalid("b200_init_uniform_i64: bad args");
  if (n == 0) return B200_OK;
  init_uniform_i64_kernel<<<init_grid(n), 256, 0, as_stream(stream)>>>(
      p, n, seed, stream_id, lo, static_cast<uint64_t>(hi - lo));
  return after_launch("b200_init_uniform_i64");
}

}  // extern "C"

// ---- FP64 pipe probe ----------------------------------------------------------

namespace {

// Sixteen independent FMA chains per thread (enough to cover the pipe's
// latency at full occupancy); out[] receives one value per thread so the
// chains are live.  `out` must hold probe_threads() doubles.
// a and b are copied into per-thread registers (through threadIdx.x and an
// argument that is zero at run time): a DFMA with a kernel-argument operand
// (constant bank or uniform register) issues at 5/6 of the rate of one whose
// operands are all per-thread registers (501 vs 595 G/s measured), and the
// probe is meant to find the pipe's full rate.
__global__ void __launch_bounds__(256) dfma_probe_kernel(double* out, double a, double b,
                                                         int iters, int zero) {
  const unsigned long long z = threadIdx.x & static_cast<unsigned>(zero);
  const double ar = __longlong_as_double(static_cast<long long>(
      static_cast<unsigned long long>(__double_as_longlong(a)) + z));
  const double br = __longlong_as_double(static_cast<long long>(
      static_cast<unsigned long long>(__double_as_longlong(b)) + z));
  double x[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 16; ++c) x[c] = fma(x[c], ar, br);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 16; ++c) s += x[c];
  out[static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

int64_t b200_probe_dfma_threads(void) {
  return static_cast<int64_t>(device_info().sm_count) * 8 * 256;
}

int b200_probe_dfma(double* out, int32_t iters, int64_t* fma_count, b200_stream_t stream) {
  if (!out || iters <= 0 || !fma_count) return invalid("b200_probe_dfma: bad args");
  int blocks = device_info().sm_count * 8;
  dfma_probe_kernel<<<blocks, 256, 0, as_stream(stream)>>>(out, 0.999999, 1e-7, iters, 0);
  *fma_count = static_cast<int64_t>(blocks) * 256 * 16 * iters;
  return after_launch("b200_probe_dfma");
}

}  // extern "C"

// ---- integer-pipe FP64 self-test ------------------------------------------------

namespace {

__device__ __forceinline__ uint64_t rnd64(uint64_t seed, uint64_t i) {
  return mix64(mix64(seed + 0x9e3779b97f4a7c15ULL * (i + 1)) ^ 0x5bd1e995ULL);
}

// Operand pairs from five families: arbitrary bit patterns (every class,
// NaNs and infinities included), nearby exponents (cancellation), exponents
// far apart (sticky), values near the overflow / underflow edges, and
// uniform [0.5, 1.5).  Counts results whose bits differ from the FP64 pipe's
// (two NaNs count as equal).
__global__ void f64emu_check_kernel(int64_t n, uint64_t seed, int op,
                                    unsigned long long* mismatches) {
  unsigned long long bad = 0;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    uint64_t ra = rnd64(seed, 2 * i), rb = rnd64(seed, 2 * i + 1);
    uint64_t A = ra, B = rb, C = 0;  // C: op 12's addend
    switch (i % 5) {
      case 0: break;
      case 1: {  // exponents within 2 of each other
        const uint64_t e = ((ra >> 12) % 2000u) + 20u;
        A = (ra & 0x800FFFFFFFFFFFFFULL) | (e << 52);
        B = (rb & 0x800FFFFFFFFFFFFFULL) | ((e + (rb >> 60) % 3u - 1u) << 52);
        break;
      }
      case 2: {  // exponents up to 70 apart
        const uint64_t e = ((ra >> 12) % 1800u) + 100u;
        A = (ra & 0x800FFFFFFFFFFFFFULL) | (e << 52);
        B = (rb & 0x800FFFFFFFFFFFFFULL) | ((e - (rb >> 56) % 71u) << 52);
        break;
      }
      case 3: {  // near the ends of the exponent range
        const uint64_t e1 = (ra >> 60) & 1u ? 2046u - (ra >> 56) % 8u : 1u + (ra >> 56) % 8u;
        const uint64_t e2 = (rb >> 60) & 1u ? 1023u + (rb >> 56) % 8u : 1023u - (rb >> 56) % 8u;
        A = (ra & 0x800FFFFFFFFFFFFFULL) | (e1 << 52);
        B = (rb & 0x800FFFFFFFFFFFFFULL) | (e2 << 52);
        break;
      }
      default: {
        A = __double_as_longlong(0.5 + static_cast<double>(ra >> 11) * 0x1.0p-53);
        B = __double_as_longlong(0.5 + static_cast<double>(rb >> 11) * 0x1.0p-53);
        break;
      }
    }
    if ((op == 7 || op == 9) && (i % 7) == 6) {  // signed zeros, infinities, NaNs
      const uint64_t sp[6] = {0x0ULL, 0x8000000000000000ULL, 0x7FF0000000000000ULL,
                              0xFFF0000000000000ULL, 0x7FF8000000000001ULL,
                              0xFFF8000000000000ULL};
      A = sp[(ra >> 60) % 6u];
      if ((rb >> 61) & 1u) B = sp[(rb >> 56) % 6u];
    }
    if (op == 6) {  // division: three more families that stress rounding
      const uint64_t bb = (rb & 0x800FFFFFFFFFFFFFULL) | ((((rb >> 52) & 0x7ffu) % 1500u + 270u) << 52);
      switch ((i >> 3) % 4) {
        case 1: {  // quotients next to a rounding midpoint: a = RN(b * (1 + odd * 2^-53))
          const double mid = 1.0 + static_cast<double>((ra >> 12) | 1u) * 0x1.0p-53;
          B = bb;
          A = __double_as_longlong(__dmul_rn(__longlong_as_double(static_cast<long long>(B)), mid));
          break;
        }
        case 2: {  // quotients next to 1: a within a few ulps of b
          B = bb;
          A = B + static_cast<uint64_t>(static_cast<int64_t>((ra >> 60) % 9u) - 4);
          break;
        }
        case 3: {  // extreme divisor significands: 1.0 or 2 - ulp
          B = (bb & 0xFFF0000000000000ULL) | (((rb >> 20) & 1u) ? 0x000FFFFFFFFFFFFFULL : 0u);
          A = (ra & 0x800FFFFFFFFFFFFFULL) | ((((ra >> 52) & 0x7ffu) % 1500u + 270u) << 52);
          break;
        }
        default: break;
      }
    }
    if (op == 10) {  // close exponents (0-4 apart), either sign, near the top of the range
      const uint64_t e = ((i % 5) == 3) ? 2040u + (ra >> 58) % 7u : ((ra >> 12) % 2000u) + 20u;
      A = (ra & 0x800FFFFFFFFFFFFFULL) | (e << 52);
      B = (rb & 0x000FFFFFFFFFFFFFULL) | ((e - (rb >> 60) % 5u) << 52) |
          (((rb >> 59) & 7u) ? (A & 0x8000000000000000ULL) : (~A & 0x8000000000000000ULL));
      if ((i % 7) == 6) {  // zeros, subnormals, infinities, NaNs: the slow path
        const uint64_t sp[6] = {0x0ULL, 0x8000000000000000ULL, 0x7FF0000000000000ULL,
                                0x0000000000000001ULL, 0x7FF8000000000001ULL,
                                0x000FFFFFFFFFFFFFULL};
        A = sp[(ra >> 60) % 6u] | (A & 0x8000000000000000ULL);
      }
    }
    if (op == 11) {  // either sign, exponents 0-4 apart, cancellations of every depth
      const uint64_t e = ((i % 5) == 3)   ? 2040u + (ra >> 58) % 7u
                         : ((i % 5) == 4) ? 1u + (ra >> 12) % 60u  // results below the normal range
                                          : ((ra >> 12) % 2000u) + 20u;
      A = (ra & 0x800FFFFFFFFFFFFFULL) | (e << 52);
      const uint64_t r = (rb >> 60) % 5u;
      B = (rb & 0x000FFFFFFFFFFFFFULL) | ((e > r ? e - r : 0u) << 52) |
          (((rb >> 59) & 1u) ? (A & 0x8000000000000000ULL) : (~A & 0x8000000000000000ULL));
      if ((i % 3) == 1) {  // b = -(a +- delta): delta of 0 to 53 bits, exact zero included
        const uint64_t mag = A & ~0x8000000000000000ULL;
        const uint64_t delta = (rb >> 2) & ((1ULL << ((rb >> 56) % 54u)) - 1u);
        const uint64_t bm = (((rb >> 1) & 1u) || delta > mag) ? mag + delta : mag - delta;
        B = bm | (~A & 0x8000000000000000ULL);
      }
      if ((i % 7) == 6) {  // zeros, subnormals, infinities, NaNs: the slow path
        const uint64_t sp[6] = {0x0ULL, 0x8000000000000000ULL, 0x7FF0000000000000ULL,
                                0x0000000000000001ULL, 0x7FF8000000000001ULL,
                                0x000FFFFFFFFFFFFFULL};
        A = sp[(ra >> 60) % 6u] | (A & 0x8000000000000000ULL);
      }
    }
    if (op == 12) {  // a * b + c: positive, c a few binades above the product (EOS), the
                     // window edges, near-ties, the top and bottom of the range, specials
      const uint64_t ea = (i % 5) == 3 ? 1000u + (ra >> 58) % 40u : 900u + (ra >> 12) % 200u;
      const uint64_t eb = (i % 5) == 4 ? 2u + (rb >> 58) % 30u : 1000u + (rb >> 12) % 46u;
      A = (ra & 0x000FFFFFFFFFFFFFULL) | (ea << 52);
      B = (rb & 0x000FFFFFFFFFFFFFULL) | (eb << 52);
      // c's exponent from D = ec + 1075 - ea - eb in [-3, 78]: the window [0, 74] and past it
      const int64_t D = static_cast<int64_t>((ra >> 40) % 82u) - 3;
      int64_t ec = D + static_cast<int64_t>(ea + eb) - 1075;
      if ((i % 5) == 3) ec = 2040 + static_cast<int64_t>((rb >> 40) % 8u);  // the top of the range
      if (ec < 0) ec = 0;
      if (ec > 2047) ec = 2047;
      const uint64_t mc = (rb >> 5) & 0x000FFFFFFFFFFFFFULL;
      C = mc | (static_cast<uint64_t>(ec) << 52);
      if ((i % 3) == 1) {  // low bits of a and b cleared: exact products, sums near ties
        A &= ~0x3FFFFFFULL;
        B &= ~0x3FFFFFFULL;
      }
      if ((i % 7) == 6) {  // zeros, subnormals, negatives, infinities, NaNs: the slow path
        const uint64_t sp[6] = {0x0ULL, 0x8000000000000000ULL, 0x7FF0000000000000ULL,
                                0x0000000000000001ULL, 0x7FF8000000000001ULL,
                                0xBFF0000000000000ULL};
        if ((ra >> 61) & 1u) A = sp[(ra >> 58) % 6u]; else C = sp[(rb >> 58) % 6u];
      }
    }
    if (op == 9 && (i % 5) != 0 && (i % 5) != 3) {  // a + tiny b: gaps 50-60 around 55
      const uint64_t e = ((ra >> 12) % 1900u) + 70u;
      const uint64_t gap = 50u + (rb >> 58) % 11u;
      A = (ra & 0x800FFFFFFFFFFFFFULL) | (e << 52);
      if ((ra >> 11) & 1u) A &= 0xFFF0000000000000ULL;  // a power of two: the tighter side
      B = (rb & 0x800FFFFFFFFFFFFFULL) | ((e - gap) << 52);
      if ((rb >> 11) & 1u) B |= 0x000FFFFFFFFFFFFFULL;  // b at the top of its binade
    }
    const double a = __longlong_as_double(static_cast<long long>(A));
    const double b = __longlong_as_double(static_cast<long long>(B));
    double want, got;
    if (op == 0) { want = __dadd_rn(a, b); got = b200::f64emu::add(a, b); }
    else if (op == 1) { want = __dadd_rn(a, -b); got = b200::f64emu::sub(a, b); }
    else if (op == 2) { want = __dmul_rn(a, b); got = b200::f64emu::mul(a, b); }
    else if (op == 3) {
      want = __dmul_rn(a, 0.5);
      bool slow = false;
      got = b200::f64emu::mul_pow2_fast<-1>(a, slow);
      if (slow) got = __dmul_rn(a, 0.5);
    } else if (op == 4) {
      want = __dmul_rn(a, 0.125);
      bool slow = false;
      got = b200::f64emu::mul_pow2_fast<-3>(a, slow);
      if (slow) got = __dmul_rn(a, 0.125);
    } else if (op == 5) {
      want = __dmul_rn(a, 2.0);
      bool slow = false;
      got = b200::f64emu::mul_pow2_fast<1>(a, slow);
      if (slow) got = __dmul_rn(a, 2.0);
    } else if (op == 6) {
      want = __ddiv_rn(a, b);
      bool slow = false;
      got = b200::f64emu::div_fast(a, b, slow);
      if (slow) got = __ddiv_rn(a, b);
    } else if (op == 7) {  // x < 0 as INDEXLIST tests it
      want = a < 0.0 ? 1.0 : 0.0;
      got = b200::f64emu::lt_zero(a) ? 1.0 : 0.0;
    } else if (op == 10) {  // a + b, close exponents, as JACOBI_2D's integer-pipe adds
      want = __dadd_rn(a, b);
      bool slow = false;
      got = b200::f64emu::add_close_fast(a, b, slow);
      if (slow) got = __dadd_rn(a, b);
    } else if (op == 12) {  // a * b + c on the integer pipes, as EOS's FMAs
      const double c = __longlong_as_double(static_cast<long long>(C));
      want = __fma_rn(a, b, c);
      bool slow = false;
      got = b200::f64emu::fma_pos_fast(a, b, c, slow);
      if (slow) got = __fma_rn(a, b, c);
    } else if (op == 11) {  // a + b, either sign, close exponents, as HEAT_3D's b(+1) - 2a
      want = __dadd_rn(a, b);
      bool slow = false;
      got = b200::f64emu::add_near_fast(a, b, slow);
      if (slow) got = __dadd_rn(a, b);
    } else if (op == 9) {  // a + b for b below a's last bit, as DEL_DOT_VEC_2D's + ptiny
      want = __dadd_rn(a, b);
      bool slow = false;
      got = b200::f64emu::add_negligible(a, b, slow);
      if (slow) got = __dadd_rn(a, b);
    } else {  // a * b on the integer pipe; every other pair as JACOBI_2D's a * 0.2
      const double c = (i & 1) ? 0.2 : b;
      want = __dmul_rn(a, c);
      bool slow = false;
      got = b200::f64emu::mul_fast(a, c, slow);
      if (slow) got = __dmul_rn(a, c);
    }
    const bool same = (__double_as_longlong(want) == __double_as_longlong(got)) ||
                      (isnan(want) && isnan(got));
    if (!same) ++bad;
  }
  if (bad) atomicAdd(mismatches, bad);
}

}  // namespace

extern "C" int b200_f64emu_selftest(int64_t n, uint64_t seed, int32_t op,
                                    unsigned long long* mismatches, b200_stream_t stream) {
  if (n < 0 || !mismatches || op < 0 || op > 12) return invalid("b200_f64emu_selftest: bad args");
  const int blocks = device_info().sm_count * 8;
  f64emu_check_kernel<<<blocks, 256, 0, as_stream(stream)>>>(n, seed, op, mismatches);
  return after_launch("b200_f64emu_selftest");
}
