// Stream_DOT with library-owned scratch: b200_stream_dot_static.
//
// Some callers cannot allocate device memory at the point where they need a
// dot product: code running under a memory manager that owns the whole device
// heap (a framework's caching allocator or a fixed arena handed out at
// start-up), and latency-critical loops where cudaMalloc's implicit device
// synchronisation is not acceptable.  For them this entry point keeps the
// reduction scratch (per-CTA partials and the arrival counter) in a
// file-scope __device__ array that every GPU loading the library holds until
// the process exits, so a call allocates nothing.
//
// The array is sized for kStaticMaxCtas CTAs; a launch shape needing more is
// rejected.  Every call shares the array: calls that overlap on the GPU (on
// different streams, or from different host threads) race on it and must be
// ordered by the caller.  The counter is cleared by each call before its
// kernel (cudaMemsetAsync, stream-ordered), so a call never depends on what
// an earlier call left behind.
//
// The device address of the array is looked up once per device with
// cudaGetSymbolAddress, on the first call made while that device is current.
// That first call on a device should therefore come before any stream
// capture that contains the entry point.
#include "b200_internal.cuh"
#include "b200_reduce.cuh"

#include <mutex>
#include <vector>

using namespace b200;

constexpr int kStaticMaxCtas = 4096;
constexpr size_t kStaticScratchBytes = 256 + static_cast<size_t>(kStaticMaxCtas) * 16;

// Scratch layout as b200_stream_dot's workspace: [counter (256 B)] [partials].
// In host code this name is only a stand-in for the symbol, never a device
// address: the address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_dot_scratch[kStaticScratchBytes];

namespace {

std::mutex g_scratch_mu;
std::vector<void*> g_scratch_ptr;  // per device; nullptr = not looked up yet

// Device address of g_dot_scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("b200_stream_dot_static: cudaGetDevice: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (static_cast<int>(g_scratch_ptr.size()) <= dev) g_scratch_ptr.resize(dev + 1, nullptr);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_dot_scratch);
    if (e != cudaSuccess || !p) {
      set_error("b200_stream_dot_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return B200_ERR_LAUNCH;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return B200_OK;
}

template <int BS, int IT>
__global__ void __launch_bounds__(BS)
dot_static_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                  double dot_init, double* __restrict__ accum,
                  double* __restrict__ partials, unsigned int* __restrict__ counter) {
  __shared__ double smem[BS / 32];
  __shared__ bool last_flag;
  double s = 0.0;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < n;
       t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
    double ra[IT], rb[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t i = t0 + u * BS + threadIdx.x;
      ra[u] = (i < n) ? __ldg(a + i) : 0.0;
      rb[u] = (i < n) ? __ldg(b + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) s += ra[u] * rb[u];
  }
  s = block_sum<BS>(s, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  if (arrive_last(counter, &last_flag)) {
    double t = 0.0;
    for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += BS)
      t += __ldcg(partials + i);
    t = block_sum<BS>(t, smem);
    if (threadIdx.x == 0) {
      *accum += dot_init + t;
      *counter = 0u;
    }
  }
}

}  // namespace

extern "C" {

size_t b200_stream_dot_static_max_scratch_bytes(void) { return kStaticScratchBytes; }

int b200_stream_dot_static(const double* a, const double* b, int64_t n, double dot_init,
                           double* dot_accum, const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!a || !b)) || !dot_accum)
    return invalid("b200_stream_dot_static: bad args");
  int block = (tune && tune->block_size) ? tune->block_size : 256;
  int items = (tune && tune->items) ? tune->items : 4;
  if (!valid_block(block))
    return invalid("b200_stream_dot_static: bad block size %d", block);
  int grid = reduce_grid(n, tune, block, items);
  if (grid > kStaticMaxCtas) {
    set_error("b200_stream_dot_static: launch shape needs %d CTAs of scratch, the static "
              "scratch holds %d (%zu bytes)", grid, kStaticMaxCtas, kStaticScratchBytes);
    return B200_ERR_WORKSPACE;
  }
  void* base = nullptr;
  int st = scratch_address(&base);
  if (st != B200_OK) return st;
  unsigned int* counter = static_cast<unsigned int*>(base);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(base) + 256);
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) {
    set_error("b200_stream_dot_static: clearing the counter: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  B200_DISPATCH_BLOCK(block, BS, B200_DISPATCH_ITEMS(items, IT,
    dot_static_kernel<BS, IT><<<grid, BS, 0, s>>>(a, b, n, dot_init, dot_accum, partials,
                                                  counter)));
  return after_launch("b200_stream_dot_static");
}

}  // extern "C"
