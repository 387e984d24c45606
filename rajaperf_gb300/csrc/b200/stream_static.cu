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
// The device address of the array is looked up with cudaGetSymbolAddress on
// the first call made in a CUDA context (the device's primary context, or
// any other context the caller makes current) and cached under that
// context's process-unique id (cuCtxGetId), so a call in a context created
// later -- after a cudaDeviceReset, or a second context on the same device --
// looks the address up again instead of reusing a stale one.  The first call
// in a context should therefore come before any stream capture that
// contains the entry point.
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

typedef int (*ctx_get_current_fn)(void** ctx);
typedef int (*ctx_get_id_fn)(void* ctx, unsigned long long* id);

struct ScratchEntry {
  unsigned long long ctx_id;
  void* ptr;
};

std::mutex g_scratch_mu;
std::vector<ScratchEntry> g_scratch;  // one entry per context seen

// Process-unique id of the current context (cuCtxGetId), found through the
// runtime's driver entry points so the library does not link libcuda.
int current_context_id(unsigned long long* id) {
  static ctx_get_current_fn get_current = nullptr;
  static ctx_get_id_fn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<ctx_get_current_fn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<ctx_get_id_fn>(p);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return B200_ERR_UNSUPPORTED;
  // With no context current, cudaSetDevice on the current device makes that
  // device's primary context current (it initialises it; it allocates no
  // device memory).
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaSetDevice(dev);
    if (e != cudaSuccess || get_current(&ctx) != 0 || !ctx) {
      cudaGetLastError();
      return B200_ERR_LAUNCH;
    }
  }
  return get_id(ctx, id) == 0 ? B200_OK : B200_ERR_LAUNCH;
}

// Device address of g_dot_scratch in the current context (looked up once
// per context).
int scratch_address(void** out) {
  unsigned long long id = 0;
  int st = current_context_id(&id);
  if (st != B200_OK) {
    set_error("b200_stream_dot_static: no current CUDA context (cuCtxGetCurrent/cuCtxGetId)");
    return st;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  for (const ScratchEntry& en : g_scratch) {
    if (en.ctx_id == id) {
      *out = en.ptr;
      return B200_OK;
    }
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_dot_scratch);
  if (e != cudaSuccess || !p) {
    // clear the error here so that the next entry point does not report it
    cudaGetLastError();
    set_error("b200_stream_dot_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  g_scratch.push_back({id, p});
  *out = p;
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
    cudaGetLastError();
    set_error("b200_stream_dot_static: clearing the counter: %s", cudaGetErrorString(e));
    return B200_ERR_LAUNCH;
  }
  B200_DISPATCH_BLOCK(block, BS, B200_DISPATCH_ITEMS(items, IT,
    dot_static_kernel<BS, IT><<<grid, BS, 0, s>>>(a, b, n, dot_init, dot_accum, partials,
                                                  counter)));
  return after_launch("b200_stream_dot_static");
}

}  // extern "C"
