// Stream group: COPY, MUL, ADD, TRIAD, DOT.
//
// Streaming layout: each CTA owns tiles of block*items 16-byte vectors
// (double2) and every thread issues all of its loads for a tile before any
// store, so a CTA keeps block*items*16 bytes per operand in flight.  The grid
// is one tile per CTA (the hardware scheduler balances the tail); arrays that
// are not 16-byte aligned take the scalar path with the same shape.
#include "b200_internal.cuh"
#include "b200_reduce.cuh"

using namespace b200;

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 4;

// Grid-stride tile loop shared by the map kernels.  `VEC` doubles per access.
#define TILE_LOOP(BS, IT, UNITS)                                              \
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT);            \
       t0 < (UNITS);                                                          \
       t0 += static_cast<int64_t>(gridDim.x) * (BS * IT))

template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

// ---- COPY ------------------------------------------------------------------
template <int BS, int IT, typename V>
__global__ void __launch_bounds__(BS)
copy_kernel(const V* __restrict__ a, V* __restrict__ c, int64_t units) {
  TILE_LOOP(BS, IT, units) {
    V r[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) r[u] = ldg(a + j);
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) c[j] = r[u];
    }
  }
}

// ---- MUL -------------------------------------------------------------------
__device__ __forceinline__ double2 mul2(double s, double2 v) {
  return make_double2(s * v.x, s * v.y);
}
__device__ __forceinline__ double mul2(double s, double v) { return s * v; }

template <int BS, int IT, typename V>
__global__ void __launch_bounds__(BS)
mul_kernel(V* __restrict__ b, const V* __restrict__ c, double alpha,
           int64_t units) {
  TILE_LOOP(BS, IT, units) {
    V r[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) r[u] = ldg(c + j);
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) b[j] = mul2(alpha, r[u]);
    }
  }
}

// ---- ADD -------------------------------------------------------------------
__device__ __forceinline__ double2 add2(double2 x, double2 y) {
  return make_double2(x.x + y.x, x.y + y.y);
}
__device__ __forceinline__ double add2(double x, double y) { return x + y; }

template <int BS, int IT, typename V>
__global__ void __launch_bounds__(BS)
add_kernel(const V* __restrict__ a, const V* __restrict__ b,
           V* __restrict__ c, int64_t units) {
  TILE_LOOP(BS, IT, units) {
    V ra[IT], rb[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) { ra[u] = ldg(a + j); rb[u] = ldg(b + j); }
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) c[j] = add2(ra[u], rb[u]);
    }
  }
}

// ---- TRIAD -----------------------------------------------------------------
__device__ __forceinline__ double2 triad2(double2 b, double alpha, double2 c) {
  return make_double2(b.x + alpha * c.x, b.y + alpha * c.y);
}
__device__ __forceinline__ double triad2(double b, double alpha, double c) {
  return b + alpha * c;
}

template <int BS, int IT, typename V>
__global__ void __launch_bounds__(BS)
triad_kernel(V* __restrict__ a, const V* __restrict__ b,
             const V* __restrict__ c, double alpha, int64_t units) {
  TILE_LOOP(BS, IT, units) {
    V rb[IT], rc[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) { rb[u] = ldg(b + j); rc[u] = ldg(c + j); }
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      int64_t j = t0 + u * BS + threadIdx.x;
      if (j < units) a[j] = triad2(rb[u], alpha, rc[u]);
    }
  }
}

// ---- DOT -------------------------------------------------------------------
// Thread partial sums run over the thread's elements in increasing index
// order; the last CTA combines the per-CTA partials in CTA order.
template <int BS, int IT>
__global__ void __launch_bounds__(BS)
dot_kernel(const double* __restrict__ a, const double* __restrict__ b,
           int64_t n, bool vec2, double dot_init, double* __restrict__ accum,
           double* __restrict__ partials, unsigned int* __restrict__ counter) {
  __shared__ double smem[BS / 32];
  __shared__ bool last_flag;
  double s = 0.0;
  if (vec2) {
    const double2* a2 = reinterpret_cast<const double2*>(a);
    const double2* b2 = reinterpret_cast<const double2*>(b);
    const int64_t units = n >> 1;
    TILE_LOOP(BS, IT, units) {
      double2 ra[IT], rb[IT];
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        int64_t j = t0 + u * BS + threadIdx.x;
        if (j < units) { ra[u] = __ldg(a2 + j); rb[u] = __ldg(b2 + j); }
      }
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        int64_t j = t0 + u * BS + threadIdx.x;
        if (j < units) { s += ra[u].x * rb[u].x; s += ra[u].y * rb[u].y; }
      }
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) s += a[n - 1] * b[n - 1];
  } else {
    TILE_LOOP(BS, IT, n) {
      double ra[IT], rb[IT];
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        int64_t j = t0 + u * BS + threadIdx.x;
        if (j < n) { ra[u] = __ldg(a + j); rb[u] = __ldg(b + j); }
      }
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        int64_t j = t0 + u * BS + threadIdx.x;
        if (j < n) s += ra[u] * rb[u];
      }
    }
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

// Shared launcher for the four map kernels: vector path when every pointer
// is 16-byte aligned, scalar path (and scalar tail) otherwise.
template <typename LaunchVec, typename LaunchScalar>
int launch_map(const char* name, int64_t n, const b200_tune* tune,
               bool all_aligned, LaunchVec&& lv, LaunchScalar&& ls) {
  Shape sh = resolve_1d(tune, 0, kBlock, kItems, 2);
  if (!valid_block(sh.block)) return invalid("%s: bad block size %d", name, sh.block);
  bool vec = all_aligned && sh.vec == 2 && n >= 2;
  int launches = 0;
  if (vec) {
    int64_t units = n >> 1;
    Shape s = resolve_1d(tune, units, kBlock, kItems, 2);
    lv(s, units);
    ++launches;
    if (n & 1) {
      ls(Shape{32, 1, 1, 1}, n - 1, int64_t{1});
      ++launches;
    }
  } else {
    Shape s = resolve_1d(tune, n, kBlock, kItems, 1);
    ls(s, int64_t{0}, n);
    ++launches;
  }
  return after_launch(name, launches);
}

}  // namespace

extern "C" {

int b200_stream_copy(const double* a, double* c, int64_t n,
                     const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!a || !c))) return invalid("b200_stream_copy: bad args");
  if (n == 0) return B200_OK;
  cudaStream_t st = as_stream(stream);
  return launch_map(
      "b200_stream_copy", n, tune, aligned16(a) && aligned16(c),
      [&](Shape s, int64_t units) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          copy_kernel<BS, IT, double2><<<s.grid, BS, 0, st>>>(
              reinterpret_cast<const double2*>(a),
              reinterpret_cast<double2*>(c), units)));
      },
      [&](Shape s, int64_t off, int64_t cnt) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          copy_kernel<BS, IT, double><<<s.grid, BS, 0, st>>>(a + off, c + off,
                                                             cnt)));
      });
}

int b200_stream_mul(double* b, const double* c, double alpha, int64_t n,
                    const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!b || !c))) return invalid("b200_stream_mul: bad args");
  if (n == 0) return B200_OK;
  cudaStream_t st = as_stream(stream);
  return launch_map(
      "b200_stream_mul", n, tune, aligned16(b) && aligned16(c),
      [&](Shape s, int64_t units) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          mul_kernel<BS, IT, double2><<<s.grid, BS, 0, st>>>(
              reinterpret_cast<double2*>(b),
              reinterpret_cast<const double2*>(c), alpha, units)));
      },
      [&](Shape s, int64_t off, int64_t cnt) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          mul_kernel<BS, IT, double><<<s.grid, BS, 0, st>>>(b + off, c + off,
                                                            alpha, cnt)));
      });
}

int b200_stream_add(const double* a, const double* b, double* c, int64_t n,
                    const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!a || !b || !c)))
    return invalid("b200_stream_add: bad args");
  if (n == 0) return B200_OK;
  cudaStream_t st = as_stream(stream);
  return launch_map(
      "b200_stream_add", n, tune, aligned16(a) && aligned16(b) && aligned16(c),
      [&](Shape s, int64_t units) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          add_kernel<BS, IT, double2><<<s.grid, BS, 0, st>>>(
              reinterpret_cast<const double2*>(a),
              reinterpret_cast<const double2*>(b),
              reinterpret_cast<double2*>(c), units)));
      },
      [&](Shape s, int64_t off, int64_t cnt) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          add_kernel<BS, IT, double><<<s.grid, BS, 0, st>>>(
              a + off, b + off, c + off, cnt)));
      });
}

int b200_stream_triad(double* a, const double* b, const double* c,
                      double alpha, int64_t n, const b200_tune* tune,
                      b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!a || !b || !c)))
    return invalid("b200_stream_triad: bad args");
  if (n == 0) return B200_OK;
  cudaStream_t st = as_stream(stream);
  return launch_map(
      "b200_stream_triad", n, tune,
      aligned16(a) && aligned16(b) && aligned16(c),
      [&](Shape s, int64_t units) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          triad_kernel<BS, IT, double2><<<s.grid, BS, 0, st>>>(
              reinterpret_cast<double2*>(a),
              reinterpret_cast<const double2*>(b),
              reinterpret_cast<const double2*>(c), alpha, units)));
      },
      [&](Shape s, int64_t off, int64_t cnt) {
        B200_DISPATCH_BLOCK(s.block, BS, B200_DISPATCH_ITEMS(s.items, IT,
          triad_kernel<BS, IT, double><<<s.grid, BS, 0, st>>>(
              a + off, b + off, c + off, alpha, cnt)));
      });
}

size_t b200_reduce_workspace_bytes(int64_t n, const b200_tune* tune) {
  int block = (tune && tune->block_size) ? tune->block_size : kBlock;
  // The smallest tile (1 item per thread) gives the largest grid, so the
  // workspace covers every reduction entry point and item count.
  return reduce_ws_bytes_for_grid(reduce_grid(n, tune, block, 1));
}

int b200_stream_dot(const double* a, const double* b, int64_t n,
                    double dot_init, double* dot_accum, void* workspace,
                    size_t workspace_bytes, const b200_tune* tune,
                    b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!a || !b)) || !dot_accum)
    return invalid("b200_stream_dot: bad args");
  int block = (tune && tune->block_size) ? tune->block_size : kBlock;
  int items = (tune && tune->items) ? tune->items : kItems;
  if (!valid_block(block)) return invalid("b200_stream_dot: bad block size %d", block);
  bool vec = aligned16(a) && aligned16(b) && !(tune && tune->vec == 1);
  int grid = reduce_grid(n, tune, block, items * (vec ? 2 : 1));
  size_t need = reduce_ws_bytes_for_grid(grid);
  if (!workspace || workspace_bytes < need) {
    set_error("b200_stream_dot: workspace %zu bytes, need %zu", workspace_bytes,
              need);
    return B200_ERR_WORKSPACE;
  }
  unsigned int* counter = static_cast<unsigned int*>(workspace);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(workspace) + 256);
  cudaStream_t st = as_stream(stream);
  B200_DISPATCH_BLOCK(block, BS, B200_DISPATCH_ITEMS(items, IT,
    dot_kernel<BS, IT><<<grid, BS, 0, st>>>(a, b, n, vec, dot_init, dot_accum,
                                            partials, counter)));
  return after_launch("b200_stream_dot");
}

}  // extern "C"
