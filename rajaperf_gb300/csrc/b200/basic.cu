// Basic group kernels used by the batched small-size suite: DAXPY, INIT3,
// MULADDSUB (suite src/basic/*.hpp bodies).
#include "b200_internal.cuh"
#include "b200_map.cuh"

using namespace b200;

namespace {

// basic/DAXPY.hpp: y[i] += a * x[i]
struct Daxpy {
  double* __restrict__ y;
  const double* __restrict__ x;
  double a;
  __device__ void operator()(int64_t i) const { y[i] += a * ld(x + i); }
};

// basic/INIT3.hpp: out1 = out2 = out3 = -in1 - in2
struct Init3 {
  double* __restrict__ out1;
  double* __restrict__ out2;
  double* __restrict__ out3;
  const double* __restrict__ in1;
  const double* __restrict__ in2;
  __device__ void operator()(int64_t i) const {
    const double v = -ld(in1 + i) - ld(in2 + i);
    out3[i] = v;
    out2[i] = v;
    out1[i] = v;
  }
};

// basic/MULADDSUB.hpp
struct MulAddSub {
  double* __restrict__ out1;
  double* __restrict__ out2;
  double* __restrict__ out3;
  const double* __restrict__ in1;
  const double* __restrict__ in2;
  __device__ void operator()(int64_t i) const {
    const double a = ld(in1 + i), b = ld(in2 + i);
    out1[i] = a * b;
    out2[i] = a + b;
    out3[i] = a - b;
  }
};

}  // namespace

extern "C" {

int b200_basic_daxpy(double* y, const double* x, double a, int64_t n,
                     const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return invalid("b200_basic_daxpy: bad args");
  return launch_map1d("b200_basic_daxpy", Daxpy{y, x, a}, n, tune, as_stream(stream));
}

int b200_basic_init3(double* out1, double* out2, double* out3, const double* in1,
                     const double* in2, int64_t n, const b200_tune* tune,
                     b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!out1 || !out2 || !out3 || !in1 || !in2)))
    return invalid("b200_basic_init3: bad args");
  return launch_map1d("b200_basic_init3", Init3{out1, out2, out3, in1, in2}, n, tune,
                      as_stream(stream));
}

int b200_basic_muladdsub(double* out1, double* out2, double* out3, const double* in1,
                         const double* in2, int64_t n, const b200_tune* tune,
                         b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!out1 || !out2 || !out3 || !in1 || !in2)))
    return invalid("b200_basic_muladdsub: bad args");
  return launch_map1d("b200_basic_muladdsub", MulAddSub{out1, out2, out3, in1, in2}, n,
                      tune, as_stream(stream));
}

}  // extern "C"
