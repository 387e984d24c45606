// FP64 adds and multiplies in the instruction form GB300's FP64 pipe issues
// fastest, with the same result bits.
//
// Measured on GB300 (a register-only loop, 2048 threads per SM): a DFMA whose
// three operands are per-thread registers sustains 595 G
// thread-instructions/s, about 2 per clock per SM; DADD, DMUL and a DFMA with
// a kernel-argument operand (constant bank, or a uniform register holding a
// value that is the same for every thread) sustain 501 G/s, 5/6 of that.
// So an add or a multiply written as a per-thread-register FMA can issue 19%
// faster:
//   a + b == fma(a, 1.0, b)    a * 1.0 is exact, then one rounding of a + b
//   a - b == fma(a, 1.0, -b)
//   a * b == fma(a, b, -0.0)   x + (-0.0) == x for every x, +0 and -0 included
// for every input, signed zeros, infinities and NaNs included.  The 1.0 and
// -0.0 must be per-thread registers the compiler cannot see through (a literal
// is folded back into the add or multiply, a kernel argument stays uniform):
// Regs builds them from threadIdx.x and a kernel argument that is zero at run
// time, and reg() does the same for a coefficient passed as a kernel argument.
#pragma once

#include <cstdint>

namespace b200 {
namespace fform {

struct Regs {
  double one;
  double negzero;
};

__device__ __forceinline__ unsigned long long thread_zero(int zero) {
  return static_cast<unsigned long long>(threadIdx.x & static_cast<unsigned>(zero));
}

__device__ __forceinline__ Regs regs(int zero) {
  const unsigned long long z = thread_zero(zero);
  return Regs{__longlong_as_double(static_cast<long long>(0x3FF0000000000000ULL + z)),
              __longlong_as_double(static_cast<long long>(0x8000000000000000ULL + z))};
}

// v in a per-thread register (for a coefficient that arrives as a kernel
// argument and would otherwise be a constant-bank or uniform operand).
__device__ __forceinline__ double reg(double v, int zero) {
  return __longlong_as_double(
      static_cast<long long>(static_cast<unsigned long long>(__double_as_longlong(v)) +
                             thread_zero(zero)));
}

__device__ __forceinline__ double add(double a, double b, const Regs& r) {
  return fma(a, r.one, b);
}
__device__ __forceinline__ double sub(double a, double b, const Regs& r) {
  return fma(a, r.one, -b);
}
__device__ __forceinline__ double mul(double a, double b, const Regs& r) {
  return fma(a, b, r.negzero);
}

}  // namespace fform
}  // namespace b200
