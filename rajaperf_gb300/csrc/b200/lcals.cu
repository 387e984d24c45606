// LCALS group: HYDRO_1D, HYDRO_2D, EOS, FIRST_DIFF, INT_PREDICT, FIRST_MIN,
// DIFF_PREDICT, PLANCKIAN.  Each functor body is the suite's macro body for
// one index (citations at each functor); the arithmetic is written in the
// macro's operation order.
#include "b200_internal.cuh"
#include "b200_f64emu.cuh"
#include "b200_fma_form.cuh"
#include "b200_map.cuh"
#include "b200_reduce.cuh"

#include <type_traits>

using namespace b200;

namespace {

// lcals/HYDRO_1D.hpp:30.  Register-operand FMAs throughout (fform: the
// product r * z as an FMA with -0, the coefficients in per-thread registers),
// which the FP64 pipe issues at its full rate; `zero` is 0 at run time.
struct Hydro1D {
  double* __restrict__ x;
  const double* __restrict__ y;
  const double* __restrict__ z;
  double q, r, t;
  int zero;
  __device__ void operator()(int64_t i) const {
    const fform::Regs fr = fform::regs(zero);
    x[i] = fma(ld(y + i), fma(fform::reg(t, zero), ld(z + i + 11),
                              fform::mul(fform::reg(r, zero), ld(z + i + 10), fr)),
               fform::reg(q, zero));
  }
};

// lcals/EOS.hpp:33: x = u + r (z + r y) + t (u3 + r (u2 + r u1) + t (u6 +
// q (u5 + q u4))), each a + b * c an FMA as the compiler contracts it, with
// q, r, t in per-thread registers (fform::reg) so that every FMA has
// register operands; `zero` is 0 at run time.
struct Eos {
  double* __restrict__ x;
  const double* __restrict__ y;
  const double* __restrict__ z;
  const double* __restrict__ u;
  double q, r, t;
  int zero;
  __device__ void operator()(int64_t i) const {
    const double rr = fform::reg(r, zero), tr = fform::reg(t, zero), qr = fform::reg(q, zero);
    const double a = fma(rr, fma(rr, ld(y + i), ld(z + i)), ld(u + i));
    const double b = fma(rr, fma(rr, ld(u + i + 1), ld(u + i + 2)), ld(u + i + 3));
    const double c = fma(qr, fma(qr, ld(u + i + 4), ld(u + i + 5)), ld(u + i + 6));
    x[i] = fma(tr, fma(tr, c, b), a);
  }
};

// Element map with part of each element's FP64 work on the integer pipes.
// F::split(i, regs, slow) computes element i with some operations in an
// exact integer form (bit-identical to the FP64 pipe's) and sets `slow` when
// an operand leaves that form's range; F::exact(i, regs) is the all-FP64
// form.  A CTA covers PT * BS consecutive elements, a thread every BS-th of
// them (coalesced).  An element that met `slow` stores nothing in the loop
// and is redone with F::exact after it (one bit per element): an FP64 redo
// inside the loop would be compiled as predicated FP64 instructions, which
// occupy the FP64 pipe in every warp.
template <int BS, int PT, class F>
__global__ void __launch_bounds__(BS) split_map_kernel(F f, int64_t n) {
  static_assert(PT >= 1 && PT <= 64, "one redo bit per element");
  const auto rg = f.regs();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * BS * PT + threadIdx.x;
  uint64_t redo = 0;
  auto element = [&](int p) {
    const int64_t i = base + static_cast<int64_t>(p) * BS;
    bool slow = false;
    const double v = f.split(i, rg, slow);
    if (!slow) f.store(i, v);
    else redo |= 1ull << p;
  };
  if (static_cast<int64_t>(blockIdx.x + 1) * BS * PT <= n) {
    // a whole CTA in range: no bounds test, so the unrolled elements' loads
    // issue together
#pragma unroll
    for (int p = 0; p < PT; ++p) element(p);
  } else {
    for (int p = 0; p < PT; ++p) {
      if (base + static_cast<int64_t>(p) * BS >= n) break;
      element(p);
    }
  }
  if (__any_sync(__activemask(), redo != 0)) {
    for (int p = 0; p < PT; ++p) {
      const int64_t i = base + static_cast<int64_t>(p) * BS;
      if (i < n && ((redo >> p) & 1u)) f.store(i, f.exact(i, rg));
    }
  }
}

// EOS with KF of each element's eight FMAs on the integer pipes
// (f64emu::fma_pos_fast), in the order r*y+z, r*u1+u2, q*u4+u5, then the
// three outer ones of each group, then the two in t.
template <int KF>
struct EosSplit {
  double* __restrict__ x;
  const double* __restrict__ y;
  const double* __restrict__ z;
  const double* __restrict__ u;
  double q, r, t;
  int zero;
  struct Regs { double q, r, t; };
  __device__ Regs regs() const {
    return {fform::reg(q, zero), fform::reg(r, zero), fform::reg(t, zero)};
  }
  __device__ double split(int64_t i, const Regs& g, bool& slow) const {
    auto f = [&](int m, double a, double b, double c) {
      return (m < KF) ? f64emu::fma_pos_fast(a, b, c, slow) : fma(a, b, c);
    };
    const double a1 = f(0, g.r, ld(y + i), ld(z + i));
    const double b1 = f(1, g.r, ld(u + i + 1), ld(u + i + 2));
    const double c1 = f(2, g.q, ld(u + i + 4), ld(u + i + 5));
    const double a = f(3, g.r, a1, ld(u + i));
    const double b = f(4, g.r, b1, ld(u + i + 3));
    const double c = f(5, g.q, c1, ld(u + i + 6));
    return f(7, g.t, f(6, g.t, c, b), a);
  }
  __device__ double exact(int64_t i, const Regs& g) const {
    const double a = fma(g.r, fma(g.r, ld(y + i), ld(z + i)), ld(u + i));
    const double b = fma(g.r, fma(g.r, ld(u + i + 1), ld(u + i + 2)), ld(u + i + 3));
    const double c = fma(g.q, fma(g.q, ld(u + i + 4), ld(u + i + 5)), ld(u + i + 6));
    return fma(g.t, fma(g.t, c, b), a);
  }
  __device__ void store(int64_t i, double v) const { x[i] = v; }
};

// Launches split_map_kernel<bs, pt, F> for bs in {128, 256, 512} and pt in
// {1, 2, 4, 8} (the caller checks both).
template <class F>
int launch_split_map(const char* name, const F& f, int64_t n, int bs, int pt, cudaStream_t st) {
  const int64_t grid = ceil_div(n, static_cast<int64_t>(bs) * pt);
  if (grid > 0x7fffffff) return invalid("%s: n too large", name);
  auto go = [&](auto B, auto P) {
    split_map_kernel<decltype(B)::value, decltype(P)::value, F>
        <<<static_cast<unsigned>(grid), decltype(B)::value, 0, st>>>(f, n);
  };
  auto by_pt = [&](auto B) {
    switch (pt) {
      case 1: go(B, std::integral_constant<int, 1>{}); break;
      case 2: go(B, std::integral_constant<int, 2>{}); break;
      case 4: go(B, std::integral_constant<int, 4>{}); break;
      default: go(B, std::integral_constant<int, 8>{}); break;
    }
  };
  if (bs == 128) by_pt(std::integral_constant<int, 128>{});
  else if (bs == 256) by_pt(std::integral_constant<int, 256>{});
  else by_pt(std::integral_constant<int, 512>{});
  return after_launch(name);
}

// lcals/FIRST_DIFF.hpp:25
struct FirstDiff {
  double* __restrict__ x;
  const double* __restrict__ y;
  __device__ void operator()(int64_t i) const { x[i] = ld(y + i + 1) - ld(y + i); }
};

// lcals/INT_PREDICT.hpp:40 -- px[0..n) is written, planes 2..12 are read.
struct IntPredict {
  double* px;
  int64_t o;
  double dm22, dm23, dm24, dm25, dm26, dm27, dm28, c0;
  // The first product runs on the integer pipe (f64emu::mul_fast, correctly
  // rounded); the rest of the sum contracts into FMAs on the FP64 pipe.
  __device__ void operator()(int64_t i) const {
    const double* p = px;
    const double p12 = ld(p + i + o * 12);
    bool slow = false;
    const double first = f64emu::mul_fast(dm28, p12, slow);
    double v = first + dm27 * ld(p + i + o * 11) +
               dm26 * ld(p + i + o * 10) + dm25 * ld(p + i + o * 9) +
               dm24 * ld(p + i + o * 8) + dm23 * ld(p + i + o * 7) +
               dm22 * ld(p + i + o * 6) +
               c0 * (ld(p + i + o * 4) + ld(p + i + o * 5)) + ld(p + i + o * 2);
    if (__any_sync(__activemask(), slow) && slow)
      v = dm28 * p12 + dm27 * ld(p + i + o * 11) +
          dm26 * ld(p + i + o * 10) + dm25 * ld(p + i + o * 9) +
          dm24 * ld(p + i + o * 8) + dm23 * ld(p + i + o * 7) +
          dm22 * ld(p + i + o * 6) +
          c0 * (ld(p + i + o * 4) + ld(p + i + o * 5)) + ld(p + i + o * 2);
    px[i] = v;
  }
};

// lcals/DIFF_PREDICT.hpp -- planes 4..13 of px are updated in place per i.
struct DiffPredict {
  double* px;
  const double* __restrict__ cx;
  int64_t o;
  // The suite reads each plane of px before overwriting it and never reads
  // it again, and for o = n >= 1 the planes are disjoint: so all ten loads
  // are issued first (independent, in flight together) and the ten stores
  // follow.  The same differences, in the same order, as the macro.
  __device__ void operator()(int64_t i) const {
    double p[9];  // planes 4..12 before the update
#pragma unroll
    for (int k = 0; k < 9; ++k) p[k] = px[i + o * (4 + k)];
    double ar, br, cr;
    double q4, q5, q6, q7, q8, q9, q10, q11, q12, q13;
    ar = ld(cx + i + o * 4);
    br = ar - p[0];
    q4 = ar;
    cr = br - p[1];
    q5 = br;
    ar = cr - p[2];
    q6 = cr;
    br = ar - p[3];
    q7 = ar;
    cr = br - p[4];
    q8 = br;
    ar = cr - p[5];
    q9 = cr;
    br = ar - p[6];
    q10 = ar;
    cr = br - p[7];
    q11 = br;
    q13 = cr - p[8];
    q12 = cr;
    px[i + o * 4] = q4;
    px[i + o * 5] = q5;
    px[i + o * 6] = q6;
    px[i + o * 7] = q7;
    px[i + o * 8] = q8;
    px[i + o * 9] = q9;
    px[i + o * 10] = q10;
    px[i + o * 11] = q11;
    px[i + o * 12] = q12;
    px[i + o * 13] = q13;
  }
};

// lcals/PLANCKIAN.hpp
struct Planckian {
  const double* __restrict__ x;
  double* __restrict__ y;
  const double* __restrict__ u;
  const double* __restrict__ v;
  double* __restrict__ w;
  // The two divisions run on the integer and FP32 pipes (f64emu::div_fast,
  // correctly rounded); an element with an operand or quotient outside its
  // fast path (zero, subnormal, non-finite) is recomputed natively.
  __device__ void operator()(int64_t i) const {
    bool slow = false;
    const double ui = ld(u + i), vi = ld(v + i), xi = ld(x + i);
    double yi = f64emu::div_fast(ui, vi, slow);
    double wi = f64emu::div_fast(xi, exp(yi) - 1.0, slow);
    if (__any_sync(__activemask(), slow) && slow) {
      yi = ui / vi;
      wi = xi / (exp(yi) - 1.0);
    }
    y[i] = yi;
    w[i] = wi;
  }
};

// ---- HYDRO_2D ---------------------------------------------------------------
// lcals/HYDRO_2D.hpp:66-90.  Pass 1 (BODY1) writes za, zb on the interior;
// pass 2 fuses BODY2 and BODY3 (both point-wise given za, zb), so a rep is two
// launches instead of three and zu/zv are not re-read for BODY3.
template <int BS>
__global__ void __launch_bounds__(BS)
hydro2d_body1(double* __restrict__ za, double* __restrict__ zb,
              const double* __restrict__ zm, const double* __restrict__ zp,
              const double* __restrict__ zq, const double* __restrict__ zr,
              int64_t kn, int64_t jn, int zero) {
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.x) * BS + threadIdx.x;
  if (j >= jn - 1) return;
  // The two divisions and the two products run on the integer and FP32
  // pipes (f64emu::div_fast and f64emu::mul_fast, correctly rounded,
  // bit-identical to the FP64 divide and multiply); the FP64 pipe keeps the
  // 10 adds of a point, as register-operand FMAs (fform, bit-identical, full
  // FP64 rate where DADD gets 5/6 of it; `zero` is 0 at run time).  A thread
  // that met a zero, subnormal or non-finite operand, product or quotient
  // rewrites its points with the FP64 pipe after the loop.
  const fform::Regs fr = fform::regs(zero);
  bool slow = false;
  for (int64_t k = 1 + blockIdx.y; k < kn - 1; k += gridDim.y) {
    const int64_t c = j + k * jn;
    za[c] = f64emu::div_fast(
        f64emu::mul_fast(
            fform::sub(fform::sub(fform::add(ld(zp + c - 1 + jn), ld(zq + c - 1 + jn), fr),
                                  ld(zp + c - 1), fr),
                       ld(zq + c - 1), fr),
            fform::add(ld(zr + c), ld(zr + c - 1), fr), slow),
        fform::add(ld(zm + c - 1), ld(zm + c - 1 + jn), fr), slow);
    zb[c] = f64emu::div_fast(
        f64emu::mul_fast(
            fform::sub(fform::sub(fform::add(ld(zp + c - 1), ld(zq + c - 1), fr), ld(zp + c), fr),
                       ld(zq + c), fr),
            fform::add(ld(zr + c), ld(zr + c - jn), fr), slow),
        fform::add(ld(zm + c), ld(zm + c - 1), fr), slow);
  }
  if (__any_sync(__activemask(), slow) && slow) {
    for (int64_t k = 1 + blockIdx.y; k < kn - 1; k += gridDim.y) {
      const int64_t c = j + k * jn;
      za[c] = (ld(zp + c - 1 + jn) + ld(zq + c - 1 + jn) - ld(zp + c - 1) - ld(zq + c - 1)) *
              (ld(zr + c) + ld(zr + c - 1)) / (ld(zm + c - 1) + ld(zm + c - 1 + jn));
      zb[c] = (ld(zp + c - 1) + ld(zq + c - 1) - ld(zp + c) - ld(zq + c)) *
              (ld(zr + c) + ld(zr + c - jn)) / (ld(zm + c) + ld(zm + c - 1));
    }
  }
}

// KH of the eight differences (du1..du4, dv1..dv4 in that order) run on the
// integer pipes (f64emu::sub_near_fast, bit-identical).  A point whose
// operands are outside that form's range stores nothing in the loop (zu and
// zv are updated in place, so its inputs stay intact) and is redone on the
// FP64 pipe after the loop; a thread holds at most 64 points (the launcher
// checks), one bit each.  An FP64 redo inside the loop would be compiled as
// predicated FP64 instructions, which occupy the FP64 pipe in every warp.
template <int BS, int KH>
__global__ void __launch_bounds__(BS)
hydro2d_body23(const double* __restrict__ za, const double* __restrict__ zb,
               const double* __restrict__ zr, double* __restrict__ zu,
               double* __restrict__ zv, const double* __restrict__ zz,
               double* __restrict__ zrout, double* __restrict__ zzout, double s,
               double t, int64_t kn, int64_t jn, int zero) {
  static_assert(KH >= 0 && KH <= 8, "0..8 integer-pipe differences");
  const int64_t j = 1 + static_cast<int64_t>(blockIdx.x) * BS + threadIdx.x;
  if (j >= jn - 1) return;
  const unsigned live = __activemask();
  // Every FP64 instruction a register-operand FMA (fform: the differences and
  // the leading products, s and t in per-thread registers), which the FP64
  // pipe issues at its full rate; `zero` is 0 at run time.  (The leading
  // product on the integer pipe gained nothing: its two-instruction fallback
  // is compiled as predicated FP64 multiplies, which occupy the FP64 pipe
  // like executed ones.)
  const fform::Regs fr = fform::regs(zero);
  const double sr = fform::reg(s, zero), tr = fform::reg(t, zero);
  auto point = [&](int64_t c, bool use_int, bool& slow) {
    const double za0 = ld(za + c), za1 = ld(za + c - 1);
    const double zb0 = ld(zb + c), zb1 = ld(zb + c + jn);
    const double zz0 = ld(zz + c), zr0 = ld(zr + c);
    const int64_t off[4] = {1, -1, -jn, jn};
    double du[4], dv[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const double zn = ld(zz + c + off[m]), rn = ld(zr + c + off[m]);
      du[m] = (use_int && m < KH) ? f64emu::sub_near_fast(zz0, zn, slow) : fform::sub(zz0, zn, fr);
      dv[m] = (use_int && m + 4 < KH) ? f64emu::sub_near_fast(zr0, rn, slow)
                                      : fform::sub(zr0, rn, fr);
    }
    // zu + s * (((za0 du1 - za1 du2) - zb0 du3) + zb1 du4), left to right as
    // the suite writes it, the products after the first and s * (...) as FMAs
    const double u = fma(sr, fma(zb1, du[3], fma(-zb0, du[2], fma(-za1, du[1], fform::mul(za0, du[0], fr)))),
                         zu[c]);
    const double v = fma(sr, fma(zb1, dv[3], fma(-zb0, dv[2], fma(-za1, dv[1], fform::mul(za0, dv[0], fr)))),
                         zv[c]);
    if (!slow) {
      zu[c] = u;
      zv[c] = v;
      zrout[c] = fma(tr, u, zr0);
      zzout[c] = fma(tr, v, zz0);
    }
  };
  uint64_t redo = 0;
  int it = 0;
  for (int64_t k = 1 + blockIdx.y; k < kn - 1; k += gridDim.y, ++it) {
    bool slow = false;
    point(j + k * jn, KH > 0, slow);
    if (slow) redo |= 1ull << it;
  }
  if (KH > 0 && __any_sync(live, redo != 0)) {
    it = 0;
    for (int64_t k = 1 + blockIdx.y; k < kn - 1; k += gridDim.y, ++it) {
      bool slow = false;
      if ((redo >> it) & 1u) point(j + k * jn, false, slow);
    }
  }
}

// ---- FIRST_MIN --------------------------------------------------------------
// lcals/FIRST_MIN.hpp:29-54, FIRST_MIN-Seq.cpp:34-48: strict '<' scan, so the
// result is the smallest index holding the minimum (or initloc when the
// initial value is not beaten).  Compares run on order-preserving integer keys
// (order_key), which order exactly as '<' on the doubles.
template <int BS, int IT, bool VEC>
__global__ void __launch_bounds__(BS)
first_min_kernel(const double* __restrict__ x, int64_t n, double xmin_init,
                 int64_t initloc, int64_t* __restrict__ minloc_out,
                 double* __restrict__ minval_out, KeyLoc* __restrict__ partials,
                 unsigned int* __restrict__ counter) {
  __shared__ KeyLoc smem[BS / 32];
  __shared__ bool last_flag;
  const long long* xb = reinterpret_cast<const long long*>(x);
  // A NaN initial value is never beaten by a strict '<' scan: give it the
  // smallest key so that nothing compares less.
  const KeyLoc init{isnan(xmin_init) ? static_cast<long long>(0x8000000000000000ULL)
                                     : order_key(__double_as_longlong(xmin_init)),
                    initloc};
  KeyLoc m = init;
  // Cheap filter: the order key of an element's high 32 bits never exceeds
  // the high word of its full key (exact for normal values; -0 and NaNs map
  // lower), so an element whose filter key is above the running minimum's
  // high word cannot be smaller and skips the full 64-bit key.
  int mh = static_cast<int>(m.key >> 32);
  auto maybe = [&](long long bits) {
    const int h = static_cast<int>(bits >> 32);
    return (h ^ ((h >> 31) & 0x7fffffff)) <= mh;
  };
  if (VEC) {
    // 16-byte loads of element pairs; a thread still meets its indices in
    // increasing order, so strict '<' keeps the first minimum it sees.
    const longlong2* xv = reinterpret_cast<const longlong2*>(x);
    const int64_t nv = n >> 1;
    for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < nv;
         t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
      longlong2 v[IT];
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int64_t iv = t0 + u * BS + threadIdx.x;
        v[u] = (iv < nv) ? __ldg(xv + iv) : make_longlong2(0LL, 0LL);
      }
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int64_t iv = t0 + u * BS + threadIdx.x;
        if (iv < nv && (maybe(v[u].x) || maybe(v[u].y))) {
          const long long k0 = order_key(v[u].x), k1 = order_key(v[u].y);
          if (k0 < m.key) { m.key = k0; m.loc = 2 * iv; }
          if (k1 < m.key) { m.key = k1; m.loc = 2 * iv + 1; }
          mh = static_cast<int>(m.key >> 32);
        }
      }
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {  // odd tail element
      const long long k = order_key(__ldg(xb + n - 1));
      if (k < m.key) { m.key = k; m.loc = n - 1; }
    }
  } else {
    for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * (BS * IT); t0 < n;
         t0 += static_cast<int64_t>(gridDim.x) * (BS * IT)) {
      long long v[IT];
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        int64_t i = t0 + u * BS + threadIdx.x;
        v[u] = (i < n) ? __ldg(xb + i) : 0LL;
      }
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        int64_t i = t0 + u * BS + threadIdx.x;
        if (i < n && maybe(v[u])) {
          long long k = order_key(v[u]);
          if (k < m.key) { m.key = k; m.loc = i; }
          mh = static_cast<int>(m.key >> 32);
        }
      }
    }
  }
  m = block_keyloc<BS>(m, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = m;
  if (arrive_last(counter, &last_flag)) {
    KeyLoc a = init;
    for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += BS) {
      KeyLoc p;
      p.key = __ldcg(&partials[i].key);
      p.loc = __ldcg(&partials[i].loc);
      a = keyloc_pick(a, p);
    }
    a = block_keyloc<BS>(a, smem);
    if (threadIdx.x == 0) {
      *minloc_out = a.loc;
      if (minval_out) {
        *minval_out = (a.loc == initloc && a.key == init.key) ? xmin_init : x[a.loc];
      }
      *counter = 0u;
    }
  }
}

dim3 rows_grid(int64_t jn, int64_t kn, int bs) {
  int64_t gx = ceil_div(jn - 2 > 0 ? jn - 2 : 1, bs);
  int64_t gy = kn - 2 > 0 ? kn - 2 : 1;
  if (gy > 65535) gy = 65535;
  return dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy), 1);
}

}  // namespace

extern "C" {

int b200_lcals_hydro_1d(double* x, const double* y, const double* z, double q,
                        double r, double t, int64_t n, const b200_tune* tune,
                        b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y || !z))) return invalid("b200_lcals_hydro_1d: bad args");
  // Its inner FMA on the integer pipes (f64emu::fma_pos_fast) measured no
  // faster at 2^27 (655-680 us against 660): at 24 bytes an element the
  // integer pipes have about 70 instructions per element to spare, and that
  // FMA takes some 80.
  return launch_map1d("b200_lcals_hydro_1d", Hydro1D{x, y, z, q, r, t, 0}, n, tune,
                      as_stream(stream));
}

// EOS FMAs per element on the integer pipes by default (0: the map kernel).
// Measured on GB300 (us at 2^24 / 2^27): 0 (map kernel, 256 x 2): 223.2 /
// 1729.5; with 128 threads and 2 elements per thread 2: 176.1 / 1374.2, 3:
// 188.4 / 1473.1; with 16 elements per thread 1: 206.8, 2: 194.6, 3: 223.2,
// 4: 258.0 at 2^24 (each integer FMA some 80 integer instructions: from 3
// on, the integer pipes are the bound).
constexpr int kEosIntFmas = 2;
constexpr int kEosPerThread = 2;

int b200_lcals_eos(double* x, const double* y, const double* z, const double* u,
                   double q, double r, double t, int64_t n, const b200_tune* tune,
                   b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y || !z || !u))) return invalid("b200_lcals_eos: bad args");
  // tune->tile_z = 1 + FMAs per element on the integer pipes (0..3), items =
  // elements per thread (1, 2, 4 or 8), block_size 128, 256 or 512; 0 keeps
  // the defaults.  No integer FMAs, or another block size: the element-map
  // kernel (tune->block_size, items), all eight FMAs on the FP64 pipe.
  const int kf = (tune && tune->tile_z > 0) ? tune->tile_z - 1 : kEosIntFmas;
  if (kf < 0 || kf > 3) return invalid("b200_lcals_eos: bad tile_z");
  const int bs = (tune && tune->block_size) ? tune->block_size : 128;
  if (kf == 0 || n == 0 || (bs != 128 && bs != 256 && bs != 512))
    return launch_map1d("b200_lcals_eos", Eos{x, y, z, u, q, r, t, 0}, n, tune,
                        as_stream(stream));
  const int pt = (tune && tune->items) ? tune->items : kEosPerThread;
  if (pt != 1 && pt != 2 && pt != 4 && pt != 8) return invalid("b200_lcals_eos: bad items %d", pt);
  cudaStream_t st = as_stream(stream);
  switch (kf) {
    case 1: return launch_split_map("b200_lcals_eos", EosSplit<1>{x, y, z, u, q, r, t, 0}, n, bs, pt, st);
    case 2: return launch_split_map("b200_lcals_eos", EosSplit<2>{x, y, z, u, q, r, t, 0}, n, bs, pt, st);
    default: return launch_split_map("b200_lcals_eos", EosSplit<3>{x, y, z, u, q, r, t, 0}, n, bs, pt, st);
  }
}

int b200_lcals_first_diff(double* x, const double* y, int64_t n, const b200_tune* tune,
                          b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return invalid("b200_lcals_first_diff: bad args");
  // 8 items per thread: more loads in flight per thread (2^24: 93.5% -> 97.9%
  // of the copy peak on GB300)
  return launch_map1d("b200_lcals_first_diff", FirstDiff{x, y}, n, tune, as_stream(stream),
                      256, 8);
}

int b200_lcals_int_predict(double* px, double dm22, double dm23, double dm24,
                           double dm25, double dm26, double dm27, double dm28,
                           double c0, int64_t n, const b200_tune* tune,
                           b200_stream_t stream) {
  if (n < 0 || (n > 0 && !px)) return invalid("b200_lcals_int_predict: bad args");
  return launch_map1d("b200_lcals_int_predict",
                      IntPredict{px, n, dm22, dm23, dm24, dm25, dm26, dm27, dm28, c0}, n,
                      tune, as_stream(stream));
}

int b200_lcals_diff_predict(double* px, const double* cx, int64_t n,
                            const b200_tune* tune, b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!px || !cx))) return invalid("b200_lcals_diff_predict: bad args");
  return launch_map1d("b200_lcals_diff_predict", DiffPredict{px, cx, n}, n, tune,
                      as_stream(stream));
}

int b200_lcals_planckian(const double* x, double* y, const double* u, const double* v,
                         double* w, int64_t n, const b200_tune* tune,
                         b200_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y || !u || !v || !w)))
    return invalid("b200_lcals_planckian: bad args");
  return launch_map1d("b200_lcals_planckian", Planckian{x, y, u, v, w}, n, tune,
                      as_stream(stream));
}

// HYDRO_2D's BODY2 differences on the integer pipes by default (of 8).
// Measured on GB300 (us per rep at 4096^2, BODY1 + BODY2/3, 64 threads):
// 0: 864.9, 2: 815.1, 4: 764.5, 6: 756.4, 8: 832.1 (BODY2/3 alone: 546 us
// at 0, 447 at 4 with the FP64 pipe 97% and the integer ALU 55% busy, 516
// at 8 with the ALU 90% busy and the FP64 pipe 63%).
constexpr int kHydroIntSubs = 6;

int b200_lcals_hydro_2d(double* za, double* zb, const double* zm, const double* zp,
                        const double* zq, const double* zr, double* zu, double* zv,
                        const double* zz, double* zrout, double* zzout, double s,
                        double t, int64_t kn, int64_t jn, const b200_tune* tune,
                        b200_stream_t stream) {
  if (kn < 0 || jn < 0 || !za || !zb || !zm || !zp || !zq || !zr || !zu || !zv || !zz ||
      !zrout || !zzout)
    return invalid("b200_lcals_hydro_2d: bad args");
  if (kn < 3 || jn < 3) return B200_OK;  // empty interior
  int bs = (tune && tune->block_size) ? tune->block_size : 128;
  if (!valid_block(bs)) return invalid("b200_lcals_hydro_2d: bad block size %d", bs);
  cudaStream_t st = as_stream(stream);
  dim3 grid = rows_grid(jn, kn, bs);
  // tune->tile_z = 1 + differences of BODY2 on the integer pipes (0, 2, 4,
  // 6 or 8); 0 keeps the default
  int kh = (tune && tune->tile_z > 0) ? tune->tile_z - 1 : kHydroIntSubs;
  if (kh < 0 || kh > 8 || (kh & 1)) return invalid("b200_lcals_hydro_2d: bad tile_z");
  if (ceil_div(kn - 2, static_cast<int64_t>(grid.y)) > 64) kh = 0;  // one redo bit per point
  B200_DISPATCH_BLOCK(bs, BS,
    hydro2d_body1<BS><<<grid, BS, 0, st>>>(za, zb, zm, zp, zq, zr, kn, jn, 0);
    auto body23 = [&](auto K) {
      hydro2d_body23<BS, decltype(K)::value><<<grid, BS, 0, st>>>(za, zb, zr, zu, zv, zz, zrout,
                                                                  zzout, s, t, kn, jn, 0);
    };
    switch (kh) {
      case 0: body23(std::integral_constant<int, 0>{}); break;
      case 2: body23(std::integral_constant<int, 2>{}); break;
      case 4: body23(std::integral_constant<int, 4>{}); break;
      case 6: body23(std::integral_constant<int, 6>{}); break;
      default: body23(std::integral_constant<int, 8>{}); break;
    });
  return after_launch("b200_lcals_hydro_2d", 2);
}

int b200_lcals_first_min(const double* x, int64_t n, double xmin_init, int64_t initloc,
                         int64_t* minloc, double* minval, void* workspace,
                         size_t workspace_bytes, const b200_tune* tune,
                         b200_stream_t stream) {
  if (n < 0 || (n > 0 && !x) || !minloc) return invalid("b200_lcals_first_min: bad args");
  int block = (tune && tune->block_size) ? tune->block_size : 256;
  int items = (tune && tune->items) ? tune->items : 8;
  if (!valid_block(block)) return invalid("b200_lcals_first_min: bad block size %d", block);
  // 16-byte pair loads when x is aligned (tune->vec == 1 forces 8-byte loads)
  const bool vec = aligned16(x) && !(tune && tune->vec == 1) && n >= 2;
  int grid = reduce_grid(vec ? (n + 1) / 2 : n, tune, block, items);
  size_t need = reduce_ws_bytes_for_grid(grid);
  if (!workspace || workspace_bytes < need) {
    set_error("b200_lcals_first_min: workspace %zu bytes, need %zu", workspace_bytes, need);
    return B200_ERR_WORKSPACE;
  }
  unsigned int* counter = static_cast<unsigned int*>(workspace);
  KeyLoc* partials = reinterpret_cast<KeyLoc*>(static_cast<char*>(workspace) + 256);
  cudaStream_t st = as_stream(stream);
  if (vec) {
    B200_DISPATCH_BLOCK(block, BS, B200_DISPATCH_ITEMS(items, IT,
      first_min_kernel<BS, IT, true><<<grid, BS, 0, st>>>(x, n, xmin_init, initloc, minloc,
                                                          minval, partials, counter)));
  } else {
    B200_DISPATCH_BLOCK(block, BS, B200_DISPATCH_ITEMS(items, IT,
      first_min_kernel<BS, IT, false><<<grid, BS, 0, st>>>(x, n, xmin_init, initloc, minloc,
                                                           minval, partials, counter)));
  }
  return after_launch("b200_lcals_first_min");
}

}  // extern "C"
