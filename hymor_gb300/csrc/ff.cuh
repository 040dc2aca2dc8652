// Float-float arithmetic on the FP32 pipe: the viscous terms of the RK-step flux and the
// Taylor propagator's matvecs.
//
// On GB300 one FP64 warp instruction issues per ~70 cycles of an SM sub-partition and one
// FP32 warp instruction per cycle, so an FP64 operation costs as much as ~70 FP32 ones. A
// float-float value is the unevaluated sum h + l of two floats with |l| <= ulp(h) / 2,
// about 48 significant bits (Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18 (1971) 224-242): an addition is Knuth's TwoSum of
// the high parts plus the low parts, a product is the exact product of the high parts
// (TwoProduct, with a fused multiply-add) plus the cross terms; each is renormalised by
// the fast two-sum. These are the "sloppy" forms: their error is ~2^-47 of the operands'
// magnitude, which is all the viscous fluxes need (their rounding then stays ~1e-15 of
// the face-flux scale).
//
// Conversions go through the bit patterns on the integer pipe, so that the FP64 pipe only
// sees the one addition that joins a result back into a double (a cvt between f32 and f64
// issues on the FP64 pipe at the DFMA rate on this GPU). The halo velocities u = rho_u / rho
// are float-float quotients too (ff_rcp), and the face area and the viscous work term are
// applied in float-float before the join, so that the FP64 pipe sees only the inviscid
// fluxes and the cell sums.
#pragma once

#include <cuda_runtime.h>

namespace hymor {

struct __align__(8) ff {
  float h, l;
};

__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = a + b;
  return ff{s, b - (s - a)};
}

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return ff{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = ff_two_sum(a.h, b.h);
  return ff_fast_two_sum(s.h, s.l + (a.l + b.l));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = a.h * b.h;
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  return ff_fast_two_sum(p, e);
}

// acc + b x, with the product's high part exact (TwoProduct by FMA) and its cross terms
// joining the low part of the sum (the FMA-chain step of a float-float dot product)
__device__ __forceinline__ ff ff_fma(ff b, ff x, ff acc) {
  const float p = b.h * x.h;
  const float e = __fmaf_rn(b.h, x.l, __fmaf_rn(b.l, x.h, __fmaf_rn(b.h, x.h, -p)));
  return ff_add(acc, ff{p, e});
}

// y + b3 x3 + b2 x2 + b1 x1 + b0 x0 (in that order): each product's high part joins the
// running high part by TwoSum and its rounding error and cross terms join the low part,
// which is renormalised (TwoSum) once after the four. The loop-carried dependency is one
// addition on each part instead of a renormalisation per term; the low part's rounding
// over the four terms is ~2^-44 of the largest partial sum.
__device__ __forceinline__ ff ff_dot4(const ff* b, const ff* x, ff y) {
  float h = y.h, l = y.l;
#pragma unroll
  for (int e = 3; e >= 0; --e) {
    const float p = b[e].h * x[e].h;
    const float pe = __fmaf_rn(b[e].h, x[e].l, __fmaf_rn(b[e].l, x[e].h, __fmaf_rn(b[e].h, x[e].h, -p)));
    const float s = h + p;
    const float bb = s - h;
    l += ((h - (s - bb)) + (p - bb)) + pe;
    h = s;
  }
  return ff_two_sum(h, l);
}

// a * 2^k for a power of two: exact, no renormalisation
__device__ __forceinline__ ff ff_scale2(ff a, float p2) { return ff{a.h * p2, a.l * p2}; }

// 1 / b for b > 0 in the float normal range: Newton-Raphson from the hardware's float
// reciprocal y0 (rcp.approx, within one ulp), with the correction carried past float
// precision. e = 1 - b y0 is formed exactly to ~2^-48 (1 - p is exact since p = b.h y0 lies
// within 2^-22 of 1, and p + pe = b.h y0 exactly by the FMA), and 1 / b = y0 (1 + e + e^2
// + ...), whose cubic term is below 2^-69. Relative error ~2^-46.
__device__ __forceinline__ ff ff_rcp(ff b) {
  float y0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(b.h));
  const float p = b.h * y0;
  const float pe = __fmaf_rn(b.h, y0, -p);
  const float e = __fmaf_rn(-b.l, y0, (1.0f - p) - pe);
  return ff_fast_two_sum(y0, y0 * __fmaf_rn(e, e, e));
}

// double -> float-float: h is x with its 29 low mantissa bits cleared (an exact float),
// l the remaining 29 bits truncated to 24. |x| must lie in the float normal range; zero
// (and anything below 2^-126) gives zero.
__device__ __forceinline__ ff ff_from_double(double x) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const unsigned sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7ffu);
  const unsigned hb = sign | ((unsigned)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  const unsigned m = lw & 0x1fffffffu;
  const int p = 31 - __clz((int)m);                                // leading bit of m, -1 if m == 0
  const unsigned mant = p > 23 ? (m >> (p - 23)) : (m << (23 - p));
  const int el = e - 948 + p;                                      // biased float exponent of l
  const unsigned lb = sign | ((unsigned)el << 23) | (mant & 0x7fffffu);
  ff r;
  r.h = e > 896 ? __uint_as_float(hb) : 0.0f;
  r.l = (e > 896 && m != 0u && el > 0) ? __uint_as_float(lb) : 0.0f;
  return r;
}

// double -> float-float as ff_from_double, with non-finite values and values beyond the
// float range as NaN (the propagator's inputs and coefficients)
__device__ __forceinline__ ff ff_from_double_checked(double x) {
  const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
  return e >= 1151u ? ff{__int_as_float(0x7fc00000), 0.0f} : ff_from_double(x);
}

// exact float -> double widening of a normal float (or zero) through the bit pattern; an
// infinity or NaN widens to NaN
__device__ __forceinline__ double ff_widen(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned ef = (b >> 23) & 0xffu;
  const unsigned hw = (b & 0x80000000u) | (ef ? (((ef + 896u) << 20) | ((b & 0x7fffffu) >> 3)) : 0u);
  const unsigned lw = ef ? (b << 29) : 0u;
  return ef == 0xffu ? __longlong_as_double(0x7ff8000000000000LL) : __hiloint2double((int)hw, (int)lw);
}

// float-float -> double: one FP64 addition
__device__ __forceinline__ double ff_to_double(ff a) { return ff_widen(a.h) + ff_widen(a.l); }

}  // namespace hymor
