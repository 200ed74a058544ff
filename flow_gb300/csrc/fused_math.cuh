// fused_math.cuh -- FP64 helpers of the fused timestep, shaped for GB300.
//
// On GB300 the FP64 pipe issues ~1.7 instructions per clock per SM, about
// 1/64 of the FP32 rate, while integer ALUs run at FP32-like rates.  DSETP
// comparisons occupy the FP64 pipe too.  So every comparison, sign test,
// absolute value, minimum and minmod selection here works on the IEEE bit
// pattern with integer instructions, and reciprocals / reciprocal square roots
// start from the MUFU approximation and finish with FMA Newton steps instead
// of the full IEEE division and square-root sequences.
//
// Semantics match the IEEE operations they replace for every finite input
// (including signed zeros); NaN inputs are not given IEEE ordering.
#pragma once

#include <cstdint>

namespace flow {

// Bit casts written as inline PTX moves, which the compiler cannot see
// through: with the plain intrinsics it folds integer tests such as
// "bits << 1 == 0" or "bits & ~sign" back into FP64 compares (DSETP) and
// absolute values, which occupy the FP64 pipe again.
__device__ __forceinline__ long long dbits(double x) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
__device__ __forceinline__ double dfrom(long long b) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(b));
  return x;
}
__device__ __forceinline__ int dhi(double x) { return (int)(dbits(x) >> 32); }
__device__ __forceinline__ int dlo(double x) { return (int)dbits(x); }
__device__ __forceinline__ double dfrom2(int hi, int lo) {
  double x;
  asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
  return x;
}
// -x with an integer instruction.
__device__ __forceinline__ double d_neg(double x) {
  return dfrom2(dhi(x) ^ (int)0x80000000, dlo(x));
}

__device__ __forceinline__ bool d_is_zero(double x) { return (dbits(x) << 1) == 0; }
// x > 0.0
__device__ __forceinline__ bool d_gt0(double x) { return dbits(x) > 0; }
// x < 0.0 (negative zero is not negative)
__device__ __forceinline__ bool d_lt0(double x) {
  const long long b = dbits(x);
  return b < 0 && (b << 1) != 0;
}
// x >= 0.0 (true for -0.0)
__device__ __forceinline__ bool d_ge0(double x) { return !d_lt0(x); }
__device__ __forceinline__ double d_abs(double x) {
  return dfrom(dbits(x) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double d_neg_if(double x, bool neg) {
  return dfrom(dbits(x) ^ (neg ? (long long)0x8000000000000000ULL : 0LL));
}
// min(0.0, x) with the ordinary-minimum rule (first argument when smaller):
// 0.0 when x > 0, else x itself.
__device__ __forceinline__ double d_min0(double x) { return d_gt0(x) ? 0.0 : x; }
// Minimum of two non-negative values (bit patterns order like the values).
__device__ __forceinline__ double d_min_pos(double a, double b) {
  return (dbits(a) < dbits(b)) ? a : b;
}
// Slope limiter: the smaller-magnitude argument when both are non-zero with
// the same sign (the second on a tie), else +0.0.
__device__ __forceinline__ double d_minmod(double a, double b) {
  const long long ia = dbits(a), ib = dbits(b);
  const bool same = ((ia ^ ib) >= 0) && ((ia << 1) != 0) && ((ib << 1) != 0);
  const unsigned long long ma = (unsigned long long)ia & 0x7fffffffffffffffULL;
  const unsigned long long mb = (unsigned long long)ib & 0x7fffffffffffffffULL;
  return same ? ((ma < mb) ? a : b) : 0.0;
}

// x * 0.5 and x * 2 on the integer pipes, with the IEEE result for every
// input (zeros, subnormals, overflow to infinity, infinities and NaNs kept).
// For a normal x away from the range ends only the exponent field of the
// high word changes; at the low end the magnitude bits are linear in the
// value (exponent fields 0 and 1), so halving is a rounded shift.
__device__ __forceinline__ double d_half(double x) {
  const int hi = dhi(x);
  const unsigned ex = (unsigned)hi & 0x7ff00000u;
  if (ex - 0x00200000u < 0x7ff00000u - 0x00200000u) {
    return dfrom2(hi - 0x00100000, dlo(x));
  }
  const long long b = dbits(x);
  const long long mag = b & 0x7fffffffffffffffLL;
  if (mag >= 0x7ff0000000000000LL) return x;
  const long long h = (mag >> 1) + (mag & (mag >> 1) & 1);  // round half to even
  return dfrom((b ^ mag) | h);
}
__device__ __forceinline__ double d_twice(double x) {
  const int hi = dhi(x);
  const unsigned ex = (unsigned)hi & 0x7ff00000u;
  if (ex - 0x00100000u < 0x7fe00000u - 0x00100000u) {
    return dfrom2(hi + 0x00100000, dlo(x));
  }
  const long long b = dbits(x);
  const long long mag = b & 0x7fffffffffffffffLL;
  const long long sign = b ^ mag;
  if (ex == 0u) return dfrom(sign | (mag << 1));
  if (ex == 0x7fe00000u) return dfrom(sign | 0x7ff0000000000000LL);
  return x;
}
// x * p for p a positive normal power of two (an exact reciprocal of a
// power-of-two mesh spacing): an add to the exponent field when x and the
// result are normal, x itself for a zero; the rare rest (subnormal input or
// result, overflow, infinity, NaN) takes the FP64 multiply in a called
// function, so the common path issues no FP64 instruction.
static __device__ __noinline__ double d_mul_slow(double x, double p) { return __dmul_rn(x, p); }
__device__ __forceinline__ double d_mul_pow2(double x, double p) {
  const int hx = dhi(x);
  const int k = ((dhi(p) >> 20) & 0x7ff) - 1023;
  const int ex = (hx >> 20) & 0x7ff;
  if ((unsigned)(ex - 1) < 2046u && (unsigned)(ex + k - 1) < 2046u) {
    return dfrom2((int)((unsigned)hx + ((unsigned)k << 20)), dlo(x));
  }
  if ((dbits(x) << 1) == 0) return x;
  return d_mul_slow(x, p);
}
// True for a positive normal power of two (an exactly invertible spacing).
__device__ __forceinline__ bool d_is_pow2(double x) {
  const long long b = dbits(x);
  const unsigned ex = (unsigned)(b >> 52);  // sign bit lands above the field
  return (b & 0x000fffffffffffffLL) == 0 && ex - 1u < 0x7feu;
}
// r * e is exact and r * e / r gives e back: r a positive normal power of
// two, e a zero or a normal number whose product with r is normal (tests on
// the bit patterns, no FP64 instruction).
__device__ __forceinline__ bool d_pow2_product_exact(double r, double e) {
  const long long eb = dbits(e);
  const int ee = (int)((eb >> 52) & 0x7ff);
  const int ex = ee + (int)((dbits(r) >> 52) & 0x7ff) - 1023;
  return d_is_pow2(r) & (((eb << 1) == 0) | ((ee != 0) & (ee != 0x7ff) & (ex >= 1) & (ex <= 2046)));
}

// Quotients of powers of two, for the spacing factors of power-of-two
// meshes: 1/y, x/(2y) and 1/(y*y) with x, y positive normal powers of two.
// The quotient is a power of two itself, so when it is a normal number it
// is formed exactly from the exponent fields on the integer pipes (the IEEE
// quotient is that same number); otherwise the IEEE expression is evaluated
// in a called function.
static __device__ __noinline__ double d_pow2_quot_slow(double x, double y, int form) {
  if (form == 1) return x / (2.0 * y);
  if (form == 2) return 1.0 / (y * y);
  return 1.0 / y;
}
__device__ __forceinline__ int d_exp_field(double x) { return (dhi(x) >> 20) & 0x7ff; }
// 1/y
__device__ __forceinline__ double d_pow2_rcp(double y) {
  const int f = 2046 - d_exp_field(y);
  if ((unsigned)(f - 1) < 2046u) return dfrom2(f << 20, 0);
  return d_pow2_quot_slow(1.0, y, 0);
}
// x / (2 y)  (2 y must not overflow, as it is formed first)
__device__ __forceinline__ double d_pow2_half_ratio(double x, double y) {
  const int ey = d_exp_field(y);
  const int f = d_exp_field(x) - ey + 1022;
  if ((unsigned)(f - 1) < 2046u && ey < 2046) return dfrom2(f << 20, 0);
  return d_pow2_quot_slow(x, y, 1);
}
// 1 / (y * y)
__device__ __forceinline__ double d_pow2_rcp_sq(double y) {
  const int f = 3069 - 2 * d_exp_field(y);
  if ((unsigned)(f - 1) < 2046u) return dfrom2(f << 20, 0);
  return d_pow2_quot_slow(1.0, y, 2);
}

// 1/x for finite normal non-zero x: MUFU seed, two Newton-Raphson steps.
__device__ __forceinline__ double d_rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}
// 1/x to ~2^-40 (one Newton step on the MUFU seed) for a reciprocal that is
// only ever used through a residual-corrected quotient (qdiv), which is then
// still correctly rounded: the correction squares the error.
__device__ __forceinline__ double d_rcp_for_qdiv(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return fma(r, fma(-x, r, 1.0), r);
}
// n/d for finite normal non-zero d when 1/d itself is not needed: one Newton
// step on the MUFU seed (relative error ~2^-20 measured -> ~2^-40), the
// quotient from it, and one residual correction q + r (n - d q) (-> ~2^-80):
// the correctly rounded quotient except in vanishingly rare near-ties, as
// d_rcp followed by qdiv gives, in 5 FP64 instructions instead of 7.
__device__ __forceinline__ double d_div(double n, double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  r = fma(r, fma(-d, r, 1.0), r);
  const double q = n * r;
  return fma(r, fma(-d, q, n), q);
}
// 1/sqrt(x) for finite normal positive x: MUFU seed, two Newton steps on
// r <- r + r*(0.5 - 0.5*x*r*r).
__device__ __forceinline__ double d_rsqrt(double x) {
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double h = d_half(x);
  double t = fma(-h * r, r, 0.5);
  r = fma(r, t, r);
  t = fma(-h * r, r, 0.5);
  return fma(r, t, r);
}

// Writes the value of interior point (ii, jj) of a w x h array into each of
// its ghost mirror images (pad layers per side): column images negated when
// flip_x, row images when flip_y, corner images by both.  This reproduces the
// reflective fill of every ghost point whose mirror source is (ii, jj).
__device__ __forceinline__ void mirror_store(double* a, int w, int h, int pad,
                                             int ii, int jj, double val,
                                             bool flip_x, bool flip_y) {
  int mc[2], mr[2];
  int nc = 0, nr = 0;
  if (jj < 2 * pad) mc[nc++] = 2 * pad - 1 - jj;
  if (jj >= w - 2 * pad) mc[nc++] = 2 * (w - pad) - 1 - jj;
  if (ii < 2 * pad) mr[nr++] = 2 * pad - 1 - ii;
  if (ii >= h - 2 * pad) mr[nr++] = 2 * (h - pad) - 1 - ii;
  if (nc == 0 && nr == 0) return;
  const double vx = flip_x ? -val : val;
  const double vy = flip_y ? -val : val;
  const double vxy = flip_x ? -vy : vy;
  for (int k = 0; k < nc; ++k) a[(size_t)ii * w + mc[k]] = vx;
  for (int r = 0; r < nr; ++r) {
    a[(size_t)mr[r] * w + jj] = vy;
    for (int k = 0; k < nc; ++k) a[(size_t)mr[r] * w + mc[k]] = vxy;
  }
}

}  // namespace flow
