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

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double dfrom(long long b) { return __longlong_as_double(b); }

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

// 1/x for finite normal non-zero x: MUFU seed, two Newton-Raphson steps.
__device__ __forceinline__ double d_rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}
// 1/sqrt(x) for finite normal positive x: MUFU seed, two Newton steps on
// r <- r + r*(0.5 - 0.5*x*r*r).
__device__ __forceinline__ double d_rsqrt(double x) {
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double h = 0.5 * x;
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
