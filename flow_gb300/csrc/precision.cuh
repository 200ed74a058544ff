// precision.cuh -- arithmetic policies of the fused timestep kernels.
//
// Prec<double>: the FP64 form.  Comparisons and selections run on the IEEE
//   bit pattern with integer instructions; reciprocal and reciprocal square
//   root start from the MUFU approximation (fused_math.cuh).
// Prec<float>:  the bulk arithmetic of the mixed form.  FP32 compares are
//   full-rate, so the native operations are used; reciprocals are the MUFU
//   approximations.
//
// to_d / from_d convert bulk values to and from FP64.  For float they work on
// the bit patterns with integer instructions: on GB300 an F2F conversion
// occupies the FP64 pipe (about 1/64 of the FP32 rate), while the integer form
// costs a handful of full-rate instructions.  to_d is exact; from_d rounds to
// nearest-even; both flush values outside the normal float range to signed
// zero (FP64 subnormal range) -- the flow fields stay far inside it.
#pragma once

#include "fused_math.cuh"

namespace flow {

template <typename R>
struct Prec;

template <>
struct Prec<double> {
  static constexpr bool kMixed = false;
  // x is an exact zero whose arithmetic a tile may skip (the result is the
  // same number).  Worth it where FP64 instructions are the bound: every
  // such test, per lane.  zero_skip_coarse marks the few skips that remove
  // a whole flux or cell update.
  __device__ static __forceinline__ bool zero_skip(double x) { return d_is_zero(x); }
  __device__ static __forceinline__ bool zero_skip_coarse(double x) { return d_is_zero(x); }
  // A zero increment whose update is skipped together with its loads and
  // stores (a momentum that does not change is neither read nor written).
  __device__ static __forceinline__ bool zero_skip_mem(double x) { return d_is_zero(x); }
  __device__ static __forceinline__ bool is_zero(double x) { return d_is_zero(x); }
  __device__ static __forceinline__ bool gt0(double x) { return d_gt0(x); }
  __device__ static __forceinline__ bool ge0(double x) { return d_ge0(x); }
  __device__ static __forceinline__ bool same_sign_nz(double a, double b) {
    return ((dbits(a) ^ dbits(b)) >= 0) && !d_is_zero(a) && !d_is_zero(b);
  }
  __device__ static __forceinline__ double abs(double x) { return d_abs(x); }
  __device__ static __forceinline__ double min0(double x) { return d_min0(x); }
  __device__ static __forceinline__ double minmod(double a, double b) { return d_minmod(a, b); }
  __device__ static __forceinline__ double rcp(double x) { return d_rcp(x); }
  // A reciprocal used only through qdiv (which corrects the quotient).
  __device__ static __forceinline__ double rcp_q(double x) { return d_rcp_for_qdiv(x); }
  __device__ static __forceinline__ double rsqrt(double x) { return d_rsqrt(x); }
  __device__ static __forceinline__ double to_d(double x) { return x; }
  __device__ static __forceinline__ double from_d(double x) { return x; }
  // m - t*s and b + h*w with the product rounded before the sum, as the
  // reference evaluates them (no contraction into an FMA).
  __device__ static __forceinline__ double msub(double m, double t, double s) {
    return __dadd_rn(m, -__dmul_rn(t, s));
  }
  __device__ static __forceinline__ double madd(double h, double w, double b) {
    return __dadd_rn(__dmul_rn(h, w), b);
  }
  // n / d from an approximate reciprocal inv of d: one FMA correction step
  // gives the correctly rounded quotient except in rare ties.
  __device__ static __forceinline__ double qdiv(double n, double d, double inv) {
    const double q = n * inv;
    return fma(inv, fma(-d, q, n), q);
  }
  // n / d when the reciprocal is not needed otherwise.
  __device__ static __forceinline__ double div(double n, double d) { return d_div(n, d); }
  // m - t/d with the quotient rounded before the difference, as the
  // reference evaluates a momentum or mass update by a mesh spacing d.
  // kPow2: d is a power of two, so t*inv is already the exact quotient and
  // the correction (always zero then) is skipped.
  template <bool kPow2 = false>
  __device__ static __forceinline__ double dsub(double m, double t, double d, double inv) {
    return __dadd_rn(m, -(kPow2 ? d_mul_pow2(t, inv) : qdiv(t, d, inv)));
  }
  // x * p; kPow2: p is a power of two and the product an exponent add.
  template <bool kPow2 = false>
  __device__ static __forceinline__ double mulp(double x, double p) {
    return kPow2 ? d_mul_pow2(x, p) : x * p;
  }
  // x * 0.5 and x * 2, exact, on the integer pipes.
  __device__ static __forceinline__ double half(double x) { return d_half(x); }
  __device__ static __forceinline__ double neg(double x) { return d_neg(x); }
  __device__ static __forceinline__ double twice(double x) { return d_twice(x); }
};

__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u;
  const unsigned ex = (b >> 23) & 0xffu;
  if (ex == 0u) return __hiloint2double((int)sign, 0);
  const unsigned hi = sign | ((ex + 896u) << 20) | ((b & 0x7fffffu) >> 3);
  const unsigned lo = b << 29;
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float f64_to_f32(double x) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int ex = (int)((hi >> 20) & 0x7ffu) - 896;
  if (ex <= 0) return __uint_as_float(sign);
  if (ex >= 255) return __uint_as_float(sign | 0x7f800000u);
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  unsigned f = sign | ((unsigned)ex << 23) | mant;
  f += (rest > 0x10000000u) || (rest == 0x10000000u && (mant & 1u));
  return __uint_as_float(f);
}

template <>
struct Prec<float> {
  static constexpr bool kMixed = true;
  // The FP32 bulk is cheap and bound by issue latency, where branches cost
  // more than most skips save (measured: ~10% slower on fields in motion
  // everywhere).  Only the coarse skips remain, taken when every active lane
  // of the warp has the zero (a warp-uniform branch; each lane's own value
  // is zero then, so the skip is exact for each).
  __device__ static __forceinline__ constexpr bool zero_skip(float) { return false; }
  __device__ static __forceinline__ bool zero_skip_coarse(float x) {
    return __all_sync(__activemask(), x == 0.0f) != 0;
  }
  // Skips that save memory traffic (a momentum that does not change is
  // neither read nor written) are worth a warp vote here too.
  __device__ static __forceinline__ bool zero_skip_mem(float x) { return zero_skip_coarse(x); }
  __device__ static __forceinline__ bool is_zero(float x) { return x == 0.0f; }
  __device__ static __forceinline__ bool gt0(float x) { return x > 0.0f; }
  __device__ static __forceinline__ bool ge0(float x) { return x >= 0.0f; }
  __device__ static __forceinline__ bool same_sign_nz(float a, float b) {
    return (a > 0.0f && b > 0.0f) || (a < 0.0f && b < 0.0f);
  }
  __device__ static __forceinline__ float abs(float x) { return fabsf(x); }
  __device__ static __forceinline__ float min0(float x) { return (x > 0.0f) ? 0.0f : x; }
  __device__ static __forceinline__ float minmod(float a, float b) {
    if ((a > 0.0f && b > 0.0f) || (a < 0.0f && b < 0.0f)) {
      return (fabsf(a) < fabsf(b)) ? a : b;
    }
    return 0.0f;
  }
  __device__ static __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  __device__ static __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
  __device__ static __forceinline__ double to_d(float x) { return f32_to_f64(x); }
  __device__ static __forceinline__ float from_d(double x) { return f64_to_f32(x); }
  __device__ static __forceinline__ float msub(float m, float t, float s) { return fmaf(-t, s, m); }
  __device__ static __forceinline__ float madd(float h, float w, float b) { return fmaf(h, w, b); }
  __device__ static __forceinline__ float qdiv(float n, float, float inv) { return n * inv; }
  __device__ static __forceinline__ float rcp_q(float x) { return rcp(x); }
  __device__ static __forceinline__ float div(float n, float d) { return n * rcp(d); }
  template <bool kPow2 = false>
  __device__ static __forceinline__ float dsub(float m, float t, float, float inv) {
    return fmaf(-t, inv, m);
  }
  template <bool kPow2 = false>
  __device__ static __forceinline__ float mulp(float x, float p) { return x * p; }
  __device__ static __forceinline__ float half(float x) { return 0.5f * x; }
  __device__ static __forceinline__ float neg(float x) { return -x; }
  __device__ static __forceinline__ float twice(float x) { return x + x; }
};

}  // namespace flow
