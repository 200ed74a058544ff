// selftest.cu -- gb300_check_fp64_helpers: checks the integer-pipe and
// MUFU-based FP64 helpers of the fused kernels (fused_math.cuh) against the
// IEEE operations on this GPU, over hashed inputs.
#include <cstring>

#include "../../include/flow_gb300.h"
#include "fused_math.cuh"

namespace flow {
namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ bool same_value(double a, double b) {
  return (a != a && b != b) || dbits(a) == dbits(b);
}

// A normal double with a random mantissa, random sign and an exponent in
// [-60, 60].
__device__ __forceinline__ double normal_from(unsigned long long h) {
  const long long ex = 1023 - 60 + (long long)((h >> 52) % 121);
  return dfrom((long long)(h & 0x800fffffffffffffull) | (ex << 52));
}

__device__ __forceinline__ long long ulp_gap(double a, double b) {
  const long long d = dbits(a) - dbits(b);
  return d < 0 ? -d : d;
}

// counts[0] d_half != x*0.5, [1] d_twice != x*2 (all bit patterns, NaN = NaN),
// [2] d_is_pow2 wrong, [3] d_div != IEEE n/d, [4] d_rcp_for_qdiv + qdiv
// != IEEE n/d, [5] d_mul_pow2(x, 2^k) != x*2^k (all bit patterns of x, k in
// [-1022, 1023]); [6] the power-of-two quotients d_pow2_rcp, d_pow2_half_ratio,
// d_pow2_rcp_sq != 1/p, x/(2p), 1/(p*p) (exponents over the whole range); ulp[0], ulp[1] the largest gaps of [3], [4]; seed_err the
// largest |rcp.approx(d) d - 1| as FP64 bits.
__global__ void k_check(long long n, unsigned long long seed, unsigned long long* counts,
                        unsigned long long* ulp, unsigned long long* seed_err) {
  unsigned long long c[7] = {0, 0, 0, 0, 0, 0, 0}, u0 = 0, u1 = 0, se = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h = mix64(seed ^ mix64((unsigned long long)i));
    // Bias three eighths of the patterns to the exponent-field ends (zeros,
    // subnormals, the smallest normals, the largest finite values, inf, NaN).
    unsigned long long b = h;
    const unsigned sel = (unsigned)(mix64(h) & 7u);
    if (sel == 0) b &= 0x801fffffffffffffull;                       // exponent 0 or 1
    if (sel == 1) b |= 0x7fe0000000000000ull;                       // exponent 0x7fe / 0x7ff
    if (sel == 2) b &= 0x8000000000000001ull;                       // zeros, tiny subnormal
    const double x = dfrom((long long)b);
    if (!same_value(d_half(x), __dmul_rn(x, 0.5))) ++c[0];
    if (!same_value(d_twice(x), __dmul_rn(x, 2.0))) ++c[1];
    int e2 = 0;
    const double m = frexp(x, &e2);
    const bool p2 = x > 0.0 && x <= 1.7976931348623157e308 && m == 0.5 && e2 >= -1021;
    if (d_is_pow2(x) != p2) ++c[2];
    // A power of two: mostly moderate exponents, an eighth over the whole range.
    const unsigned long long hp = mix64(h + 3);
    const long long kp = (hp & 7u) ? (long long)((hp >> 3) % 121) - 60
                                   : (long long)((hp >> 3) % 2046) - 1022;
    const double pw = dfrom((kp + 1023) << 52);
    if (!same_value(d_mul_pow2(x, pw), __dmul_rn(x, pw))) ++c[5];
    const unsigned long long hq = mix64(h + 4);
    const long long kq = (hq & 7u) ? (long long)((hq >> 3) % 121) - 60
                                   : (long long)((hq >> 3) % 2046) - 1022;
    const double pq = dfrom((kq + 1023) << 52);
    if (!same_value(d_pow2_rcp(pw), __ddiv_rn(1.0, pw))) ++c[6];
    if (!same_value(d_pow2_half_ratio(pq, pw), __ddiv_rn(pq, __dmul_rn(2.0, pw)))) ++c[6];
    if (!same_value(d_pow2_rcp_sq(pw), __ddiv_rn(1.0, __dmul_rn(pw, pw)))) ++c[6];
    const double nn = normal_from(mix64(h + 1)), dd = normal_from(mix64(h + 2));
    const double q = __ddiv_rn(nn, dd);
    const double qa = d_div(nn, dd);
    const double r = d_rcp_for_qdiv(dd);
    const double qb = fma(r, fma(-dd, nn * r, nn), nn * r);
    if (dbits(qa) != dbits(q)) {
      ++c[3];
      const unsigned long long g = (unsigned long long)ulp_gap(qa, q);
      u0 = g > u0 ? g : u0;
    }
    if (dbits(qb) != dbits(q)) {
      ++c[4];
      const unsigned long long g = (unsigned long long)ulp_gap(qb, q);
      u1 = g > u1 ? g : u1;
    }
    double s;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(s) : "d"(dd));
    const double err = fabs(fma(s, dd, -1.0));
    const unsigned long long eb = (unsigned long long)dbits(err);
    se = eb > se ? eb : se;
  }
  for (int k = 0; k < 7; ++k) {
    if (c[k]) atomicAdd(&counts[k], c[k]);
  }
  atomicMax(&ulp[0], u0);
  atomicMax(&ulp[1], u1);
  atomicMax(seed_err, se);
}

}  // namespace
}  // namespace flow

extern "C" int gb300_check_fp64_helpers(long long n, unsigned long long seed,
                                        long long* counts, long long* max_ulp,
                                        double* max_seed_rel_err) {
  if (n <= 0 || !counts || !max_ulp || !max_seed_rel_err) return GB300_ERR_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 10 * sizeof(unsigned long long)) != cudaSuccess) return GB300_ERR_CUDA;
  cudaMemset(d, 0, 10 * sizeof(unsigned long long));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  flow::k_check<<<sms * 8, 256>>>(n, seed, d, d + 7, d + 9);
  unsigned long long h[10];
  cudaError_t err = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err != cudaSuccess) return GB300_ERR_CUDA;
  for (int k = 0; k < 7; ++k) counts[k] = (long long)h[k];
  max_ulp[0] = (long long)h[7];
  max_ulp[1] = (long long)h[8];
  double e;
  memcpy(&e, &h[9], sizeof(e));
  *max_seed_rel_err = e;
  return GB300_OK;
}
