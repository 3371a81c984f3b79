// fp64_int.cuh -- IEEE-754 binary64 square root, division and comparisons,
// round to nearest even, computed on the integer pipes.
//
// GB300 executes 2 FP64 operations per SM per clock (one warp instruction
// holds an SM sub-partition's FP64 pipe for 64 cycles), against 64 integer
// operations per SM per clock.  The hardware's correctly rounded sqrt and
// division are sequences of ~10 and ~7 FP64-pipe operations; the force law
// needs 7 of each per contact and is FP64-pipe bound with most issue slots
// idle.  The versions here take an FP32 seed, refine it in 64-bit fixed point
// and settle the last bit with an exact integer rounding test, so they run
// beside the FP64 pipe instead of on it.  Results are bit-identical to the
// hardware's __dsqrt_rn / __ddiv_rn for every input: normal operands and zeros
// take the integer path; subnormal, infinite and NaN operands, and results
// outside the normal range, take the hardware instruction.  (Plain additions
// and multiplications stay on the FP64 pipe: one instruction there beats the
// ~30-40 integer instructions of an exact emulation, measured on GB300.)
//
// The functions are __host__ __device__ so that the CPU tests compare them
// with the host's IEEE arithmetic on billions of operands, including exact
// squares and quotients, ties, exponent extremes and deliberately degraded
// seeds.
#pragma once
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline __attribute__((always_inline))
#endif

namespace fpi {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kMant = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kHid = 0x0010000000000000ull;

__host__ __device__ __forceinline__ uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
__host__ __device__ __forceinline__ double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ uint64_t mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
__host__ __device__ __forceinline__ int clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}
// the hardware operation, for the rare operands the integer path leaves out
__host__ __device__ __forceinline__ double hw_mul(double x, double y) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(x, y);
#else
  return x * y;
#endif
}

__host__ __device__ __forceinline__ double hw_sqrt(double x) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(x);
#else
  return __builtin_sqrt(x);
#endif
}
__host__ __device__ __forceinline__ double hw_div(double x, double y) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(x, y);
#else
  return x / y;
#endif
}
__host__ __device__ __forceinline__ uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ float ffrom(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}
// single-precision seeds: ~22 correct bits are all the refinement needs
__host__ __device__ __forceinline__ float rsqrt_seed(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  float r = 1.0f / __builtin_sqrtf(x);
#ifdef FPI_HOST_SEED_HOOK
  r = FPI_HOST_SEED_HOOK(r);
#endif
  return r;
#endif
}
__host__ __device__ __forceinline__ float rcp_seed(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  float r = 1.0f / x;
#ifdef FPI_HOST_SEED_HOOK
  r = FPI_HOST_SEED_HOOK(r);
#endif
  return r;
#endif
}
__host__ __device__ __forceinline__ int64_t smulhi(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * b) >> 64);
#endif
}
// Q2.62 fixed point: value * 2^62 in a 64-bit word (values below 4)
__host__ __device__ __forceinline__ uint64_t q62_from_seed(float r) {
  // r = 1.m * 2^k, k in [-3, 1]: (2^23 + m) * 2^(39 + k) = r * 2^62
  const uint32_t rb = fbits(r);
  const int k = (int)(rb >> 23) - 127;
  return ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u)) << (39 + k);
}

// sqrt(x), correctly rounded.  Positive normal x take the integer path:
// x = M * 2^(2h) with M in [1, 4); a single-precision seed of 1/sqrt(M) is
// refined by two coupled Newton (Goldschmidt) steps in Q3.61 fixed point,
// g -> sqrt(M), h -> 1/(2 sqrt(M)), residual d = 1/2 - g*h (Goldschmidt,
// 1964; Markstein, IBM J. Res. Dev. 34(1), 1990), which leave g within a
// few 2^-58 of sqrt(M).  The candidate S = round(g * 2^52) is then settled by
// the exact integer test of round-to-nearest, S^2 - S < M*2^104 <= S^2 + S,
// and moved by one unit while it fails.  Other x take the hardware sqrt.
__host__ __device__ __forceinline__ double sqrt_rn(double x) {
  const uint64_t u = bits(x);
  const uint32_t e = (uint32_t)(u >> 52);      // the sign bit makes negatives large
  if (e - 1u >= 2046u) {
    if ((u << 1) == 0) return x;               // sqrt(+-0) = +-0
    return hw_sqrt(x);
  }
  const uint64_t f = u & kMant;
  const int E = (int)e - 1023;
  const uint32_t odd = (uint32_t)E & 1u;
  const uint64_t A = ((f | kHid) << 10) << odd;            // M in Q2.62
  const float fm = ffrom(((127u + odd) << 23) | (uint32_t)(f >> 29));
  const uint64_t R0 = q62_from_seed(rsqrt_seed(fm));       // ~1/sqrt(M), Q2.62
  // g and h in Q3.61: sqrt(M) reaches 2, and a seed error must not overflow
  int64_t g = (int64_t)(mulhi(A, R0) << 1);                 // ~sqrt(M)
  int64_t hh = (int64_t)(R0 >> 2);                          // ~1/(2 sqrt(M))
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const int64_t p = (int64_t)(mulhi((uint64_t)g, (uint64_t)hh) << 3);
    const int64_t d = ((int64_t)1 << 60) - p;
    g += (int64_t)((uint64_t)smulhi(g, d) << 3);
    hh += (int64_t)((uint64_t)smulhi(hh, d) << 3);
  }
  uint64_t S = ((uint64_t)g + (1u << 8)) >> 9;              // ~sqrt(M) * 2^52
  // D = M*2^104 - S^2, exact in 64 bits while S is within a few units
  const uint64_t Nlo = A << 42;
  int64_t D = (int64_t)(Nlo - S * S);
#pragma unroll
  for (int it = 0; it < 2; it++) {
    if (D > (int64_t)S) { D -= (int64_t)(2 * S + 1); S += 1; }
    else if (D <= -(int64_t)S) { D += (int64_t)(2 * S - 1); S -= 1; }
  }
  const int er = ((E - (int)odd) >> 1) + 1023;
  return from_bits((((uint64_t)(er - 1)) << 52) + S);
}

// x / y, correctly rounded.  Normal x and y with a normal quotient take the
// integer path: the significand ratio Q = (mx/my) * 2^k in [1, 2) comes from a
// single-precision seed of 1/my refined by two Newton steps in Q2.62
// (z <- z + z*(1 - my*z)), the candidate S = round(Q * 2^52) is settled by the
// exact remainder R = mx*2^(52+k) - S*my (round to nearest: |R| <= my/2, ties
// to the even S) and moved by one unit while the test fails.  Zeros,
// subnormals, infinities, NaNs and quotients outside the normal range take
// the hardware division.  The refined reciprocal depends on y only, so
// several quotients by one divisor share it (Divisor).
struct Divisor {
  double y;
  uint64_t mb;    // significand of y, [2^52, 2^53)
  int64_t z;      // ~1/my in Q2.62
  uint32_t eb;    // biased exponent of y
  bool normal;
};

__host__ __device__ __forceinline__ Divisor divisor(double y) {
  Divisor v;
  v.y = y;
  const uint64_t b = bits(y);
  v.eb = (uint32_t)(b >> 52) & 0x7FFu;
  v.normal = v.eb - 1u < 2046u;
  v.mb = (b & kMant) | kHid;
  const uint64_t B = v.mb << 10;                           // my in Q2.62, [1, 2)
  const float fb = ffrom((127u << 23) | (uint32_t)((v.mb & kMant) >> 29));
  int64_t z = (int64_t)q62_from_seed(rcp_seed(fb));
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const int64_t t = ((int64_t)1 << 62) - (int64_t)(mulhi(B, (uint64_t)z) << 2);   // 1 - my*z
    z += (int64_t)((uint64_t)smulhi(z, t) << 2);
  }
  v.z = z;
  return v;
}

__host__ __device__ __forceinline__ double div_by(double x, const Divisor& v) {
  const uint64_t a = bits(x);
  const uint32_t ea = (uint32_t)(a >> 52) & 0x7FFu;
  if (ea - 1u >= 2046u || !v.normal) {
    if ((a << 1) == 0 && v.normal) return from_bits((a ^ bits(v.y)) & kSign);   // +-0 / normal
    return hw_div(x, v.y);
  }
  const uint64_t ma = (a & kMant) | kHid, mb = v.mb;
  const uint32_t k = ma < mb ? 1u : 0u;                    // Q = ma*2^k/mb in [1, 2)
  const int eq = (int)ea - (int)v.eb + 1023 - (int)k;
  if (eq < 1 || eq > 2046) return hw_div(x, v.y);
  const uint64_t Aq = (ma << 10) << k;                     // mx*2^k in Q2.62 (below 4)
  const uint64_t q = mulhi(Aq, (uint64_t)v.z) << 2;        // ~Q in Q2.62
  uint64_t S = (q + (1u << 9)) >> 10;                      // ~Q * 2^52
  // R = ma*2^(52+k) - S*mb, exact in 64 bits while S is within a few units
  int64_t R = (int64_t)(((ma << 52) << k) - S * mb);
  const int64_t hb = (int64_t)mb;
#pragma unroll
  for (int it = 0; it < 2; it++) {
    if (2 * R > hb || (2 * R == hb && (S & 1u))) { R -= hb; S += 1; }
    else if (2 * R < -hb || (2 * R == -hb && (S & 1u))) { R += hb; S -= 1; }
  }
  const uint64_t sg = (a ^ bits(v.y)) & kSign;
  return from_bits(sg | ((((uint64_t)(eq - 1)) << 52) + S));
}

__host__ __device__ __forceinline__ double div_rn(double x, double y) { return div_by(x, divisor(y)); }

// IEEE comparisons on the integer pipes (false with a NaN; +0 == -0): the
// bit patterns, with the magnitude bits of negatives flipped, order like the
// values.
__host__ __device__ __forceinline__ int64_t order_key(uint64_t u) {
  return (int64_t)(u ^ ((uint64_t)((int64_t)u >> 63) >> 1));
}
__host__ __device__ __forceinline__ bool unordered_or_zeros(uint64_t a, uint64_t b) {
  const uint64_t aa = a << 1, bb = b << 1;     // magnitudes, shifted out sign
  return aa > 0xFFE0000000000000ull || bb > 0xFFE0000000000000ull || (aa | bb) == 0;
}
__host__ __device__ __forceinline__ bool gt(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  return !unordered_or_zeros(a, b) && order_key(a) > order_key(b);
}
__host__ __device__ __forceinline__ bool lt(double x, double y) { return gt(y, x); }
__host__ __device__ __forceinline__ bool ge(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  const uint64_t aa = a << 1, bb = b << 1;
  if (aa > 0xFFE0000000000000ull || bb > 0xFFE0000000000000ull) return false;   // NaN
  if ((aa | bb) == 0) return true;                                                // +-0 >= +-0
  return order_key(a) >= order_key(b);
}
__host__ __device__ __forceinline__ bool le(double x, double y) { return ge(y, x); }

// floor(q) as an int when 0 <= floor(q) < n (q = -0 counts as 0), else -1;
// NaN and infinities give -1.  Integer work only.
__host__ __device__ __forceinline__ int floor_in_range(double q, int n) {
  const uint64_t u = bits(q);
  if ((u << 1) == 0) return n > 0 ? 0 : -1;
  if (u >> 63) return -1;                        // negative
  const uint32_t e = (uint32_t)(u >> 52);
  if (e < 1023u) return n > 0 ? 0 : -1;          // 0 < q < 1
  if (e > 1023u + 30u) return -1;                // >= 2^31, infinity, NaN
  const uint64_t v = ((u & kMant) | kHid) >> (1075u - e);
  return v < (uint64_t)n ? (int)v : -1;
}

// (q - k) in Q1.31, truncated, for the quotient q >= 0 and its floor k
// (0 <= k < 2^31).
__host__ __device__ __forceinline__ int32_t frac31(double q, int k) {
  const uint64_t u = bits(q);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7FFu;
  const uint64_t m = (u & kMant) | (e ? kHid : 0ull);
  const int s = (e ? (int)e : 1) - 1023 - 20;    // q * 2^32 = m * 2^s, s <= 10
  const uint64_t qf = s >= 0 ? (m << s) : (s > -64 ? (m >> -s) : 0ull);
  return (int32_t)((qf - ((uint64_t)k << 32)) >> 1);
}

// floor(x / y) of the IEEE quotient as an int in [0, n), else -1 (as
// floor_in_range of div_by), and where x / y lies inside that unit: off31 =
// (x/y - floor) in Q1.31, within 2^-29 (an estimate for single-precision
// copies, not part of the exact result).  Fast path (positive normal x and y,
// quotient below 2^27): the quotient in Q32.32 from the divisor's reciprocal,
// error below 2^-30; the rounded quotient differs from the exact one by less
// than q*2^-53 < 2^-26, so when the estimate is at least 2^-20 from an integer
// both have the floor of the estimate.  Other operands, and estimates inside
// that band, take the exact division.
__host__ __device__ __forceinline__ int floor_div(double x, const Divisor& v, int n, int32_t& off31) {
  const uint64_t a = bits(x);
  const uint32_t ea = (uint32_t)(a >> 52);     // the sign bit makes negatives large
  const int sh = (int)ea - (int)v.eb;          // x/y = (mx/my) * 2^sh
  if (ea - 1u < 2046u && v.normal && (bits(v.y) >> 63) == 0 && sh <= 26) {
    const uint64_t ma = (a & kMant) | kHid;
    const uint64_t r61 = mulhi(ma << 11, (uint64_t)v.z);   // mx/my in Q3.61
    const int rs = 29 - sh;
    const uint64_t qf = rs >= 64 ? 0ull : (r61 >> rs);     // ~x/y in Q32.32
    const uint32_t fr = (uint32_t)qf;
    if (fr >= (1u << 12) && fr <= 0xFFFFFFFFu - (1u << 12)) {
      off31 = (int32_t)(fr >> 1);
      const uint64_t k = qf >> 32;
      return k < (uint64_t)n ? (int)k : -1;
    }
  }
  const double q = div_by(x, v);
  const int k = floor_in_range(q, n);
  off31 = k >= 0 ? frac31(q, k) : 0;
  return k;
}

// A single-precision copy of x for estimates: truncated (relative error below
// 2^-23) from the bits for normal x in the float range, else converted.
__host__ __device__ __forceinline__ float to_float_trunc(double x) {
  const uint64_t u = bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7FFu;
  if (e - 897u < 254u)   // 2^-126 <= |x| < 2^128
    return ffrom((uint32_t)(u >> 63) << 31 | (e - 896u) << 23 | (uint32_t)((u & kMant) >> 29));
  return (float)x;
}

// x * (-0.5), exact for every x whose half is a normal number or zero: the
// exponent field drops by one and the sign flips.  Subnormal halves (which
// round), infinities and NaNs take the hardware multiplication.
__host__ __device__ __forceinline__ double mul_neg_half(double x) {
  const uint64_t u = bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7FFu;
  if (e - 2u < 2045u) return from_bits((u - (1ull << 52)) ^ kSign);
  if ((u << 1) == 0) return from_bits(u ^ kSign);
  return hw_mul(x, -0.5);
}

}  // namespace fpi
