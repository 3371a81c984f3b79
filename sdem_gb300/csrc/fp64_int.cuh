// fp64_int.cuh -- IEEE-754 binary64 addition and multiplication, round to
// nearest even, computed on the integer pipes.
//
// GB300 executes 2 FP64 operations per SM per clock (one warp instruction
// holds an SM sub-partition's FP64 pipe for 64 cycles), against 64 integer
// operations per SM per clock.  The force and integration kernels are
// FP64-pipe bound with most issue slots idle, so a share of their additions
// and multiplications is computed here, from the operands' bit patterns, while
// the FP64 pipe works on the rest.  Results are bit-identical to the hardware's
// __dadd_rn / __dmul_rn for every input: normal operands and zeros take the
// integer path; subnormal, infinite and NaN operands, and results that
// overflow or fall below the normal range, take the hardware instruction.
//
// Method: the textbook sign-magnitude algorithms of IEEE 754-2019 section 6
// (alignment with guard and sticky bits, normalisation, round to nearest even
// by the round bit and the sticky OR of the bits below it; e.g. Muller et al.,
// Handbook of Floating-Point Arithmetic, 2nd ed., ch. 7-8).  The functions are
// __host__ __device__ so that the CPU tests compare them with the host's IEEE
// arithmetic on hundreds of millions of operand pairs, including ties,
// cancellations and exponent extremes.
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
__host__ __device__ __forceinline__ double hw_add(double x, double y) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(x, y);
#else
  return x + y;
#endif
}
__host__ __device__ __forceinline__ double hw_mul(double x, double y) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(x, y);
#else
  return x * y;
#endif
}

// x * y, rounded to nearest even.
__host__ __device__ __forceinline__ double mul(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  const uint32_t ea = (uint32_t)(a >> 52) & 0x7FFu, eb = (uint32_t)(b >> 52) & 0x7FFu;
  const uint64_t s = (a ^ b) & kSign;
  if (ea - 1u >= 2046u || eb - 1u >= 2046u) {
    // a zero times a finite number is a signed zero; everything else special
    // (subnormal, infinity, NaN) goes to the hardware
    const bool za = (a << 1) == 0, zb = (b << 1) == 0;
    if ((za && eb != 0x7FFu) || (zb && ea != 0x7FFu)) return from_bits(s);
    return hw_mul(x, y);
  }
  // significands: ma in [2^63, 2^64) (shifted left by 11), mb in [2^52, 2^53);
  // the product P * 2^11 = hi * 2^64 + lo with hi in [2^51, 2^53)
  const uint64_t ma = ((a & kMant) | kHid) << 11;
  const uint64_t mb = (b & kMant) | kHid;
  const uint64_t hi = mulhi(ma, mb);
  const uint64_t lo = ma * mb;
  // e: biased exponent of the result before rounding
  int e = (int)(ea + eb) - 1023;
  uint64_t m, rb, st;
  if (hi >> 52) {          // product in [2^105, 2^106): one more binade
    e += 1;
    m = hi;
    rb = lo >> 63;
    st = (lo << 1) != 0;
  } else {
    m = (hi << 1) | (lo >> 63);
    rb = (lo >> 62) & 1u;
    st = (lo << 2) != 0;
  }
  if (e < 1 || e > 2046) return hw_mul(x, y);   // overflow or subnormal result
  // m in [2^52, 2^53) carries the hidden bit: adding it to (e-1) << 52 sets the
  // exponent field to e; a rounding carry to 2^53 moves to the next binade
  // (or to infinity from e = 2046, which is the correct overflow)
  const uint64_t inc = rb & (st | (m & 1u));
  return from_bits(s | ((((uint64_t)(e - 1)) << 52) + m + inc));
}

// x + y, rounded to nearest even.
__host__ __device__ __forceinline__ double add(double x, double y) {
  uint64_t a = bits(x), b = bits(y);
  uint64_t aa = a & ~kSign, bb = b & ~kSign;
  if (aa < bb) {  // |a| >= |b| from here on
    const uint64_t t = a; a = b; b = t;
    const uint64_t u = aa; aa = bb; bb = u;
  }
  const uint32_t ea = (uint32_t)(aa >> 52), eb = (uint32_t)(bb >> 52);
  if (ea - 1u >= 2046u || eb == 0u) {
    if (bb == 0) {
      if (aa == 0) return from_bits(a & b & kSign);   // (+-0) + (+-0): -0 only for -0 + -0
      if (ea != 0x7FFu && ea != 0u) return from_bits(a);   // x + (+-0) = x
    }
    return hw_add(x, y);   // subnormal, infinity, NaN
  }
  const bool sub = ((a ^ b) & kSign) != 0;
  // significands with 10 guard bits: [2^62, 2^63)
  const uint64_t ma = ((aa & kMant) | kHid) << 10;
  uint64_t mb = ((bb & kMant) | kHid) << 10;
  const uint32_t d = ea - eb;
  uint64_t inexact = 0;
  if (d > 63u) {
    inexact = 1;
    mb = 0;
  } else if (d > 0u) {
    inexact = (mb << (64u - d)) != 0;
    mb >>= d;
  }
  // exact value = m + f, 0 <= f < 1 (in units of bit 0), f > 0 iff inexact
  uint64_t m = sub ? (ma - mb - inexact) : (ma + mb);
  if (m == 0) return from_bits(0);   // exact cancellation: +0
  int e = (int)ea;
  uint64_t st = inexact;
  if (m >> 63) {            // carry out of the addition
    st |= m & 1u;
    m >>= 1;
    e += 1;
  } else {
    const int lz = clz64(m) - 1;   // bring the leading bit to position 62
    m <<= lz;
    e -= lz;
  }
  if (e < 1 || e > 2046) return hw_add(x, y);   // overflow or subnormal result
  const uint64_t rb = (m >> 9) & 1u;
  st |= (m & 0x1FFu) != 0;
  const uint64_t q = m >> 10;     // [2^52, 2^53), hidden bit included
  const uint64_t inc = rb & (st | (q & 1u));
  return from_bits((a & kSign) | ((((uint64_t)(e - 1)) << 52) + q + inc));
}

__host__ __device__ __forceinline__ double sub(double x, double y) { return add(x, from_bits(bits(y) ^ kSign)); }

}  // namespace fpi
