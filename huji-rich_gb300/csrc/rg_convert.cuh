// rg_convert.cuh -- float <-> double conversions and double comparisons on
// the integer pipe.
//
// GB300 issues FP64-pipe instructions, the float <-> double conversions and
// the double comparisons included, at about one per clock per SM against 64
// per clock for integer ones, and its FP64 kernels leave most issue slots
// idle.  The kernels that convert or compare many values (the FP32 copies of
// the per-mesh geometry, the FP32-mixed update, the FP64 limiter's tests and
// its FP32 screening) form the results from the IEEE-754 bit patterns
// instead, with the same results as the hardware instruction for every
// input, the orderings of the FP64 limiter's extrema and thresholds
// included.  Host-compilable, so the same code is checked against the C
// casts and operators on the CPU.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#define RG_CONV_FN static inline
#else
#define RG_CONV_FN __host__ __device__ __forceinline__
#endif

namespace rg {

RG_CONV_FN uint64_t conv_dbits(double x) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
RG_CONV_FN uint32_t conv_fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
RG_CONV_FN float conv_float(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
RG_CONV_FN double conv_double_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(u));
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}
RG_CONV_FN double conv_double(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
#else
  const uint64_t u = (static_cast<uint64_t>(hi) << 32) | lo;
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}

// double -> float rounded to nearest, ties to even: static_cast<float>(x)
// for every x.  Results in the normal float range and zeros are formed on
// the integer pipe (the 29 dropped significand bits decide the rounding; a
// carry out of the significand raises the exponent, and out of the largest
// exponent gives the infinity the rounding calls for); subnormal results,
// infinities and NaNs take the hardware conversion.
RG_CONV_FN float narrow(double x) {
  const uint64_t u = conv_dbits(x);
  const uint32_t hi = static_cast<uint32_t>(u >> 32), lo = static_cast<uint32_t>(u);
  const uint32_t ex = (hi >> 20) & 0x7ffu;
  // double exponents 897..1150 are the normal float exponents 1..254
  if (ex - 897u < 254u) {
    uint32_t f = (hi & 0x80000000u) | ((ex - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1fffffffu, half = 0x10000000u;
    f += (rest > half || (rest == half && (f & 1u))) ? 1u : 0u;
    return conv_float(f);
  }
  if (((hi & 0x7fffffffu) | lo) == 0u) return conv_float(hi & 0x80000000u);
  return static_cast<float>(x);
}

// float -> double, exact (static_cast<double>(f) for every f): zeros,
// normal floats, infinities and NaNs on the integer pipe, subnormal floats
// through the hardware conversion.
RG_CONV_FN double widen_exact(float f) {
  const uint32_t u = conv_fbits(f);
  const uint32_t ex = (u >> 23) & 0xffu, mant = u & 0x7fffffu;
  if (ex == 0u && mant != 0u) return static_cast<double>(f);
  const uint32_t dex = ex == 0u ? 0u : (ex == 0xffu ? 0x7ffu : ex + 896u);  // rebias 127 -> 1023
  return conv_double((u & 0x80000000u) | (dex << 20) | (mant >> 3), mant << 29);
}

// ---------------------------------------------------------------- comparisons
// IEEE-754 semantics: false when either operand is NaN, -0 == +0.

constexpr uint64_t kMagMask = 0x7fffffffffffffffull;
constexpr uint64_t kInfBits64 = 0x7ff0000000000000ull;

// |a| > t for t >= 0 or NaN
RG_CONV_FN bool abs_gt(double a, double t) {
  const uint64_t ma = conv_dbits(a) & kMagMask, ut = conv_dbits(t);
  return ma <= kInfBits64 && ut <= kInfBits64 && ma > ut;
}
// |a| in [lo, hi] for 0 < lo <= hi finite (the FP32 screening range test)
RG_CONV_FN bool abs_within(double a, double lo, double hi) {
  const uint64_t ma = conv_dbits(a) & kMagMask;
  return ma >= conv_dbits(lo) && ma <= conv_dbits(hi);
}
// a * b < 0 as the FP64 multiply rounds it.  Nonzero normal operands whose
// exponents sum to at least -1020 give a product of at least 2^-1020 in
// magnitude: negative exactly when the signs differ.  Zeros give a zero or
// NaN product; infinities, NaNs, subnormals and tiny products take the
// multiply.
RG_CONV_FN bool prod_neg(double a, double b) {
  const uint64_t ua = conv_dbits(a), ub = conv_dbits(b);
  const uint32_t ea = static_cast<uint32_t>(ua >> 52) & 0x7ffu, eb = static_cast<uint32_t>(ub >> 52) & 0x7ffu;
  if (((ua | ub) & kMagMask) != 0u && ((ua & kMagMask) == 0u || (ub & kMagMask) == 0u)) {
    // one zero and one nonzero: a zero product, or NaN for an infinity
    return false;
  }
  if (ea - 1u < 2046u && eb - 1u < 2046u && ea + eb >= 1026u) return ((ua ^ ub) >> 63) != 0u;
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b) < 0;
#else
  const volatile double p = a * b;
  return p < 0;
#endif
}

// The IEEE order of non-NaN doubles as signed integers: -0 and +0 map to 0,
// a larger value to a larger key.
RG_CONV_FN int64_t order_key(uint64_t u) {
  const int64_t m = static_cast<int64_t>(u & kMagMask);
  return (u >> 63) ? -m : m;
}
RG_CONV_FN bool nan_bits(uint64_t u) { return (u & kMagMask) > kInfBits64; }
// a < b on the bit patterns of two doubles (false when either is NaN; -0 == +0)
RG_CONV_FN bool lt_u(uint64_t ua, uint64_t ub) {
  return !nan_bits(ua) && !nan_bits(ub) && order_key(ua) < order_key(ub);
}
RG_CONV_FN bool lt(double a, double b) { return lt_u(conv_dbits(a), conv_dbits(b)); }
// std::max(a, b) = a < b ? b : a and std::min(a, b) = b < a ? b : a, bit for
// bit (the first operand on equality, -0 against +0 and NaN included).  The
// _u forms select between bit patterns, so that no FP64 instruction moves
// the chosen value.
RG_CONV_FN uint64_t max_first_u(uint64_t a, uint64_t b) { return lt_u(a, b) ? b : a; }
RG_CONV_FN uint64_t min_first_u(uint64_t a, uint64_t b) { return lt_u(b, a) ? b : a; }
RG_CONV_FN double max_first(double a, double b) { return lt(a, b) ? b : a; }
RG_CONV_FN double min_first(double a, double b) { return lt(b, a) ? b : a; }
RG_CONV_FN uint64_t abs_u(double a) { return conv_dbits(a) & kMagMask; }

}  // namespace rg

#undef RG_CONV_FN
