// rg_div.cuh -- correctly rounded FP64 division and square root on the
// integer and FP32 pipes.
//
// GB300 issues about 2 FP64 operations per clock per SM against 64-128
// 32-bit integer or FP32 ones, and an IEEE FP64 division costs about ten
// FP64 operations there.  div_rn(a, b) returns the same bits as a / b
// (round to nearest even) for every pair of doubles while using no FP64
// operation on its fast path (both operands normal or a zero numerator, the
// quotient normal); the other operands take a / b itself.
//
// Method (Newton-Raphson reciprocal refinement, quotient by multiplication,
// exact remainder and a remainder-based rounding step, as in Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34 (1990), and Cornea et al., "Correctness
// proofs outline for Newton-Raphson based floating-point divide and square
// root algorithms", ARITH 14 (1999); the exact remainder is taken modulo 2^64
// as in Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994).  With Ma, Mb the 53-bit significands:
//
//  1. A = Ma << borrow (borrow = Ma < Mb), so that the exact quotient
//     significand Qt = A * 2^52 / Mb lies in [2^52, 2^53).
//  2. Seed: r0 ~ 1/f, f = mb truncated to 23 fraction bits (mb = Mb / 2^52 in
//     [1, 2)), from the FP32 reciprocal approximation.  One Newton step in
//     float-float: e = 1 - mb*r0 from two FP32 FMAs on f and the rest of mb,
//     c = r0*e, r1 = r0 + c held as a 64-bit fixed-point R1 = r1 * 2^63
//     (r0 * 2^25 and c * 2^50 converted to 32-bit integers: the first exactly,
//     the second to within 2^-51).
//     The step is taken only when the computed |e| <= 2^-22 (else a / b).
//     The two FMAs and the rounding of the low part of mb to float leave e
//     within 2^-45 of 1 - mb*r0, and c rounds once (2^-24 relative), so
//     |r1*mb - 1| <= (2^-22 + 2^-45)^2 + 2^-45 + 2^-46 + 2^-51 < 1.76 * 2^-44.
//  3. Q0 = the high 64 bits of 2A * R1 without the low-by-low partial product
//     and the carries of the low words (at most 2 below the exact high word),
//     so Q0 is within
//     2^53 * 1.76 * 2^-44 + 4 < 910 of Qt.
//  4. The remainder R = A * 2^52 - Mb * Q0 = Mb * (Qt - Q0) is below
//     2^53 * 910 < 2^62.9 in magnitude, so it is exact as a signed 64-bit
//     value computed modulo 2^64.
//  5. k = nearest integer to R / Mb from an FP32 estimate (the high word of
//     R times r0: error below 910 * 2^-21.3 + 2^-20 < 2^-11),
//     R2 = R - k*Mb (exact), |R2| / Mb < 1/2 + 2^-11.
//  6. Q = Q0 + k, plus 1 if 2 R2 > Mb, minus 1 if 2 R2 < -Mb: the nearest
//     integer to Qt.  Qt is never a half-integer (2 A * 2^52 = Mb * (2Q+1)
//     needs Mb to divide a power of two, and then the quotient is exact), so
//     there are no ties.  Q = 2^53 (rounding up into the next binade) carries
//     into the exponent field when the result is assembled.
//
// tests/test_cpu_div.py checks the host build of this code against the
// host's division (random operands over the whole exponent range, operands
// at and next to powers of two, quotients next to rounding midpoints, seeds
// perturbed to the edge of the error bound); tests/test_gpu_div.py checks
// the device build against the device's a / b.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define RG_DIV_FN __host__ __device__ __forceinline__
#else
#define RG_DIV_FN inline
#endif

namespace rg {
namespace div_detail {

RG_DIV_FN uint64_t d2u(double x) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t u;
  std::memcpy(&u, &x, sizeof u);
  return u;
#endif
}
RG_DIV_FN double u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(u));
#else
  double x;
  std::memcpy(&x, &u, sizeof x);
  return x;
#endif
}
RG_DIV_FN uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, sizeof u);
  return u;
#endif
}
RG_DIV_FN float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, sizeof x);
  return x;
#endif
}
RG_DIV_FN uint64_t umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}
RG_DIV_FN float fma32(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}
RG_DIV_FN float mul32(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

RG_DIV_FN uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return static_cast<uint32_t>((static_cast<uint64_t>(a) * b) >> 32);
#endif
}
// float -> integer: an integer-valued float in [0, 2^32); round to nearest even
RG_DIV_FN uint32_t f2u_int(float x) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(x);
#else
  return static_cast<uint32_t>(x);
#endif
}
RG_DIV_FN int32_t f2i_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(x);
#else
  return static_cast<int32_t>(__builtin_rintf(x));
#endif
}

constexpr uint64_t kFrac = (uint64_t(1) << 52) - 1;
constexpr uint64_t kHidden = uint64_t(1) << 52;
constexpr uint64_t kSign = uint64_t(1) << 63;

}  // namespace div_detail

// The FP32 reciprocal approximation of the device (the seed of step 2).
struct RcpSeedDevice {
#if defined(__CUDACC__)
  __device__ __forceinline__ float operator()(float f) const {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    return r;
  }
#endif
};

// a / b on the fast path; returns false (and leaves *q) where the operands are
// outside it.  Seed: a callable float -> float approximating 1/f on [1, 2).
template <class Seed>
RG_DIV_FN bool div_rn_fast(double a, double b, const Seed& seed, double* q) {
  using namespace div_detail;
  const uint64_t ua = d2u(a), ub = d2u(b);
  const uint32_t ea = static_cast<uint32_t>(ua >> 52) & 0x7ffu, eb = static_cast<uint32_t>(ub >> 52) & 0x7ffu;
  const uint64_t sign = (ua ^ ub) & kSign;
  if (eb - 1u >= 2046u) return false;  // b zero, subnormal, infinite or NaN
  if (ea == 0u && (ua & kFrac) == 0u) {
    *q = u2d(sign);  // +-0 / normal
    return true;
  }
  const int d = static_cast<int>(ea) - static_cast<int>(eb);
  if (ea - 1u >= 2046u || d < -1021 || d > 1022) return false;  // a subnormal / special, quotient not normal
  const uint64_t ma = (ua & kFrac) | kHidden, mb = (ub & kFrac) | kHidden;
  const uint32_t borrow = ma < mb ? 1u : 0u;
  const uint64_t A = ma << borrow;
  // step 2: seed and one float-float Newton step
  const float f_hi = u2f(0x3f800000u | static_cast<uint32_t>((mb & kFrac) >> 29));
  const float f_lo = mul32(static_cast<float>(static_cast<uint32_t>(mb & 0x1fffffffu)), 2.220446049250313e-16f);
  const float r0 = seed(f_hi);
  float e = fma32(-f_hi, r0, 1.0f);
  e = fma32(-f_lo, r0, e);
  if (!(e <= 2.384185791015625e-07f && e >= -2.384185791015625e-07f)) return false;  // |e| <= 2^-22
  const float c = mul32(r0, e);
  // r0 in [0.25, 1] (the test above fails otherwise): r0 * 2^25 is an integer
  // below 2^26; |c| < 2^-21.9, so |c * 2^50| < 2^29
  const uint32_t r0i = f2u_int(mul32(r0, 33554432.0f));
  const int32_t ci = f2i_rn(mul32(c, 1125899906842624.0f));
  const uint64_t R1 = (static_cast<uint64_t>(r0i) << 38) + static_cast<uint64_t>(static_cast<int64_t>(ci) * 8192);
  // step 3: quotient estimate from three 32 x 32-bit products
  const uint64_t X = A << 1;
  const uint32_t x1 = static_cast<uint32_t>(X >> 32), x0 = static_cast<uint32_t>(X);
  const uint32_t y1 = static_cast<uint32_t>(R1 >> 32), y0 = static_cast<uint32_t>(R1);
  const uint64_t Q0 = static_cast<uint64_t>(x1) * y1 + mulhi32(x1, y0) + mulhi32(x0, y1);
  // step 4: exact remainder (modulo 2^64)
  const int64_t R = static_cast<int64_t>((A << 52) - mb * Q0);
  // step 5: nearest integer to R / Mb (|R / Mb| < 910; R >> 32 fits 31 bits)
  const int32_t k = f2i_rn(mul32(mul32(static_cast<float>(static_cast<int32_t>(R >> 32)), r0), 9.5367431640625e-07f));
  const int64_t R2 = R - static_cast<int64_t>(k) * static_cast<int64_t>(mb);
  // step 6: round to nearest
  const int64_t twice = R2 * 2;
  const int64_t m = static_cast<int64_t>(mb);
  const uint64_t Q = Q0 + static_cast<uint64_t>(static_cast<int64_t>(k)) + (twice > m ? 1u : 0u) -
                     (twice < -m ? 1u : 0u);
  // exponent field d + 1023 - borrow; Q's hidden bit (or Q = 2^53) adds to it
  *q = u2d(sign | ((static_cast<uint64_t>(d + 1022 - static_cast<int>(borrow)) << 52) + Q));
  return true;
}

// The FP32 reciprocal square root approximation of the device (the seed of sqrt_rn_fast).
struct RsqrtSeedDevice {
#if defined(__CUDACC__)
  __device__ __forceinline__ float operator()(float f) const {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    return r;
  }
#endif
};

// sqrt(x) correctly rounded on the fast path (x a positive normal double or
// a zero); returns false (and leaves *r) otherwise.  Seed: a callable float
// -> float approximating 1/sqrt(f) on [1, 4).  With Mx the 53-bit
// significand, x = m * 2^E, m = Mx * 2^(odd - 52) in [1, 4), E even, the
// result significand is S = nearest integer to sqrt(N), N = Mx * 2^(52 + odd):
//  1. y ~ 1/sqrt(f), f = m truncated to 24 bits; e = 1 - f*y^2 (the step is
//     taken only when |e| <= 2^-21, else sqrt(x)); s0 = f*y, within
//     1.5 * 2^-22 of sqrt(m); the remainder m - s0^2 in float-float (s0^2
//     split exactly by an FMA, m as f plus its low part) and one Newton step
//     c = (m - s0^2) / (2 s0) with 1/s0 ~ y + y*e; S1 = (s0 + c) * 2^52 in
//     fixed point, within 2^-42 (relative) of sqrt(N), so |N - S1^2| < 2^66.
//  2. The remainder N - S1^2 exactly in 128 bits; k = (its top bits as a
//     float) / (2 S1), rounded: error below 2^-4, so S2 = S1 + k is within
//     1/2 + 2^-4 of sqrt(N).
//  3. R = N - S2^2, exact modulo 2^64 (|R| < 2^55): sqrt(N) > S2 + 1/2 iff
//     R > S2, and sqrt(N) < S2 - 1/2 iff R <= -S2 (N and S2 are integers,
//     so (S2 +- 1/2)^2 is never N: no ties).  S = S2 + 1, S2 - 1 or S2; S =
//     2^53 carries into the exponent field.
template <class Seed>
RG_DIV_FN bool sqrt_rn_fast(double x, const Seed& seed, double* r) {
  using namespace div_detail;
  const uint64_t ux = d2u(x);
  if ((ux & ~kSign) == 0u) {
    *r = x;  // sqrt(+-0) = +-0
    return true;
  }
  const uint32_t ex = static_cast<uint32_t>(ux >> 52);  // with the sign: negative x is out of range
  if (ex - 1u >= 2046u) return false;                   // negative, subnormal, infinite or NaN
  const uint32_t odd = (ex & 1u) ^ 1u;                  // ex - 1023 odd
  const uint64_t mx = (ux & kFrac) | kHidden;
  // step 1 (f in [1, 4); the low part is the 29 bits below f's significand)
  const float f = u2f(((127u + odd) << 23) | static_cast<uint32_t>((ux & kFrac) >> 29));
  const float f_lo = mul32(static_cast<float>(static_cast<uint32_t>(ux & 0x1fffffffu)),
                           odd ? 4.440892098500626e-16f : 2.220446049250313e-16f);
  const float y = seed(f);
  const float e = fma32(-f, mul32(y, y), 1.0f);
  if (!(e <= 4.76837158203125e-07f && e >= -4.76837158203125e-07f)) return false;  // |e| <= 2^-21
  const float s0 = mul32(f, y);
  const float p = mul32(s0, s0);
  const float pe = fma32(s0, s0, -p);
  const float rm = ((f - p) - pe) + f_lo;  // m - s0^2 (f - p is exact)
  const float inv = fma32(y, e, y);        // 1 / s0
  const float c = mul32(mul32(rm, inv), 0.5f);
  // s0 in [0.5, 2]: s0 * 2^24 is an integer below 2^25 + 1; |c| < 2^-19, so
  // |c * 2^50| < 2^31
  const uint64_t S1 = (static_cast<uint64_t>(f2u_int(mul32(s0, 16777216.0f))) << 28) +
                      static_cast<uint64_t>(static_cast<int64_t>(f2i_rn(mul32(c, 1125899906842624.0f))) * 4);
  // step 2: N - S1^2 in 128 bits, then its top bits
  const uint64_t n_lo = mx << (52 + odd), n_hi = mx >> (12 - odd);
  const uint64_t q_lo = S1 * S1, q_hi = umulhi(S1, S1);
  const uint64_t r_lo = n_lo - q_lo;
  const uint64_t r_hi = n_hi - q_hi - (n_lo < q_lo ? 1u : 0u);
  const int64_t r48 = static_cast<int64_t>((r_hi << 16) | (r_lo >> 48));  // floor(remainder / 2^48), |.| < 2^18
  // k = remainder / (2 S1) = remainder * inv * 2^-53
  const int32_t k = f2i_rn(mul32(mul32(static_cast<float>(static_cast<int32_t>(r48)), inv), 0.03125f));
  const uint64_t S2 = S1 + static_cast<uint64_t>(static_cast<int64_t>(k));
  // step 3: exact remainder and rounding
  const int64_t R = static_cast<int64_t>(n_lo - S2 * S2);
  const int64_t s2 = static_cast<int64_t>(S2);
  const uint64_t S = S2 + (R > s2 ? 1u : 0u) - (R <= -s2 ? 1u : 0u);
  // exponent field E/2 + 1023 (E = ex - 1023 - odd, even); S's hidden bit adds the one
  const int field = (static_cast<int>(ex) - static_cast<int>(odd) - 1023) / 2 + 1022;
  *r = u2d((static_cast<uint64_t>(field) << 52) + S);
  return true;
}

#if defined(__CUDACC__)
// The IEEE division for the operands outside the fast path, kept out of line
// so that the compiler cannot compute it ahead of the branch.
static __device__ __noinline__ double div_ieee(double a, double b) { return a / b; }

// a / b, bitwise (the fast path above, a / b outside it)
__device__ __forceinline__ double div_rn(double a, double b) {
  double q;
  if (div_rn_fast(a, b, RcpSeedDevice{}, &q)) return q;
  return div_ieee(a, b);
}

static __device__ __noinline__ double sqrt_ieee(double x) { return sqrt(x); }

// sqrt(x), bitwise (the fast path above, sqrt(x) outside it)
__device__ __forceinline__ double sqrt_rn(double x) {
  double r;
  if (sqrt_rn_fast(x, RsqrtSeedDevice{}, &r)) return r;
  return sqrt_ieee(x);
}

// a / b of the kernels' real type: div_rn for double, the FP32 division for float
__device__ __forceinline__ double quot(double a, double b) { return div_rn(a, b); }
__device__ __forceinline__ float quot(float a, float b) { return a / b; }
// sqrt of the kernels' real type: sqrt_rn for double, the FP32 square root for float
__device__ __forceinline__ double root(double x) { return sqrt_rn(x); }
__device__ __forceinline__ float root(float x) { return sqrtf(x); }
#endif

}  // namespace rg
