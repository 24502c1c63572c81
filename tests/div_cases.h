// div_cases.h -- operand families for the FP64 division and square root
// checks (tests/div_check.cpp and tests/sqrt_check.cpp on the host,
// tests/div_check_gpu.cu on the device).
//
// Families: random bit patterns (every class of double), random normal
// operands over the whole exponent range, operands of moderate size,
// divisors and numerators at or next to powers of two, quotients next to
// rounding midpoints (a = RN(b * (Q + 1/2) * 2^-52) and its neighbours),
// quotients next to powers of two, zero numerators, and exponent
// differences at the edges of the division's fast path.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

namespace divcases {

inline uint64_t bits(double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
}
inline double from(uint64_t u) {
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

// calls check(a, b) for about 7 n pairs
template <class F>
void generate(std::mt19937_64& rng, long long n, F&& check) {
  std::uniform_int_distribution<uint64_t> u64;
  auto frac = [&]() { return u64(rng) & ((uint64_t(1) << 52) - 1); };
  auto sgn = [&]() { return (u64(rng) & 1) << 63; };
  // random bit patterns: zeros, subnormals, infinities and NaNs included
  for (long long i = 0; i < n; ++i) check(from(u64(rng)), from(u64(rng)));
  // random normal operands over the whole exponent range
  for (long long i = 0; i < n; ++i) {
    const uint64_t ea = 1 + u64(rng) % 2046, eb = 1 + u64(rng) % 2046;
    check(from(sgn() | ea << 52 | frac()), from(sgn() | eb << 52 | frac()));
  }
  // operands of moderate size (the physics range), every exponent difference near 0
  for (long long i = 0; i < n; ++i) {
    const uint64_t ea = 1023 - 40 + u64(rng) % 80, eb = 1023 - 40 + u64(rng) % 80;
    check(from(sgn() | ea << 52 | frac()), from(sgn() | eb << 52 | frac()));
  }
  // divisors that are powers of two or next to them; numerators likewise
  for (long long i = 0; i < n; ++i) {
    const uint64_t eb = 900 + u64(rng) % 250;
    const uint64_t near = u64(rng) % 5;  // 0: exact, 1-2: +1/+2 ulp, 3-4: -1/-2 ulp
    uint64_t ub = eb << 52;
    if (near == 1 || near == 2) ub += near;
    if (near >= 3) ub -= near - 2;
    const uint64_t ea = 900 + u64(rng) % 250;
    const uint64_t ua = (u64(rng) & 1) ? (ea << 52 | frac()) : (ea << 52) + (u64(rng) % 3) - 1;
    check(from(sgn() | ua), from(sgn() | ub));
  }
  // quotients within about 2^-60 (relative) of a rounding midpoint:
  // a = RN(b * (Q + 1/2) * 2^e) for a 53-bit Q
  for (long long i = 0; i < n; ++i) {
    const uint64_t mb = frac() | (uint64_t(1) << 52);
    const uint64_t Q = frac() | (uint64_t(1) << 52);
    const unsigned __int128 N = static_cast<unsigned __int128>(mb) * (2 * Q + 1);  // < 2^107
    int top = 127;
    while (!((N >> top) & 1)) --top;
    // round N to 53 significant bits (to nearest even)
    const int sh = top - 52;
    unsigned __int128 m = N >> sh;
    const unsigned __int128 rem = N & ((static_cast<unsigned __int128>(1) << sh) - 1);
    const unsigned __int128 half = static_cast<unsigned __int128>(1) << (sh - 1);
    if (rem > half || (rem == half && (m & 1))) m += 1;
    int top2 = sh;
    if (m >> 53) {
      m >>= 1;
      ++top2;
    }
    const uint64_t eb = 1023 - 20 + u64(rng) % 40;
    // a = m * 2^(top2 + eb - 1023 - 52 - 52 - 1 ...): keep the quotient normal
    const int64_t ea = static_cast<int64_t>(eb) + (top2 + 52) - 105;
    if (ea < 1 || ea > 2046) continue;
    const uint64_t ua = static_cast<uint64_t>(ea) << 52 | (static_cast<uint64_t>(m) & ((uint64_t(1) << 52) - 1));
    const uint64_t ub = eb << 52 | (mb & ((uint64_t(1) << 52) - 1));
    check(from(sgn() | ua), from(sgn() | ub));
    // and the neighbours of a
    check(from(ua + 1), from(ub));
    check(from(ua - 1), from(ub));
  }
  // quotients next to powers of two: a = b * (1 - k ulp) and b * (1 + k ulp)
  for (long long i = 0; i < n; ++i) {
    const uint64_t ub = (1000 + u64(rng) % 46) << 52 | frac();
    const double b = from(ub);
    const int k = 1 + static_cast<int>(u64(rng) % 4);
    check(from(bits(b) + k), b);
    check(from(bits(b) - k), b);
    check(from(bits(b * 2.0) - k), b);
    check(from(bits(b * 0.5) + k), b);
  }
  // zero numerators; exponent differences at the edges of the fast path
  for (long long i = 0; i < n / 8 + 1; ++i) {
    const uint64_t ub = (1 + u64(rng) % 2046) << 52 | frac();
    check(from(sgn()), from(sgn() | ub));
    for (int d : {-1023, -1022, -1021, -1020, 1021, 1022, 1023, 1024}) {
      const int64_t eb = 1023 - d / 2, ea = eb + d;
      if (ea < 1 || ea > 2046 || eb < 1 || eb > 2046) continue;
      check(from(sgn() | static_cast<uint64_t>(ea) << 52 | frac()),
            from(sgn() | static_cast<uint64_t>(eb) << 52 | frac()));
    }
  }
}


// calls check(x) for about 11 n values of x: random bit patterns, random
// positive normals over the whole exponent range and near 1, exact squares
// of 26-bit integers and their neighbours, values next to (S + 1/2)^2 for a
// 53-bit S (the rounding midpoints of the square root), powers of two and
// their neighbours, zeros
template <class F>
void generate_sqrt(std::mt19937_64& rng, long long n, F&& check) {
  std::uniform_int_distribution<uint64_t> u64;
  const uint64_t kFrac = (uint64_t(1) << 52) - 1;
  for (long long i = 0; i < n; ++i) check(from(u64(rng)));
  for (long long i = 0; i < n; ++i) check(from((1 + u64(rng) % 2046) << 52 | (u64(rng) & kFrac)));
  for (long long i = 0; i < n; ++i) check(from((1021 + u64(rng) % 4) << 52 | (u64(rng) & kFrac)));
  // exact squares of 26-bit integers (scaled), and their neighbours
  for (long long i = 0; i < n; ++i) {
    const uint64_t S = (uint64_t(1) << 25) | (u64(rng) & ((uint64_t(1) << 25) - 1));
    const double sq = static_cast<double>(S * S);  // < 2^52: exact
    const double x = ldexp(sq, static_cast<int>(u64(rng) % 200) - 100);
    check(x);
    check(from(bits(x) + 1));
    check(from(bits(x) - 1));
  }
  // next to (S + 1/2)^2 for a 53-bit S: x = RN((S + 1/2)^2 * 2^e) and neighbours
  for (long long i = 0; i < n; ++i) {
    const uint64_t S = (uint64_t(1) << 52) | (u64(rng) & kFrac);
    const unsigned __int128 T = static_cast<unsigned __int128>(2 * S + 1) * (2 * S + 1);  // 4 (S + 1/2)^2, < 2^108
    int top = 127;
    while (!((T >> top) & 1)) --top;
    const int sh = top - 52;
    unsigned __int128 m = T >> sh;
    const unsigned __int128 rem = T & ((static_cast<unsigned __int128>(1) << sh) - 1);
    const unsigned __int128 half = static_cast<unsigned __int128>(1) << (sh - 1);
    if (rem > half || (rem == half && (m & 1))) m += 1;
    int top2 = sh;
    if (m >> 53) {
      m >>= 1;
      ++top2;
    }
    // value m * 2^(top2 - 2) * 2^(2j) for an even scale
    const int j = static_cast<int>(u64(rng) % 200) - 100;
    const double x = ldexp(static_cast<double>(static_cast<uint64_t>(m)), top2 - 2 - 104 + 2 * j);
    check(x);
    check(from(bits(x) + 1));
    check(from(bits(x) - 1));
  }
  // powers of two and their neighbours, zeros
  for (long long i = 0; i < n / 4 + 1; ++i) {
    const uint64_t e = 1 + u64(rng) % 2046;
    const uint64_t u = e << 52;
    check(from(u));
    check(from(u + 1 + u64(rng) % 3));
    check(from(u - 1 - u64(rng) % 3));
    check(0.0);
    check(-0.0);
  }
}

}  // namespace divcases
