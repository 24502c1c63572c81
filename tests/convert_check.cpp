// Checks rg::narrow and rg::widen_exact (huji-rich_gb300/csrc/rg_convert.cuh,
// the integer-pipe float <-> double conversions of the FP32-mixed kernels)
// against the C casts, bit for bit: random bit patterns, values across the
// float range, rounding ties and carries, the special values, and a stride
// through every float; and the integer-pipe double tests (abs_gt,
// abs_within, prod_neg, lt, max_first, min_first) against the C operators.  Exit status 0 when every value agrees.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "rg_convert.cuh"

static long n_bad = 0;

static void check_narrow(double x) {
  const float a = rg::narrow(x), b = static_cast<float>(x);
  uint32_t ua, ub;
  memcpy(&ua, &a, 4);
  memcpy(&ub, &b, 4);
  if (ua != ub && !(std::isnan(a) && std::isnan(b))) {
    if (n_bad < 5) printf("narrow(%a) = %a, cast %a\n", x, a, b);
    ++n_bad;
  }
}

int main() {
  std::mt19937_64 g(20260101);
  for (long i = 0; i < 4000000; ++i) {
    const uint64_t u = g();
    double x;
    memcpy(&x, &u, 8);
    check_narrow(x);
  }
  std::uniform_real_distribution<double> ud(-1, 1);
  for (long i = 0; i < 2000000; ++i) check_narrow(ud(g) * std::ldexp(1.0, static_cast<int>(g() % 300) - 150));
  // halfway cases and their neighbours, carries into the exponent
  for (long i = 0; i < 2000000; ++i) {
    const uint32_t fu = static_cast<uint32_t>(g());
    float f;
    memcpy(&f, &fu, 4);
    if (!std::isfinite(f)) continue;
    double x = f;
    uint64_t u;
    memcpy(&u, &x, 8);
    u += (uint64_t{1} << 28) + (g() % 3) - 1;
    memcpy(&x, &u, 8);
    check_narrow(x);
    check_narrow(-x);
    check_narrow(std::nextafter(static_cast<double>(f), 1e300));
  }
  const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 3.4028235677973366e38, 3.4028235e38, 3.5e38,
                            1.1754943508222875e-38, 1.1754942e-38, 1e-45, 1.4e-45, 7e-46, 2.1e-45, 1e300, -1e-300};
  for (double x : special) check_narrow(x);
  for (uint64_t u = 0; u < (uint64_t{1} << 32); u += 613) {
    const uint32_t fu = static_cast<uint32_t>(u);
    float f;
    memcpy(&f, &fu, 4);
    const double a = rg::widen_exact(f), b = static_cast<double>(f);
    uint64_t ua, ub;
    memcpy(&ua, &a, 8);
    memcpy(&ub, &b, 8);
    if (ua != ub && !(std::isnan(a) && std::isnan(b))) {
      if (n_bad < 5) printf("widen_exact(%a) = %a\n", static_cast<double>(f), a);
      ++n_bad;
    }
  }
  // comparisons: values drawn from a pool that mixes special values, zeros
  // of both signs, subnormals, tiny and huge magnitudes and random bits
  const double pool_special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, 0x1p-1074, -0x1p-1074, 0x1p-1022,
                                 -0x1p-1022, 1e-36, 1e36, 1.0, -1.0, 0x1p-511, 0x1p-510, 0x1p-509, -0x1p-512,
                                 1.7976931348623157e308, -1.7976931348623157e308, 0x1.8p-1022, 3.0};
  const int n_special = sizeof(pool_special) / sizeof(pool_special[0]);
  auto draw = [&]() -> double {
    const uint64_t r = g();
    switch (r % 5) {
      case 0: return pool_special[(r >> 8) % n_special];
      case 1: {
        uint64_t u = g();
        double x;
        memcpy(&x, &u, 8);
        return x;
      }
      case 2: return ud(g) * std::ldexp(1.0, static_cast<int>(g() % 2100) - 1075);
      case 3: return ud(g) * std::ldexp(1.0, static_cast<int>(g() % 40) - 20);
      default: return std::ldexp(static_cast<double>(static_cast<int>(g() % 7) - 3), static_cast<int>(g() % 8));
    }
  };
  for (long i = 0; i < 6000000; ++i) {
    const double a = draw(), b = draw();
    const double t = std::fabs(draw());
    bool ok = rg::abs_gt(a, t) == (std::fabs(a) > t) &&
              rg::abs_within(a, 1e-36, 1e36) == (std::fabs(a) >= 1e-36 && std::fabs(a) <= 1e36);
    volatile double p = a * b;
    ok = ok && rg::prod_neg(a, b) == (p < 0);
    ok = ok && rg::lt(a, b) == (a < b) && rg::lt(b, a) == (b < a) && rg::lt(a, a) == (a < a);
    const double mx = rg::max_first(a, b), mn = rg::min_first(a, b);
    const double rmx = a < b ? b : a, rmn = b < a ? b : a;
    uint64_t u1, u2, u3, u4;
    memcpy(&u1, &mx, 8);
    memcpy(&u2, &rmx, 8);
    memcpy(&u3, &mn, 8);
    memcpy(&u4, &rmn, 8);
    ok = ok && u1 == u2 && u3 == u4;
    if (!ok) {
      if (n_bad < 5) printf("comparison mismatch at a=%a b=%a t=%a\n", a, b, t);
      ++n_bad;
    }
  }
  printf("%ld mismatches\n", n_bad);
  return n_bad == 0 ? 0 : 1;
}
