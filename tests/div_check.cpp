// div_check.cpp -- the host build of huji-rich_gb300/csrc/rg_div.cuh against
// the host's IEEE division, bit for bit.
//
//   div_check <seed kind> <cases per family> <rng seed>
//
// Seed kinds (the FP32 reciprocal approximation the fast path starts from):
//   0 the correctly rounded 1/f;  1, 2 one ulp above / below it;
//   3, 4 two ulps above / below it (near the fast path's |e| <= 2^-22 limit);
//   5 a crude approximation (about 2^-4), so that every division falls back;
//   6 1/f times (1 + u * 2^-22), u in [-1, 1) from a hash of f: errors over
//     the whole band the fast path accepts.
// Operand families: tests/div_cases.h.
// Prints one JSON line: cases, mismatches, fast-path count, first mismatch.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "div_cases.h"
#include "rg_div.cuh"

namespace {

int g_kind = 0;

float next_up(float x, int n) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u += n;
  std::memcpy(&x, &u, 4);
  return x;
}

struct HostSeed {
  float operator()(float f) const {
    const float r = 1.0f / f;
    switch (g_kind) {
      case 1: return next_up(r, 1);
      case 2: return next_up(r, -1);
      case 3: return next_up(r, 2);
      case 4: return next_up(r, -2);
      case 5: {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        u = 0x7ef311c7u - u;  // a bit-pattern reciprocal estimate
        float y;
        std::memcpy(&y, &u, 4);
        return y;
      }
      case 6: {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        u = (u ^ (u >> 15)) * 0x2c1b3c6du;
        u = (u ^ (u >> 12)) * 0x297a2d39u;
        u ^= u >> 15;
        const double t = (static_cast<double>(u) / 2147483648.0 - 1.0) * 2.384185791015625e-07;
        return static_cast<float>((1.0 + t) / static_cast<double>(f));
      }
      default: return r;
    }
  }
};

using divcases::bits;
using divcases::from;

long long g_cases = 0, g_bad = 0, g_fast = 0;
double g_bad_a = 0, g_bad_b = 0;

void check(double a, double b) {
  ++g_cases;
  double q;
  const bool fast = rg::div_rn_fast(a, b, HostSeed{}, &q);
  if (!fast) q = a / b;
  g_fast += fast;
  const double ref = a / b;
  const bool same = bits(q) == bits(ref) || (std::isnan(q) && std::isnan(ref));
  if (!same) {
    if (g_bad == 0) {
      g_bad_a = a;
      g_bad_b = b;
    }
    ++g_bad;
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: div_check <seed kind> <cases per family> <rng seed>\n");
    return 2;
  }
  g_kind = std::atoi(argv[1]);
  const long long n = std::atoll(argv[2]);
  std::mt19937_64 rng(std::strtoull(argv[3], nullptr, 10));
  divcases::generate(rng, n, check);
  std::printf("{\"seed_kind\": %d, \"cases\": %lld, \"mismatches\": %lld, \"fast\": %lld, "
              "\"first_a\": %.17g, \"first_b\": %.17g}\n",
              g_kind, g_cases, g_bad, g_fast, g_bad_a, g_bad_b);
  return g_bad == 0 ? 0 : 1;
}
