// sqrt_check.cpp -- the host build of rg::sqrt_rn_fast
// (huji-rich_gb300/csrc/rg_div.cuh) against the host's IEEE square root,
// bit for bit.
//
//   sqrt_check <seed kind> <cases per family> <rng seed>
//
// Seed kinds (the FP32 reciprocal square root the fast path starts from):
//   0 the correctly rounded 1/sqrt(f); 1, 2 one ulp above / below it;
//   3, 4 two ulps above / below it; 5 a crude estimate (every root falls
//   back); 6 1/sqrt(f) times (1 + u * 2^-22), u in [-1, 1) from a hash of f
//   (errors over the whole band the fast path accepts).
// Operand families: tests/div_cases.h (generate_sqrt).  Prints one JSON line.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "div_cases.h"
#include "rg_div.cuh"

namespace {

int g_kind = 0;

using divcases::bits;
float next_up(float x, int n) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u += n;
  std::memcpy(&x, &u, 4);
  return x;
}

struct HostRsqrt {
  float operator()(float f) const {
    const float r = static_cast<float>(1.0 / std::sqrt(static_cast<double>(f)));
    switch (g_kind) {
      case 1: return next_up(r, 1);
      case 2: return next_up(r, -1);
      case 3: return next_up(r, 2);
      case 4: return next_up(r, -2);
      case 5: {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        u = 0x5f3759dfu - (u >> 1);  // a bit-pattern estimate
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
        return static_cast<float>((1.0 + t) / std::sqrt(static_cast<double>(f)));
      }
      default: return r;
    }
  }
};

long long g_cases = 0, g_bad = 0, g_fast = 0;
double g_bad_x = 0;

void check(double x) {
  ++g_cases;
  double r;
  const bool fast = rg::sqrt_rn_fast(x, HostRsqrt{}, &r);
  if (!fast) r = std::sqrt(x);
  g_fast += fast;
  const double ref = std::sqrt(x);
  if (!(bits(r) == bits(ref) || (std::isnan(r) && std::isnan(ref)))) {
    if (g_bad == 0) g_bad_x = x;
    ++g_bad;
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: sqrt_check <seed kind> <cases per family> <rng seed>\n");
    return 2;
  }
  g_kind = std::atoi(argv[1]);
  const long long n = std::atoll(argv[2]);
  std::mt19937_64 rng(std::strtoull(argv[3], nullptr, 10));
  divcases::generate_sqrt(rng, n, check);
  std::printf("{\"seed_kind\": %d, \"cases\": %lld, \"mismatches\": %lld, \"fast\": %lld, \"first_x\": %.17g}\n",
              g_kind, g_cases, g_bad, g_fast, g_bad_x);
  return g_bad == 0 ? 0 : 1;
}
