// Checks fegpu::sf_add (csrc/softf64.cuh) against the host's IEEE binary64
// addition, bit for bit, on random and constructed operand pairs: uniform bit
// patterns (every class: zeros, subnormals, infinities, NaNs), operands with
// exponent differences 0..70 and random signs, near-cancellations, exact ties
// (operands whose sum lies halfway between two doubles), sums at the top and
// bottom of the normal range, and signed zeros.  Prints "ok" when all agree.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "softf64.cuh"

using fegpu::sf_add;
using fegpu::sf_bits;
using fegpu::sf_double;

static uint64_t failures = 0, checked = 0;

static void check(double x, double y) {
  volatile double ref = x + y;
  const double got = sf_add(x, y);
  ++checked;
  const bool same = sf_bits(got) == sf_bits(ref) || (std::isnan(got) && std::isnan(ref));
  if (!same && failures++ < 20)
    std::printf("MISMATCH x=%a y=%a got=%a ref=%a\n", x, y, got, static_cast<double>(ref));
}

static double make(uint64_t sign, uint64_t exp, uint64_t frac) {
  return sf_double((sign << 63) | (exp << 52) | (frac & 0x000fffffffffffffull));
}

int main(int argc, char **argv) {
  const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 2000000;
  std::mt19937_64 rng(20261204);
  // uniform bit patterns
  for (uint64_t i = 0; i < n; ++i) check(sf_double(rng()), sf_double(rng()));
  // exponent differences 0..70, random signs and fractions
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t ex = 1 + rng() % 2046;
    const uint64_t d = rng() % 71;
    const uint64_t ey = ex > d ? ex - d : 1;
    check(make(rng() & 1, ex, rng()), make(rng() & 1, ey, rng()));
  }
  // near-cancellations: y = -(x + a few ulps)
  for (uint64_t i = 0; i < n; ++i) {
    const double x = make(rng() & 1, 1 + rng() % 2046, rng());
    const int64_t k = static_cast<int64_t>(rng() % 9) - 4;
    const double y = -sf_double(sf_bits(x) + k);
    check(x, y);
  }
  // ties: the smaller operand has its lowest set bit exactly half an ulp of
  // the sum below it (fractions with few low bits set)
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t ex = 60 + rng() % 1900;
    const uint64_t d = 1 + rng() % 56;
    const uint64_t fx = rng() & ~0xffull;
    const uint64_t fy = (rng() & 0x000ffffffffff000ull) | (1ull << (rng() % 12));
    check(make(rng() & 1, ex, fx), make(rng() & 1, ex - d, fy));
  }
  // top and bottom of the normal range (overflow to infinity, results that
  // are subnormal or cross into the subnormals)
  for (uint64_t i = 0; i < n / 4; ++i) {
    check(make(rng() & 1, 2046 - rng() % 3, rng()), make(rng() & 1, 2046 - rng() % 60, rng()));
    check(make(rng() & 1, 1 + rng() % 3, rng()), make(rng() & 1, 1 + rng() % 3, rng()));
    check(make(rng() & 1, 1 + rng() % 2, rng()), make(rng() & 1, 0, rng()));
  }
  // zeros
  const double z[] = {0.0, -0.0};
  for (double a : z)
    for (double b : z) check(a, b);
  for (uint64_t i = 0; i < 1000; ++i) {
    const double x = make(rng() & 1, rng() % 2048, rng());
    check(x, z[rng() & 1]);
    check(z[rng() & 1], x);
  }
  std::printf("%" PRIu64 " sums, %" PRIu64 " mismatches\n", checked, failures);
  if (failures == 0) std::printf("ok\n");
  return failures == 0 ? 0 : 1;
}
