// Prints (h, l, ff_to_double_exact(h, l), ff_to_double(h, l)) as hex bit
// patterns for a seeded set of float-float pairs, for tests/test_ffconv.py,
// which checks them against exact rational arithmetic.  Pairs: accumulations
// of random contributions by two-sum (as the row gather forms them), pairs
// with chosen exponent gaps and signs, and edge cases (zeros, subnormals,
// powers of two with an opposite-sign remainder, inf, nan).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "ffconv.h"

using namespace fegpu;

static uint32_t fb(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
}
static uint64_t db(double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
}
static float fromb(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
static void emit(float h, float l) {
  std::printf("%08x %08x %016llx %016llx\n", fb(h), fb(l),
              static_cast<unsigned long long>(db(ff_to_double_exact(h, l))),
              static_cast<unsigned long long>(db(ff_to_double(h, l))));
}
static void two_sum(float &h, float &l, float v) {
  const float s = h + v;
  const float bb = s - h;
  const float err = (h - (s - bb)) + (v - bb);
  h = s;
  l = l + err;
}

int main() {
  std::mt19937_64 rng(2024);
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  std::uniform_int_distribution<int> ex(-40, 40);
  // accumulations of 1..9 contributions of mixed magnitudes and signs
  for (int t = 0; t < 20000; ++t) {
    float h = 0.f, l = 0.f;
    const int n = 1 + static_cast<int>(rng() % 9);
    const int base = ex(rng);
    for (int k = 0; k < n; ++k)
      two_sum(h, l, std::ldexp(u(rng), base + static_cast<int>(rng() % 12) - 6));
    emit(h, l);
  }
  // chosen exponent gaps d = e_h - e_l in [-3, 70], both signs
  for (int t = 0; t < 20000; ++t) {
    const float h = std::ldexp(0.5f + 0.5f * std::fabs(u(rng)), ex(rng)) * (rng() & 1 ? 1.f : -1.f);
    int eh;
    std::frexp(h, &eh);
    const int d = static_cast<int>(rng() % 74) - 3;
    const float l = std::ldexp(0.5f + 0.5f * std::fabs(u(rng)), eh - d) * (rng() & 1 ? 1.f : -1.f);
    emit(h, l);
  }
  // powers of two with a small opposite remainder, all-ones mantissas
  for (int t = 0; t < 2000; ++t) {
    const int e = ex(rng);
    const float h = std::ldexp(1.f, e) * (t & 1 ? 1.f : -1.f);
    const float l = -std::ldexp(0.5f + 0.5f * std::fabs(u(rng)), e - 24 - static_cast<int>(rng() % 30)) *
                    (t & 1 ? 1.f : -1.f);
    emit(h, l);
    const float h2 = fromb((fb(h) & 0xff800000u) | 0x7fffffu);
    emit(h2, -l);
  }
  // edge cases
  const float inf = INFINITY, nan = NAN;
  const float cases[][2] = {{0.f, 0.f}, {-0.f, 0.f}, {0.f, -0.f}, {1e-40f, 0.f}, {1.f, 1e-40f},
                            {-1.f, 1e-40f}, {inf, 0.f}, {-inf, 1.f}, {nan, 0.f}, {1.f, 0.f},
                            {3.f, -1.f}, {1.f, -1.f}, {1e30f, 1e22f}, {1.17549435e-38f, 1e-45f}};
  for (auto &c : cases) emit(c[0], c[1]);
  return 0;
}
