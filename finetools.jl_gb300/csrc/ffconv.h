// Float-float (h + l, two FP32 words) to FP64 with integer arithmetic only:
// the mixed path's final conversion of each CSR value.  GB300's FP64 pipe
// (and its FP32 <-> FP64 conversions) runs at a small fraction of the integer
// and FP32 rates, so the conversion works on the bit patterns.  The file is
// also compiled by the host compiler (tests/ffconv_check.cpp checks both
// routines against exact rational arithmetic).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define FEGPU_HD __host__ __device__
#define FEGPU_NOINLINE __noinline__
#else
#define FEGPU_HD
#define FEGPU_NOINLINE __attribute__((noinline))
#endif

namespace fegpu {
namespace ffconv {

FEGPU_HD inline uint32_t fbits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
FEGPU_HD inline double dfrom(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(u));
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
FEGPU_HD inline float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;  // host builds use -ffp-contract=off (IEEE single)
#endif
}
FEGPU_HD inline float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
FEGPU_HD inline int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(x));
#else
  return __builtin_clzll(x);
#endif
}

// (h, l) -> (fl(h + l), exact remainder): two-sum (Knuth), exact whatever
// the magnitudes, so |l| <= ulp(h) / 2 afterwards.
FEGPU_HD inline void renormalise(float &h, float &l) {
  const float s = fadd(h, l);
  const float bb = fsub(s, h);
  const float err = fadd(fsub(h, fsub(s, bb)), fsub(l, bb));
  h = s;
  l = err;
}

}  // namespace ffconv

// (h + l) rounded to FP64 (nearest, ties to even).  The pair is first
// renormalised (h = fl(h + l), l = the exact remainder), then the exact sum is
// formed as a 64-bit fixed-point integer aligned 37 bits below h's leading
// bit (bits of l further down are truncated: below 2^-60 relative),
// normalised and rounded to 53 bits.  Zero and FP32-subnormal sums give a
// signed zero; inf and nan keep their class.
FEGPU_HD inline FEGPU_NOINLINE double ff_to_double_exact(float h, float l) {
  using namespace ffconv;
  renormalise(h, l);
  uint32_t hb = fbits(h), lb = fbits(l);
  if (((hb >> 23) & 0xffu) == 0xffu) {  // inf / nan sum: keep its class
    const uint64_t nanbit = (hb & 0x7fffffu) ? (1ull << 51) : 0ull;
    return dfrom((static_cast<uint64_t>(hb >> 31) << 63) | (0x7ffull << 52) | nanbit);
  }
  if ((lb & 0x7fffffffu) > (hb & 0x7fffffffu)) {  // keep |h| >= |l|
    const uint32_t t = hb;
    hb = lb;
    lb = t;
  }
  const uint32_t eh = (hb >> 23) & 0xffu;
  if (eh == 0u) return dfrom(static_cast<uint64_t>(hb >> 31) << 63);
  const uint64_t mh = static_cast<uint64_t>((hb & 0x7fffffu) | 0x800000u);
  uint64_t H = mh << 37;
  const uint32_t el = (lb >> 23) & 0xffu;
  if (el != 0u && el != 0xffu) {
    const uint64_t ml = static_cast<uint64_t>((lb & 0x7fffffu) | 0x800000u);
    const int d = static_cast<int>(eh) - static_cast<int>(el);  // >= 0
    uint64_t L = 0;
    if (d <= 37) L = ml << (37 - d);
    else if (d < 37 + 24) L = ml >> (d - 37);
    if ((lb >> 31) == (hb >> 31)) H += L;
    else H -= L;
  }
  if (H == 0) return dfrom(static_cast<uint64_t>(hb >> 31) << 63);
  const int p = 63 - clz64(H);
  uint64_t mant;
  int p2 = p;
  if (p >= 52) {
    const int drop = p - 52;
    mant = drop ? (H >> drop) : H;
    if (drop) {
      const uint64_t rem = H & ((1ull << drop) - 1ull);
      const uint64_t half = 1ull << (drop - 1);
      if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    }
    if (mant >> 53) {
      mant >>= 1;
      ++p2;
    }
  } else {
    mant = H << (52 - p);
  }
  // value = mant * 2^(p2 - 52) * 2^(eh - 127 - 60): FP64 exponent field
  const int64_t E = static_cast<int64_t>(p2) + static_cast<int64_t>(eh) - 187 + 1023;
  if (E <= 0) return dfrom(static_cast<uint64_t>(hb >> 31) << 63);
  return dfrom((static_cast<uint64_t>(hb >> 31) << 63) | (static_cast<uint64_t>(E) << 52) |
               (mant & ((1ull << 52) - 1ull)));
}

// (h + l) as FP64, faithfully (error below one unit in the last place), in
// about 25 integer operations for the common case: after renormalisation l
// is at least 24 binades below h (d = e_h - e_l >= 24), so h's 24-bit
// mantissa fills the top of the FP64 mantissa, whose low 29 bits are free,
// and l adds or subtracts c = m_l * 2^(29 - d) < 2^29 units of the last place
// (bits of l below the last place truncated).  An addition cannot carry out
// of the free bits; a subtraction borrows across h's binade only when h's
// mantissa is zero.  Other inputs (zero, subnormal, inf/nan, d < 24, that
// borrow) take ff_to_double_exact.
FEGPU_HD inline double ff_to_double(float h0, float l0) {
  using namespace ffconv;
  float h = h0, l = l0;
  renormalise(h, l);
  const uint32_t hb = fbits(h), lb = fbits(l);
  const uint32_t eh = (hb >> 23) & 0xffu, el = (lb >> 23) & 0xffu;
  const uint32_t mh = hb & 0x7fffffu;
  const int d = static_cast<int>(eh) - static_cast<int>(el);
  if (eh == 0u || eh == 0xffu || (el != 0u && d < 24)) return ff_to_double_exact(h0, l0);
  const bool same = ((hb ^ lb) >> 31) == 0u;
  uint32_t c = 0u;
  if (el != 0u) {
    const uint32_t ml = (lb & 0x7fffffu) | 0x800000u;
    c = d <= 29 ? (ml << (29 - d)) : (d < 61 ? (ml >> (d - 29)) : 0u);
  }
  if (c != 0u && !same && mh == 0u) return ff_to_double_exact(h0, l0);
  uint64_t D = (static_cast<uint64_t>(eh + 896u) << 52) | (static_cast<uint64_t>(mh) << 29);
  D = same ? (D | c) : (D - c);
  return dfrom(D | (static_cast<uint64_t>(hb >> 31) << 63));
}

}  // namespace fegpu
