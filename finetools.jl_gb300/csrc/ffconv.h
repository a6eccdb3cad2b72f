// Float-float (h + l, two FP32 words) to FP64 without the FP64 pipe: the
// mixed path's final conversion of each CSR value.  GB300's FP64 pipe (and
// its FP32 <-> FP64 conversions) runs at a small fraction of the integer and
// FP32 rates, so the conversion works on the bit patterns.  The file is
// also compiled by the host compiler (tests/ffconv_check.cpp checks both
// routines against exact rational arithmetic).
#pragma once

#include <cmath>
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
FEGPU_HD inline float ffrom(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
FEGPU_HD inline float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
// nearest integer, ties to even (|x| < 2^31)
FEGPU_HD inline int32_t f2i_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(x);
#else
  return static_cast<int32_t>(std::nearbyint(x));  // default rounding mode
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

// (h + l) rounded to FP64 (nearest, ties to even) in about 20 integer
// operations, one FP32 multiply and one float-to-integer conversion for the
// common case.  After renormalisation |l| <= ulp_32(h) / 2, so the exact sum
// is h's FP64 image (24-bit mantissa at the top of the 52-bit field, low 29
// bits zero) plus c_f units of its last place, c_f = l * 2^(179 - e_h),
// |c_f| <= 2^28.  The scaling by a power of two (carrying h's sign, so that a
// positive c_f grows the magnitude) is exact; rounding c_f to the nearest
// integer (ties to even: the parity of the result's last bit is c's) and
// adding it to the bit pattern rounds the sum once.  An addition cannot carry
// out of the free bits; when h is a power of two and l lowers its magnitude
// the sum lies in the binade below, whose units are half as large: c_f is
// then taken at twice the scale and the borrow lands on the right pattern.
// Other inputs (zero, subnormal or tiny h with e_h < 53, inf/nan) take
// ff_to_double_exact.
FEGPU_HD inline double ff_to_double(float h0, float l0) {
  using namespace ffconv;
  float h = h0, l = l0;
  renormalise(h, l);
  const uint32_t hb = fbits(h), lb = fbits(l);
  const uint32_t eh = (hb >> 23) & 0xffu;
  if (eh - 53u > 201u) return ff_to_double_exact(h0, l0);
  const uint32_t down = ((hb & 0x7fffffu) == 0u && ((hb ^ lb) >> 31) != 0u) ? 1u : 0u;
  const float scale = ffrom(((306u - eh + down) << 23) | (hb & 0x80000000u));
  const int32_t c = f2i_rn(fmul(l, scale));
  const uint64_t mag = (static_cast<uint64_t>(((hb & 0x7fffffffu) >> 3) + (896u << 20)) << 32) |
                       static_cast<uint64_t>(hb << 29);
  const uint64_t D = mag + static_cast<uint64_t>(static_cast<int64_t>(c));
  return dfrom(D | (static_cast<uint64_t>(hb >> 31) << 63));
}

}  // namespace fegpu
