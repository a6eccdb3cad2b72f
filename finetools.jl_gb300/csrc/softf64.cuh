// IEEE 754 binary64 addition with round-to-nearest-even on the 32-bit
// integer units.
//
// GB300 executes FP64 arithmetic at about 2 lane operations per clock per SM
// (a DGEMM reaches 1.1 TFLOP/s on 152 SMs), against 128 lane instructions per
// clock of issue; 64-bit integer instructions run on the same narrow pipe.
// The reference-order element kernels are bound by that pipe, so part of
// their separately rounded additions run here instead, in 32-bit integer
// words only, with results identical bit for bit to the FP64 unit's.
//
// Method (IEEE 754-2019 5.4.1 addition, 4.3.1 roundTiesToEven; the textbook
// guard/round/sticky construction), without branches on the common path:
// order the operands by magnitude, align the smaller significand to the
// larger one's exponent keeping the bits shifted out as a sticky bit, add the
// two-word integers (two's complement of the smaller one when the signs
// differ), normalise (one place right after a carry, clz - 1 places left after
// a cancellation), round the 53-bit significand to nearest with ties to even
// on the 10 bits below it, and pack (a carry out of the rounding increments
// the exponent field).  A zero or subnormal smaller operand is aligned like
// any other (no hidden bit, exponent 1).  A larger operand that is zero,
// subnormal, infinite or NaN, and a result that is zero, subnormal or
// overflows, take the FP64 unit's own addition, called out of line so that it
// is not executed speculatively.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SF_FN __host__ __device__ __forceinline__
#else
#define SF_FN inline
#endif

namespace fegpu {

SF_FN double sf_double(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(u));
#else
  double x;
  std::memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

SF_FN uint64_t sf_bits(double x) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

SF_FN uint32_t sf_hi(double x) {
#ifdef __CUDA_ARCH__
  return static_cast<uint32_t>(__double2hiint(x));
#else
  return static_cast<uint32_t>(sf_bits(x) >> 32);
#endif
}

SF_FN uint32_t sf_lo(double x) {
#ifdef __CUDA_ARCH__
  return static_cast<uint32_t>(__double2loint(x));
#else
  return static_cast<uint32_t>(sf_bits(x));
#endif
}

SF_FN double sf_make(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
#else
  return sf_double((static_cast<uint64_t>(hi) << 32) | lo);
#endif
}

SF_FN int sf_clz32(uint32_t v) {  // 32 for v = 0
#ifdef __CUDA_ARCH__
  return __clz(static_cast<int>(v));
#else
  return v ? __builtin_clz(v) : 32;
#endif
}

// funnel shifts of the 64-bit word (hi:lo): the low word of (hi:lo) >> (s mod
// 32), the high word of (hi:lo) << (s mod 32), and the high word of
// (hi:lo) << min(s, 32)
SF_FN uint32_t sf_shr_w(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lo, hi, s);
#else
  return static_cast<uint32_t>(((static_cast<uint64_t>(hi) << 32) | lo) >> (s & 31u));
#endif
}

SF_FN uint32_t sf_shl_w(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, s);
#else
  return static_cast<uint32_t>((((static_cast<uint64_t>(hi) << 32) | lo) << (s & 31u)) >> 32);
#endif
}

SF_FN uint32_t sf_shl_wc(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
  return __funnelshift_lc(lo, hi, s);
#else
  const uint32_t c = s < 32u ? s : 32u;
  return static_cast<uint32_t>((((static_cast<uint64_t>(hi) << 32) | lo) << c) >> 32);
#endif
}

// (h:l) += (bh:bl) + cin (cin 0 or 1), in two words with a carry chain
SF_FN void sf_add2(uint32_t &h, uint32_t &l, uint32_t bh, uint32_t bl, uint32_t cin) {
#ifdef __CUDA_ARCH__
  asm("add.cc.u32 %0, %0, %2;\n\t"
      "addc.u32 %1, %1, %3;\n\t"
      "add.cc.u32 %0, %0, %4;\n\t"
      "addc.u32 %1, %1, 0;"
      : "+r"(l), "+r"(h)
      : "r"(bl), "r"(bh), "r"(cin));
#else
  const uint64_t s = ((static_cast<uint64_t>(h) << 32) | l) +
                     ((static_cast<uint64_t>(bh) << 32) | bl) + cin;
  h = static_cast<uint32_t>(s >> 32);
  l = static_cast<uint32_t>(s);
#endif
}

#ifdef __CUDACC__
// the FP64 unit's own addition, out of line (special operands and results)
static __device__ __noinline__ double sf_add_hw_dev(double x, double y) { return __dadd_rn(x, y); }
#endif

SF_FN double sf_add_hw(double x, double y) {
#ifdef __CUDA_ARCH__
  return sf_add_hw_dev(x, y);
#else
  volatile double s = x + y;  // one IEEE addition (no contraction on the host)
  return s;
#endif
}

SF_FN double sf_add(double x, double y) {
  const uint32_t xh = sf_hi(x), xl = sf_lo(x), yh = sf_hi(y), yl = sf_lo(y);
  // p: the operand of larger magnitude, q: the other (bit patterns of
  // non-negative doubles order as their values)
  const uint32_t axh = xh & 0x7fffffffu, ayh = yh & 0x7fffffffu;
  const bool sw = (axh < ayh) | ((axh == ayh) & (xl < yl));
  const uint32_t ph = sw ? yh : xh, pl = sw ? yl : xl;
  const uint32_t qh = sw ? xh : yh, ql = sw ? xl : yl;
  const uint32_t ep = (ph >> 20) & 0x7ffu, eq = (qh >> 20) & 0x7ffu;
  // p zero or subnormal (then q too), infinite or NaN
  if (ep - 1u >= 2046u) return sf_add_hw(x, y);
  // significands with the hidden bit at bit 62 (bit 30 of the high word): 10
  // bits below the unit in the last place of the result, one spare bit above;
  // a zero or subnormal q has no hidden bit and the exponent of 1
  const uint32_t ah = sf_shl_w(pl, (ph & 0x000fffffu) | 0x00100000u, 10u), al = pl << 10;
  uint32_t bh = sf_shl_w(ql, (qh & 0x000fffffu) | (eq ? 0x00100000u : 0u), 10u), bl = ql << 10;
  uint32_t d = ep - (eq ? eq : 1u);
  d = d < 63u ? d : 63u;
  // b >> d; the bits shifted out become a sticky bit 0 (b >> 63 is 0: a
  // nonzero q is then all sticky)
  {
    const uint32_t t = bh >> (d & 31u);
    uint32_t sticky;
    if (d < 32u) {
      sticky = sf_shl_wc(0u, bl, 32u - d);
      bl = sf_shr_w(bl, bh, d);
      bh = t;
    } else {
      sticky = bl | sf_shl_wc(0u, bh, 64u - d);
      bl = t;
      bh = 0u;
    }
    bl |= sticky != 0u ? 1u : 0u;
  }
  // a + b, or a - b (two's complement) when the signs differ: a - b >= 0
  const uint32_t sub = (xh ^ yh) >> 31, m = 0u - sub;
  uint32_t h = ah, l = al;
  sf_add2(h, l, bh ^ m, bl ^ m, sub);
  // normalise the top bit to bit 62: one place right after a carry into bit
  // 63, clz - 1 places left after a cancellation (a zero difference gives an
  // exponent below 1: the FP64 unit returns its +0)
  const int lz = (h ? sf_clz32(h) : 32 + sf_clz32(l)) - 1;
  const int e = (h | l) ? static_cast<int>(ep) - lz : 0;
  if (lz < 0) {
    l = (l >> 1) | (h << 31) | (l & 1u);
    h >>= 1;
  } else if (lz < 32) {
    h = sf_shl_w(l, h, static_cast<uint32_t>(lz));
    l <<= lz;
  } else {
    h = l << (lz - 32);
    l = 0u;
  }
  if (static_cast<uint32_t>(e - 1) >= 2046u) return sf_add_hw(x, y);  // zero, subnormal, overflow
  // the 53-bit significand (mh:ml) = (h:l) >> 10, rounded to nearest even on
  // the 10 bits below it
  uint32_t mh = h >> 10, ml = sf_shr_w(l, h, 10u);
  const uint32_t r = l & 0x3ffu;
  const uint32_t up = (r > 0x200u ? 1u : 0u) | ((r == 0x200u ? 1u : 0u) & ml);
  sf_add2(mh, ml, 0u, 0u, up);
  // mh holds the hidden bit: it adds one to the exponent field, and a carry
  // out of the rounding (a significand of 2^53) one more
  const uint32_t rh = (ph & 0x80000000u) + (static_cast<uint32_t>(e - 1) << 20) + mh;
  if ((rh & 0x7ff00000u) == 0x7ff00000u) return sf_add_hw(x, y);  // rounded up to infinity
  return sf_make(rh, ml);
}

}  // namespace fegpu

#undef SF_FN
