// IEEE-754 binary64 addition, subtraction, multiplication, multiplication by
// the constants 3, 1.5 and 4.5, and division by 3, round to nearest even,
// computed with integer instructions.
//
// GB300 issues about 0.5 T FP64 add/mul per second but more than 30 T integer
// operations, and integer instructions issue beside a busy FP64 pipe without
// slowing it. The reference-rounding kernels therefore move a share of their
// FP64 operations onto these routines: each returns exactly the bits of the
// hardware instruction, so the split changes nothing in the results.
//
// Method (IEEE 754-2008 clause 4.3 / 5.4, not any library's code): operands
// are finite normal numbers; significands get their hidden bit and 10 guard
// bits (leading one at bit 62 of a 64-bit word). Addition orders the operands
// by magnitude, aligns the smaller with a sticky right shift (bits shifted out
// are OR-ed into bit 0), adds or subtracts, and renormalises with a
// count-leading-zeros shift. Multiplication forms the 106-bit significand
// product from one 64x64 multiply (high and low words; the low word only
// feeds the sticky bit). Rounding adds half a unit in the last place and
// clears the last bit on an exact tie; packing adds the significand into the
// exponent field so that a carry out of the significand raises the exponent.
// Any other case (zero, subnormal, infinity or NaN operand, exact
// cancellation, a result outside the normal range) is handed to the hardware
// instruction, which defines it.
//
// The host build (g++) of the same code is what the CPU unit test checks
// against the host's own IEEE arithmetic.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define IMX_EMU_FI __device__ __forceinline__
#define IMX_EMU_CLZ(x) __clzll((long long)(x))
#define IMX_EMU_MULHI(a, b) __umul64hi(a, b)
#define IMX_EMU_HW_ADD(a, b) imx::emu::hw_add(a, b)
#define IMX_EMU_HW_SUB(a, b) imx::emu::hw_sub(a, b)
#define IMX_EMU_HW_MUL(a, b) imx::emu::hw_mul(a, b)
#define IMX_EMU_HW_DIV(a, b) imx::emu::hw_div(a, b)
#define IMX_EMU_MIN(a, b) min(a, b)
#else
#include <cstring>
#define IMX_EMU_FI inline
#define IMX_EMU_CLZ(x) ((x) ? __builtin_clzll(x) : 64)
#define IMX_EMU_MULHI(a, b) ((uint64_t)(((unsigned __int128)(a) * (b)) >> 64))
#define IMX_EMU_MIN(a, b) ((a) < (b) ? (a) : (b))
#ifndef IMX_EMU_HW_ADD  // the host test may route the other cases elsewhere
#define IMX_EMU_HW_ADD(a, b) ((a) + (b))
#define IMX_EMU_HW_SUB(a, b) ((a) - (b))
#define IMX_EMU_HW_MUL(a, b) ((a) * (b))
#define IMX_EMU_HW_DIV(a, b) ((a) / (b))
#endif
#endif

namespace imx {
namespace emu {

constexpr uint64_t kFrac = 0x000fffffffffffffull;
constexpr uint64_t kHid = 1ull << 52;
constexpr uint64_t kSign = 1ull << 63;
constexpr uint64_t kMag = ~kSign;

#ifdef __CUDACC__
// The hand-off to the FP64 instruction sits in functions that are never
// inlined: inlined, the compiler would issue the (cheap-looking) instruction
// on every call and select its result, putting all the work back on the FP64
// pipe that the emulation exists to relieve.
static __device__ __noinline__ double hw_add(double a, double b) { return __dadd_rn(a, b); }
static __device__ __noinline__ double hw_sub(double a, double b) { return __dsub_rn(a, b); }
static __device__ __noinline__ double hw_mul(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double hw_div(double a, double b) { return __ddiv_rn(a, b); }
IMX_EMU_FI uint64_t bits(double v) { return (uint64_t)__double_as_longlong(v); }
IMX_EMU_FI double dbl(uint64_t b) { return __longlong_as_double((long long)b); }
#else
inline uint64_t bits(double v) {
  uint64_t b;
  std::memcpy(&b, &v, 8);
  return b;
}
inline double dbl(uint64_t b) {
  double v;
  std::memcpy(&v, &b, 8);
  return v;
}
#endif

// r: significand with its leading one at bit 62 (10 bits below the last kept
// bit); e: biased exponent of the rounded result. Returns the magnitude bits.
IMX_EMU_FI uint64_t round_pack(uint64_t r, int e) {
  const uint32_t rb = (uint32_t)r & 0x3ffu;
  uint64_t q = (r + 0x200u) >> 10;
  q &= ~(uint64_t)(rb == 0x200u);  // exact tie: to even
  return ((uint64_t)(uint32_t)(e - 1) << 52) + q;
}

template <bool SUB>
IMX_EMU_FI double add(double a, double b) {
  const uint64_t ia = bits(a);
  const uint64_t ib = bits(b) ^ (SUB ? kSign : 0ull);
  const bool sw = (ib & kMag) > (ia & kMag);
  const uint64_t x = sw ? ib : ia;  // larger magnitude
  const uint64_t y = sw ? ia : ib;
  const uint32_t ex = (uint32_t)(x >> 52) & 0x7ffu;
  const uint32_t ey = (uint32_t)(y >> 52) & 0x7ffu;
  const uint64_t sx = ((x & kFrac) | kHid) << 10;
  const uint64_t sy0 = ((y & kFrac) | kHid) << 10;
  const uint32_t d = IMX_EMU_MIN(ex - ey, 63u);
  const uint64_t lost = (sy0 << (63u - d)) << 1;  // the bits the alignment drops
  const uint64_t sy = (sy0 >> d) | (uint64_t)(lost != 0);
  const bool sub = ((x ^ y) >> 63) != 0;
  uint64_t r = sub ? sx - sy : sx + sy;
  int e = (int)ex;
  const int lz = IMX_EMU_CLZ(r);
  if (lz == 0) {  // carry out of the addition
    r = (r >> 1) | (r & 1u);
    e += 1;
  } else {
    r <<= (lz - 1);
    e -= lz - 1;
  }
  const bool other = (ey == 0u) | (ex == 0x7ffu) | (r == 0u) | ((uint32_t)(e - 1) >= 0x7fdu);
  if (other) return SUB ? IMX_EMU_HW_SUB(a, b) : IMX_EMU_HW_ADD(a, b);
  return dbl((x & kSign) | round_pack(r, e));
}

IMX_EMU_FI double dadd(double a, double b) { return add<false>(a, b); }
IMX_EMU_FI double dsub(double a, double b) { return add<true>(a, b); }

IMX_EMU_FI double dmul(double a, double b) {
  const uint64_t ia = bits(a), ib = bits(b);
  const uint32_t ea = (uint32_t)(ia >> 52) & 0x7ffu;
  const uint32_t eb = (uint32_t)(ib >> 52) & 0x7ffu;
  const uint64_t ma = ((ia & kFrac) | kHid) << 11;
  const uint64_t mb = ((ib & kFrac) | kHid) << 10;
  // significand product P in [2^104, 2^106); hi:lo = P << 21
  uint64_t hi = IMX_EMU_MULHI(ma, mb);
  uint64_t lo = ma * mb;
  int e = (int)(ea + eb) - 1022;
  if (hi < (1ull << 62)) {
    hi = (hi << 1) | (lo >> 63);
    lo <<= 1;
    e -= 1;
  }
  hi |= (uint64_t)(lo != 0);
  const bool other = ((ea - 1u) >= 0x7feu) | ((eb - 1u) >= 0x7feu) | ((uint32_t)(e - 1) >= 0x7fdu);
  if (other) return IMX_EMU_HW_MUL(a, b);
  return dbl(((ia ^ ib) & kSign) | round_pack(hi, e));
}

// a * (K * 2^S) for K = 3 or 9 (the constants 3, 1.5 and 4.5): the
// significand product is m + (m << 1) or m + (m << 3), at most 57 bits, so it
// is exact before the single rounding.
template <int K, int S>
IMX_EMU_FI double mul_small(double a) {
  static_assert(K == 3 || K == 9, "3 or 9");
  const uint64_t ia = bits(a);
  const uint32_t ea = (uint32_t)(ia >> 52) & 0x7ffu;
  const uint64_t m = (ia & kFrac) | kHid;
  const uint64_t mk = m + (m << (K == 3 ? 1 : 3));
  const int lz = IMX_EMU_CLZ(mk);  // leading one at bit 63 - lz
  const uint64_t r = mk << (lz - 1);
  const int e = (int)ea + 11 - lz + S;
  const bool other = ((ea - 1u) >= 0x7feu) | ((uint32_t)(e - 1) >= 0x7fdu);
  constexpr double c = S >= 0 ? (double)(K << (S >= 0 ? S : 0)) : (double)K / (double)(1 << (S < 0 ? -S : 0));
  if (other) return IMX_EMU_HW_MUL(a, c);
  return dbl((ia & kSign) | round_pack(r, e));
}

// a / 3, correctly rounded. With n = m << 11 (the significand, leading one at
// bit 63), floor(2n / 3) = mulhi(n, (2^65 + 1) / 3) exactly for every 64-bit
// n: the error term n / (3 * 2^64) stays below 1/3 and 2n/3 has a fractional
// part of 0, 1/3 or 2/3. The remainder 2n - 3q (0..2, exact modulo 2^64)
// gives the sticky bit.
IMX_EMU_FI double div3(double a) {
  const uint64_t ia = bits(a);
  const uint32_t ea = (uint32_t)(ia >> 52) & 0x7ffu;
  const uint64_t n = ((ia & kFrac) | kHid) << 11;
  const uint64_t q = IMX_EMU_MULHI(n, 0xAAAAAAAAAAAAAAABull);  // leading one at 62 or 63
  const uint64_t sticky = (uint64_t)(((n << 1) - q * 3u) != 0);
  const bool top = (q >> 63) != 0;
  const uint64_t r = (top ? (q >> 1) | (q & 1u) : q) | sticky;
  const int e = (int)ea - (top ? 1 : 2);
  const bool other = ((ea - 1u) >= 0x7feu) | ((uint32_t)(e - 1) >= 0x7fdu);
  if (other) return IMX_EMU_HW_DIV(a, 3.0);
  return dbl((ia & kSign) | round_pack(r, e));
}

}  // namespace emu
}  // namespace imx
