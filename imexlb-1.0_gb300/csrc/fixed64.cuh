// 64-bit fixed-point numbers for the IMEXLB_FIX64 storage kind.
//
// A population (and every moment and intermediate of the node update) is a
// signed 64-bit integer v standing for v * 2^-60 ("Q3.60": range (-8, 8),
// resolution 8.7e-19). Sums are exact integer additions; products round to
// nearest; conversions to and from IEEE double round to nearest. All of it
// runs on the integer pipes: GB300's FP64 pipe issues about 1.6 operations
// per clock per SM, the integer pipes about 64-128.
//
// The value INT64_MIN is reserved: it marks a slot the boundary program
// fills from outside the reference's arrays, or a node whose state left the
// range the update is valid for, and converts to NaN.
#pragma once

#include <cstdint>

#include "lattice.h"

namespace imx {

constexpr int kFixFrac = 60;                        // fractional bits of a value
constexpr long long kFixInvalid = (long long)(1ull << 63);  // INT64_MIN: NaN

// Storage type of the population buffers of the fixed-point kind.
struct alignas(8) Fix64 {
  long long v;
};

#if defined(__CUDACC__)

// IEEE double -> Q3.60, rounded to nearest (ties away from zero). |x| >= 8,
// infinities and NaN give kFixInvalid. Exponent e of x: the significand m
// (53 bits with the hidden one) stands for m * 2^(e-1075), so the fixed value
// is m * 2^(e-1015): a left shift by up to 10, or a rounded right shift.
__device__ __forceinline__ long long fix_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffu);
  const unsigned long long m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const int sh = e - 1015;
  const int ls = sh > 0 ? (sh > 10 ? 10 : sh) : 0;  // e > 1025 is invalid anyway
  const int rs0 = -sh;
  const int rs = rs0 < 0 ? 0 : (rs0 > 63 ? 63 : rs0);
  const unsigned long long half = rs > 0 ? (1ull << (rs - 1)) : 0ull;
  unsigned long long r = ((m << ls) + half) >> rs;
  if (rs0 > 63) r = 0ull;  // below 2^-61 in magnitude (zero and subnormals too)
  const long long sr = (long long)r;
  const long long v = (b >> 63) ? -sr : sr;
  return e > 1025 ? kFixInvalid : v;
}

// Q3.60 -> IEEE double, rounded to nearest even (kFixInvalid -> NaN).
__device__ __forceinline__ double fix_to_double(long long v) {
  const unsigned long long s = (unsigned long long)(v >> 63);  // 0 or all ones
  const unsigned long long a = ((unsigned long long)v ^ s) - s;
  const int lz = __clzll((long long)(a | 1ull));  // a == 0 handled below
  const unsigned long long n = a << lz;            // leading one at bit 63
  unsigned long long mant = n >> 11;               // 53 bits with the hidden one
  const unsigned rem = (unsigned)(n & 0x7ffu);
  mant += (rem + (unsigned)(mant & 1ull) + 0x3ffu) >> 11;
  // the leading one has weight 2^(3-lz): biased exponent 1026-lz, and the
  // hidden one of mant adds 1 to the field (also when rounding carries)
  unsigned long long bits = ((unsigned long long)(1025 - lz) << 52) + mant;
  bits = a == 0ull ? 0ull : (bits | (s << 63));
  if (v == kFixInvalid) bits = 0x7ff8000000000000ull;
  return __longlong_as_double((long long)bits);
}

// round(a * k / 2^63): a value a in Q3.60 times a factor k in Q0.63
// (|k| < 1) gives Q3.60; with a in Q.62 and k in Q.60 it gives Q.59. The
// 128-bit product is exact; adding 2^62 before the shift rounds to nearest.
__device__ __forceinline__ long long fix_mul(long long a, long long k) {
  long long hi = __mul64hi(a, k);
  const unsigned long long lo = (unsigned long long)a * (unsigned long long)k;
  const unsigned long long lo2 = lo + (1ull << 62);
  hi += lo2 < lo ? 1 : 0;
  return (long long)(((unsigned long long)hi << 1) | (lo2 >> 63));
}

// |v| < 2^bits (v's top 64-bits bits are all equal)
__device__ __forceinline__ bool fix_below(long long v, int bits) {
  const long long t = v >> bits;
  return t == 0 || t == -1;
}

#endif  // __CUDACC__

}  // namespace imx
