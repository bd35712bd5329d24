// Host check of csrc/fp64_emu.cuh: the integer emulation against the host's
// IEEE-754 binary64 add, subtract, multiply, multiply by 3 / 1.5 / 4.5 and
// divide by 3 (round to nearest even), over
// seeded operand pairs from six distributions. With -DCOUNT_OTHER the
// hardware hand-off returns a marker instead, so mismatches count the pairs
// the emulation does not compute itself.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#ifdef COUNT_OTHER
static double other_marker() { return std::nan("7"); }
#define IMX_EMU_HW_ADD(a, b) other_marker()
#define IMX_EMU_HW_SUB(a, b) other_marker()
#define IMX_EMU_HW_MUL(a, b) other_marker()
#define IMX_EMU_HW_DIV(a, b) other_marker()
#endif
#include "fp64_emu.cuh"

using namespace imx::emu;

static uint64_t splitmix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static void pair(uint64_t i, int kind, double& a, double& b) {
  const uint64_t r1 = splitmix(4 * i + 1), r2 = splitmix(4 * i + 2), r3 = splitmix(4 * i + 3);
  const uint64_t sf = kFrac | kSign;
  switch (kind) {
    case 0:  // any bit pattern
      a = dbl(r1);
      b = dbl(r2);
      break;
    case 1: {  // exponent differences 0..70
      const uint64_t ea = 900 + (r3 & 255), d = (r3 >> 8) % 71;
      a = dbl((r1 & sf) | (ea << 52));
      b = dbl((r2 & sf) | ((ea - d) << 52));
      break;
    }
    case 2: {  // near cancellation
      const uint64_t ea = 1000 + (r3 & 63);
      const uint64_t ia = (r1 & kFrac) | (ea << 52);
      const uint64_t flip = r2 & ((1ull << ((r3 >> 8) % 53)) - 1);
      a = dbl(ia);
      b = dbl((ia ^ flip) | kSign);
      if ((r3 >> 20) & 1) b = -b;
      break;
    }
    case 3: {  // lattice Boltzmann magnitudes, +-[2^-32, 2)
      const double x = (double)(r1 >> 11) * 0x1.0p-53, y = (double)(r2 >> 11) * 0x1.0p-53;
      a = std::ldexp(x, -(int)(r3 & 31)) * (((r3 >> 10) & 1) ? -2.0 : 2.0);
      b = std::ldexp(y, -(int)((r3 >> 5) & 31)) * (((r3 >> 11) & 1) ? -2.0 : 2.0);
      break;
    }
    case 4: {  // subnormal, zero, overflow and underflow ranges
      const uint64_t sel = r3 % 6;
      const uint64_t ea = sel < 3 ? (r3 >> 8) % 60 : 2046 - (r3 >> 8) % 60;
      uint64_t eb = sel < 3 ? (r3 >> 16) % 60 : 2046 - (r3 >> 16) % 60;
      if (sel == 1) eb = 1023 - (r3 >> 16) % 1000;
      if (sel == 5) eb = 1023 + (r3 >> 16) % 1000;
      a = dbl((r1 & sf) | (ea << 52));
      b = dbl((r2 & sf) | (eb << 52));
      if (sel == 2) b = 0.0 * b;
      break;
    }
    default: {  // short significands: exact ties occur
      const uint64_t ea = 1000 + (r3 & 31), d = (r3 >> 8) % 60;
      const uint64_t ma = r1 & kFrac & ~((1ull << ((r3 >> 16) % 52)) - 1);
      const uint64_t mb = r2 & kFrac & ~((1ull << ((r3 >> 24) % 52)) - 1);
      a = dbl(ma | (ea << 52) | (r1 & kSign));
      b = dbl(mb | ((ea - d) << 52) | (r2 & kSign));
    }
  }
}

static bool same(double x, double y) { return (x != x && y != y) || bits(x) == bits(y); }

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  long bad[6] = {0, 0, 0, 0, 0, 0};
  for (long i = 0; i < n; ++i) {
    const int kind = (int)(i % 6);
    double a, b;
    pair((uint64_t)i, kind, a, b);
    volatile double va = a, vb = b;  // host arithmetic, not constant-folded
    volatile double c3 = 3.0, c15 = 1.5, c45 = 4.5;
    const double want[7] = {va + vb, va - vb, va * vb, va * c3, va * c15, va * c45, va / c3};
    const double got[7] = {dadd(a, b), dsub(a, b), dmul(a, b), mul_small<3, 0>(a),
                           mul_small<3, -1>(a), mul_small<9, -1>(a), div3(a)};
    for (int op = 0; op < 7; ++op) {
      if (!same(got[op], want[op])) {
#ifndef COUNT_OTHER
        if (bad[kind] < 5)
          std::printf("kind %d op %d a=%a b=%a got %a want %a\n", kind, op, a, b, got[op], want[op]);
#endif
        ++bad[kind];
      }
    }
  }
  std::printf("pairs_per_kind %ld mismatches %ld %ld %ld %ld %ld %ld\n", n / 6, bad[0], bad[1], bad[2],
              bad[3], bad[4], bad[5]);
  return 0;
}
