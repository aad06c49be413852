// Divisor table and IEEE-exact division by a table entry (FP64 leapfrog).
//
// Shared by the step kernels (div_tab), the C ABI (build_div_table, at
// handle creation) and the GPU test of the division (tests/div_gpu.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace phono {

// Divisor table of the FP64 leapfrog: for each distinct spacing value b of
// the mesh (and 1.0), entry {b, yh, yl, exact} with yh = RN(1/b),
// yl = RN((1 - b*yh)/b) and exact = 1.0 when two_op_exact(b), at slot
// ((lo ^ hi) * mult) >> shift of b's two 32-bit halves (a hash the host picks
// to be collision-free over the mesh's divisors).  The step divides by b
// through yh + yl (div_tab below), which gives the IEEE quotient; a divisor
// whose slot holds another value takes the IEEE division.
// tab == nullptr: every division is the IEEE one.
struct DivTable {
  const double* tab;  // slots of 4 doubles
  unsigned mult;
  int shift;
};
constexpr int DIV_TABLE_SLOTS_MAX = 4096;  // 128 KB; about 200 distinct divisors fit

// x / b rounded to nearest (the IEEE quotient) from the divisor table entry
// of b: yh = RN(1/b), yl = RN((1 - b*yh)/b),
//   q0 = RN(x*yh + RN(x*yl))  differs from x/b by less than 2^-105 relative
//        (yh + yl is 1/b to about 2^-106, and one rounding of that order
//        follows), so it is within one ulp of x/b; and it is RN(x/b) unless
//        x/b lies within 2^-105 of a rounding midpoint.  The host enumerates,
//        for each divisor, every x that comes that close (a handful per
//        binade, from the odd part of b's significand) and marks b "exact"
//        when q0 rounds all of them correctly (the approach of Brisebarre,
//        Muller and Raina, IEEE Trans. Computers 54(7), 2005): then q0 is the
//        IEEE quotient for every x.
//   Otherwise r = x - q0*b is exact (one FMA, q0 being within one ulp) and
//   q = RN(q0 + r*yh) is RN(x/b) by Markstein's theorem (yh within half an
//        ulp of 1/b, q0 within one ulp of x/b, r exact; P. W. Markstein,
//        IBM J. Res. Dev. 34(1):111-119, 1990).
// The argument needs no underflow or overflow on the way, which holds for
// 2^-800 <= |x| < 2^801 with 2^-40 <= b <= 2^40 (the host enters only such b).
// Other x (zero, tiny, huge, inf, nan) and divisors without an entry take the
// IEEE division, except that a zero returns x*yh, the correctly signed zero.
// Two FP64 operations (four for a divisor that is not exact) against about a
// dozen of a general division; the lookup and the range tests are integer work.
__device__ __forceinline__ double div_tab(double x, double b, const DivTable& d) {
  const unsigned blo = (unsigned)__double2loint(b), bhi = (unsigned)__double2hiint(b);
  const unsigned slot = ((blo ^ bhi) * d.mult) >> d.shift;
  const double2* e = reinterpret_cast<const double2*>(d.tab) + 2 * slot;
  const double2 e0 = __ldg(e);      // b, yh
  const double2 e1 = __ldg(e + 1);  // yl, exact flag (1.0 or 0.0)
  const bool hit = (unsigned)__double2loint(e0.x) == blo && (unsigned)__double2hiint(e0.x) == bhi;
  const unsigned xhi = (unsigned)__double2hiint(x);
  const unsigned ex = (xhi >> 20) & 0x7ffu;  // biased exponent of x
  if (!hit || ex - 223u > 1600u) {
    const bool zero = ((xhi & 0x7fffffffu) | (unsigned)__double2loint(x)) == 0u;
    return (hit && zero) ? __dmul_rn(x, e0.y) : __ddiv_rn(x, b);
  }
  const double q0 = __fma_rn(x, e0.y, __dmul_rn(x, e1.x));
  if (__double2hiint(e1.y) != 0) return q0;
  const double r = __fma_rn(-q0, b, x);
  return __fma_rn(r, e0.y, q0);
}

// Whether q0 = RN(x*yh + RN(x*yl)) is the IEEE quotient x/b for every x (no
// underflow or overflow).  q0 is off x/b by less than 2^-105 relative, so it
// can round the wrong way only where x/b lies that close to a rounding
// midpoint mu.  With b = H * 2^e (H odd) and mu = M * 2^f (M odd, 54 bits),
// x = X * 2^g is that close exactly when H*M = X * 2^D + c with a small
// integer c (|c| <= 4 follows from the bound; 8 are tried) and D the
// alignment of X against H*M: M = c * H^-1 mod 2^D.  Every such x (up to a
// power of two, which scales the quotient exactly) is tried here.  Approach
// of Brisebarre, Muller and Raina (IEEE Trans. Computers 54(7), 2005).
inline bool two_op_exact(double b, double yh, double yl) {
  uint64_t hb;
  std::memcpy(&hb, &b, 8);
  int eh = (int)((hb >> 52) & 0x7ff) - 1075;
  uint64_t H = (hb & ((1ull << 52) - 1)) | (1ull << 52);
  while (!(H & 1)) {
    H >>= 1;
    eh++;
  }
  uint64_t inv = H;  // H^-1 mod 2^64 by Newton iteration
  for (int q = 0; q < 6; q++) inv *= 2 - H * inv;
  for (int D = 50; D <= 54; D++) {
    const uint64_t mask = (1ull << D) - 1;
    for (int c = -8; c <= 8; c++) {
      if (c == 0) continue;
      for (uint64_t M = ((uint64_t)(int64_t)c * inv) & mask; M < (1ull << 54); M += 1ull << D) {
        if (M >= (1ull << 53) && (M & 1)) {
          const unsigned __int128 Xc = (unsigned __int128)H * M - (unsigned __int128)(__int128)c;
          if ((uint64_t)(Xc & mask) == 0) {
            const uint64_t X = (uint64_t)(Xc >> D);
            if (X != 0 && X < (1ull << 53)) {
              const double x = std::ldexp((double)X, D + eh);
              if (std::fma(x, yh, x * yl) != x / b) return false;
            }
          }
        }
        if (D == 54) break;
      }
    }
  }
  return true;
}

// Divisor table: one slot of {b, RN(1/b), RN((1-b*yh)/b), exact} per
// distinct value b of `values` in [2^-40, 2^40] (the FP64 leapfrog passes
// every spacing value and 1.0), exact = 1.0 when two_op_exact(b), at slot ((lo ^ hi) * mult) >> shift
// of b's 32-bit halves; mult and the slot count are searched until no two
// divisors share a slot.  Empty slots hold a bit pattern no divisor has, so
// they never match.  false: no table (too many distinct values), every
// division stays the IEEE one.
inline bool build_div_table(const std::vector<double>& values, std::vector<double>& tbl, unsigned* mult, int* shift) {
  std::vector<uint64_t> keys;
  for (double b : values) {
    if (!(b >= std::ldexp(1.0, -40) && b <= std::ldexp(1.0, 40))) continue;
    uint64_t u;
    std::memcpy(&u, &b, 8);
    keys.push_back(u);
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  auto slot_of = [](uint64_t u, unsigned m, int sh) { return (((unsigned)u ^ (unsigned)(u >> 32)) * m) >> sh; };
  for (int bits = 4; (1 << bits) <= DIV_TABLE_SLOTS_MAX; bits++) {
    if ((size_t)(1 << bits) < 2 * keys.size()) continue;
    const int sh = 32 - bits;
    for (unsigned k = 0; k < 4096; k++) {
      const unsigned m = 0x9E3779B1u + 2u * k * 0x632BE5ABu;  // odd multipliers
      std::vector<char> used((size_t)1 << bits, 0);
      bool ok = true;
      for (uint64_t u : keys) {
        char& c = used[slot_of(u, m, sh)];
        if (c) {
          ok = false;
          break;
        }
        c = 1;
      }
      if (!ok) continue;
      const uint64_t empty = ~0ull;
      double none;
      std::memcpy(&none, &empty, 8);
      tbl.assign((size_t)4 * DIV_TABLE_SLOTS_MAX, none);
      for (uint64_t u : keys) {
        double b;
        std::memcpy(&b, &u, 8);
        const double yh = 1.0 / b;
        double* e = &tbl[(size_t)4 * slot_of(u, m, sh)];
        e[0] = b;
        e[1] = yh;
        e[2] = std::fma(-b, yh, 1.0) / b;  // the remainder 1 - b*yh is exact
        e[3] = two_op_exact(b, yh, e[2]) ? 1.0 : 0.0;
      }
      *mult = m;
      *shift = sh;
      return true;
    }
  }
  return false;
}

}  // namespace phono
