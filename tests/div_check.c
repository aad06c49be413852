/* Check of the divisor-table division of the FP64 leapfrog (div_tab and
 * two_op_exact in phonomena_gb300/csrc/div_table.cuh) against
 * IEEE division on the host.
 *
 * The method: yh = RN(1/h), yl = RN((1 - h*yh)/h); for 2^-800 <= |x| < 2^801
 * q0 = RN(x*yh + RN(x*yl)), which is the quotient itself when h passed the
 * exactness check (every x whose quotient lies within 2^-105 of a rounding
 * midpoint rounds correctly), else r = x - q0*h (FMA, exact) and
 * q = RN(q0 + r*yh) (Markstein's theorem); other x take the division.  Built
 * with -ffp-contract=off so that every operation rounds as written; fma() is
 * the correctly rounded C99 function.
 *
 * Usage: div_check N SEED  -> prints "cases mismatches" and exits 0 when
 * every quotient equals x / h bit for bit (signed zeros included). */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t bits(double x) {
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}
static double from_bits(uint64_t u) {
  double x;
  memcpy(&x, &u, 8);
  return x;
}

typedef struct {
  double h, yh, yl;
  int exact;
} entry_t;

/* the host's exactness check of q0 for divisor h (two_op_exact in api.cu) */
static int two_op_exact(double b, double yh, double yl) {
  uint64_t hb = bits(b);
  int eh = (int)((hb >> 52) & 0x7ff) - 1075;
  uint64_t H = (hb & ((1ull << 52) - 1)) | (1ull << 52);
  while (!(H & 1)) {
    H >>= 1;
    eh++;
  }
  uint64_t inv = H;
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
              const double x = ldexp((double)X, D + eh);
              if (fma(x, yh, x * yl) != x / b) return 0;
            }
          }
        }
        if (D == 54) break;
      }
    }
  }
  return 1;
}

static long long n_exact = 0, n_inexact = 0;
static entry_t make_entry(double h) {
  entry_t d;
  d.h = h;
  d.yh = 1.0 / h;
  d.yl = fma(-h, d.yh, 1.0) / h;
  d.exact = two_op_exact(h, d.yh, d.yl);
  if (d.exact) n_exact++;
  else n_inexact++;
  return d;
}

static double div_entry(double x, const entry_t* d) {
  const unsigned e = (unsigned)(bits(x) >> 52) & 0x7ffu;
  if (e - 223u > 1600u) return x == 0.0 ? x * d->yh : x / d->h;
  const double q0 = fma(x, d->yh, x * d->yl);
  if (d->exact) return q0;
  const double r = fma(-q0, d->h, x);
  return fma(r, d->yh, q0);
}

static uint64_t s[2];
static uint64_t next(void) { /* xorshift128+ */
  uint64_t a = s[0], b = s[1];
  s[0] = b;
  a ^= a << 23;
  s[1] = a ^ b ^ (a >> 17) ^ (b >> 26);
  return s[1] + b;
}
/* random double with biased exponent in [lo, hi] and a random sign */
static double rnd(unsigned lo, unsigned hi) {
  const uint64_t m = next() & ((1ull << 52) - 1);
  const uint64_t e = lo + next() % (hi - lo + 1);
  const uint64_t sg = next() & 1ull;
  return from_bits((sg << 63) | (e << 52) | m);
}

static long long cases = 0, bad = 0;
static void check(double x, const entry_t* d);

/* Quotients within |c| * 2^-107 (relative) of a rounding midpoint, the cases
 * a division method is most likely to round the wrong way.  With h = H * 2^eh
 * (H odd) and a midpoint mu = M * 2^em (M odd, 2^53 <= M < 2^54), pick
 * M = c * H^-1 mod 2^54: then H * M = X * 2^54 + c exactly, so x = X * 2^e
 * is a double and x / h = mu * (1 - c / (H * M)). */
static void hard_cases(const entry_t* d, int cmax) {
  uint64_t hb = bits(d->h);
  int eh = (int)((hb >> 52) & 0x7ff) - 1075;
  uint64_t H = (hb & ((1ull << 52) - 1)) | (1ull << 52);
  while (!(H & 1)) {
    H >>= 1;
    eh++;
  }
  uint64_t inv = H; /* Newton iteration for H^-1 mod 2^64 */
  for (int q = 0; q < 6; q++) inv *= 2 - H * inv;
  const uint64_t mask54 = (1ull << 54) - 1;
  for (int c = -cmax; c <= cmax; c++) {
    if (c == 0) continue;
    const uint64_t M = ((uint64_t)(int64_t)c * inv) & mask54;
    if (M < (1ull << 53) || !(M & 1)) continue;
    const unsigned __int128 P = (unsigned __int128)H * M;
    const unsigned __int128 Xc = P - (unsigned __int128)(__int128)c;
    if ((uint64_t)(Xc & mask54) != 0) continue;
    const uint64_t X = (uint64_t)(Xc >> 54);
    if (X == 0 || X >= (1ull << 53)) continue;
    /* x = X * 2^(54 + eh + em); choose em so that |x| sits in the middle of the range */
    for (int em = -600; em <= 600; em += 300) {
      const double x = ldexp((double)X, 54 + eh + em);
      check(x, d);
      check(-x, d);
    }
  }
}
static void check(double x, const entry_t* d) {
  const double want = x / d->h, got = div_entry(x, d);
  cases++;
  if (isnan(want) ? !isnan(got) : bits(want) != bits(got)) {
    if (bad < 10) printf("mismatch: x=%a h=%a want=%a got=%a\n", x, d->h, want, got);
    bad++;
  }
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  s[0] = 0x9e3779b97f4a7c15ull ^ (uint64_t)(argc > 2 ? atoll(argv[2]) : 1);
  s[1] = 0xbf58476d1ce4e5b9ull;
  for (int q = 0; q < 20; q++) next();
  double hs[256];
  const int NH = 256;
  int nh = 0;
  const double fixed[] = {1e-5, 1.0, 0x1p-17, 0.1, 3.0, 1e-3, 2.5e-6, 0x1.fffffffffffffp-1, 0x1.0000000000001p0,
                          0x1p-40, 0x1p40, 0x1.fffffffffffffp39, 7.0, 1.0 / 3.0};
  for (unsigned q = 0; q < sizeof fixed / sizeof fixed[0]; q++) hs[nh++] = fixed[q];
  while (nh < NH) hs[nh++] = fabs(rnd(1023 - 40, 1023 + 39));
  const long long per = n / nh > 0 ? n / nh : 1;
  for (int t = 0; t < nh; t++) {
    const entry_t d = make_entry(hs[t]);
    for (long long q = 0; q < per; q++) {
      /* random x over the whole fast range and its edges */
      check(rnd(223, 1823), &d);
      /* quotients next to a rounding midpoint: x ~ (q + ulp(q)/2) * h */
      const double qq = rnd(1023 - 700, 1023 + 700);
      const long double mid = ((long double)qq + (long double)nextafter(qq, INFINITY)) / 2.0L;
      const double x = (double)(mid * (long double)d.h);
      check(x, &d);
      check(nextafter(x, INFINITY), &d);
      check(nextafter(x, -INFINITY), &d);
      /* exact multiples */
      check(qq * d.h, &d);
    }
    hard_cases(&d, 3000);
    /* values outside the fast range and special values */
    const double special[] = {0.0, -0.0, 0x1p-1074, -0x1p-1074, 0x1p-1022, 0x1p-801, 0x1p-800, 0x1p800, 0x1.fffffffffffffp800,
                              0x1p801, 0x1p1000, INFINITY, -INFINITY, NAN, 1.0, -1.0};
    for (unsigned q = 0; q < sizeof special / sizeof special[0]; q++) check(special[q], &d);
    for (int q = 0; q < 1000; q++) check(rnd(0, 240), &d);
  }
  fprintf(stderr, "divisors: %lld exact (two operations), %lld corrected\n", n_exact, n_inexact);
  printf("%lld %lld\n", cases, bad);
  return bad ? 1 : 0;
}
