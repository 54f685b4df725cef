// Host check of photic_fastmath.cuh: the same source the kernels compile,
// built with g++, against glibc's exp and IEEE division.
//
//   fastmath_check <log2 samples per divisor> <log2 exp samples>
//
// Prints one line per check and exits non-zero on any failure:
//  * div_by(a, b, RN(1/b)) == a / b bit for bit, b in {pi, 120, 1..64},
//    random dividends over 2^-60..2^60 plus zeros, subnormals, infinities
//    and NaN;
//  * div_count(a, n) == a / n bit for bit, n in 1..64;
//  * self_ratio(q) == q / q (NaN-ness for the NaN cases);
//  * exp_t within 1 ulp of glibc's exp on [-760, 700] and at the special
//    arguments, identical to it on at least 96 % of arguments.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "photic_fastmath.cuh"

using photic::fm::bits;
using photic::fm::from_bits;

static uint64_t mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

static bool same(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return std::isnan(a) && std::isnan(b);
  return bits(a) == bits(b);
}

// A random double with a uniformly random mantissa and sign, exponent in
// [-60, 60].
static double dividend(uint64_t i) {
  const uint64_t h = mix(i);
  const int64_t e = (int64_t)((h >> 53) % 121) - 60;
  const uint64_t sign = (h >> 52) & 1;
  return from_bits((int64_t)((sign << 63) | ((uint64_t)(1023 + e) << 52) | (mix(h) & 0xFFFFFFFFFFFFFULL)));
}

int main(int argc, char **argv) {
  const int ldiv = argc > 1 ? atoi(argv[1]) : 20;
  const int lexp = argc > 2 ? atoi(argv[2]) : 20;
  int failures = 0;

  const double specials[] = {0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1e-310,
                             INFINITY, -INFINITY, NAN, 1.7976931348623157e308};
  std::vector<double> divisors = {3.141592653589793, 120.0};
  for (int n = 1; n <= 64; n++) divisors.push_back((double)n);
  for (double b : divisors) {
    const double inv = 1.0 / b;
    const int64_t n = (int64_t)1 << ldiv;
    int64_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
    for (int64_t i = 0; i < n; i++) {
      const double a = dividend((uint64_t)i * 0x10001ULL + (uint64_t)bits(b));
      if (!same(photic::fm::div_by(a, b, inv), a / b)) bad++;
    }
    for (double a : specials)
      if (!same(photic::fm::div_by(a, b, inv), a / b)) bad++;
    if (bad) {
      printf("div_by b=%.17g: %" PRId64 " mismatches of %" PRId64 "\n", b, bad, n);
      failures++;
    }
  }
  printf("div_by: %zu divisors x 2^%d dividends checked\n", divisors.size(), ldiv);

  for (int n = 1; n <= 64; n++) {
    int64_t bad = 0;
    for (int64_t i = 0; i < 4096; i++) {
      const double a = std::fabs(dividend((uint64_t)i + 77));
      if (!same(photic::fm::div_count(a, n), a / (double)n)) bad++;
    }
    for (double a : specials)
      if (!same(photic::fm::div_count(a, n), a / (double)n)) bad++;
    if (bad) {
      printf("div_count n=%d: %" PRId64 " mismatches\n", n, bad);
      failures++;
    }
  }
  printf("div_count: n = 1..64 checked\n");

  {
    int64_t bad = 0;
    for (double q : specials)
      if (!same(photic::fm::self_ratio(std::fabs(q)), std::fabs(q) / std::fabs(q))) bad++;
    for (int64_t i = 0; i < 100000; i++) {
      const double q = std::fabs(dividend((uint64_t)i + 5));
      if (!same(photic::fm::self_ratio(q), q / q)) bad++;
    }
    printf("self_ratio: %" PRId64 " mismatches\n", bad);
    if (bad) failures++;
  }

  {
    const int64_t n = (int64_t)1 << lexp;
    int64_t ident = 0, over = 0;
    int64_t maxu = 0;
    double worst = 0.0;
#pragma omp parallel for reduction(+ : ident, over) schedule(static)
    for (int64_t i = 0; i < n; i++) {
      const uint64_t h = mix((uint64_t)i + 99);
      const double u = (double)(h >> 11) * 0x1.0p-53;
      double x;
      switch (i % 4) {
        case 0: x = -760.0 * u; break;      // down to the underflow
        case 1: x = -40.0 * u; break;       // the attenuation range
        case 2: x = -1e-3 * u; break;       // near zero
        default: x = 700.0 * u; break;      // positive arguments
      }
      const double r = std::exp(x), y = photic::fm::exp_t(x);
      const int64_t d = std::llabs(bits(r) - bits(y));
      if (d == 0) ident++;
      if (d > 1) over++;
#pragma omp critical
      if (d > maxu) {
        maxu = d;
        worst = x;
      }
    }
    const double xs[] = {0.0, -0.0, -INFINITY, NAN, -745.2, -745.0, -744.4, -720.0,
                         -708.4, -708.0, -707.9, 708.0, 709.7, 709.8, 710.5, 1e300,
                         -1e300, -1e-300, 1e-300};
    int64_t sbad = 0;
    for (double x : xs) {
      const double r = std::exp(x), y = photic::fm::exp_t(x);
      if (std::isnan(r) ? !std::isnan(y) : std::llabs(bits(r) - bits(y)) > 1) {
        printf("exp_t(%.17g) = %.17g, libm %.17g\n", x, y, r);
        sbad++;
      }
    }
    const double frac = (double)ident / (double)n;
    printf("exp_t: 2^%d arguments, %.5f identical to libm, %" PRId64 " beyond 1 ulp (max %" PRId64
           " ulp at %.17g), %" PRId64 " special mismatches\n",
           lexp, frac, over, maxu, worst, sbad);
    if (over || sbad || frac < 0.96) failures++;
  }
  printf("%s\n", failures ? "FAIL" : "OK");
  return failures ? 1 : 0;
}
