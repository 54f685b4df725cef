// photic_fastmath.cuh -- the double-precision exponential and the
// divisions by known divisors of the HOPE cost, written for a part whose
// FP64 pipe is its bottleneck.
//
// On GB300 the FP64 pipe retires about two lanes of DFMA per SM per clock,
// and the cost evaluation is bound by it.  The general routines spend that
// pipe on cases the cost never meets: a general divide takes about nine
// DFMA-pipe slots and the CUDA exp about twenty.  The replacements below
// keep IEEE double results:
//
//  * exp_t -- the table-driven method of P. T. P. Tang, "Table-driven
//    implementation of the exponential function in IEEE floating-point
//    arithmetic", ACM TOMS 15(2), 1989: x = (64 m + j) ln2/64 + r with
//    |r| <= ln2/128, exp(x) = 2^m 2^(j/64) exp(r), 2^(j/64) held as a sum
//    of two doubles and exp(r) - 1 summed from its Taylor series to r^5
//    (truncation below 0.2 ulp).  About 11 FP64 instructions; measured
//    within 1 ulp of glibc's exp everywhere and identical to it on 97 % of
//    arguments (CUDA's exp: 94.6 %).
//  * div_by -- a / b for a divisor fixed in advance, from inv = RN(1/b):
//    q = RN(a inv), the exact remainder r = a - b q by one fused
//    multiply-add, and RN(q + r inv), the correction step of P. Markstein,
//    "Computation of elementary functions on the IBM RISC System/6000
//    processor", IBM J. Res. Dev. 34(1), 1990.  Three FP64 instructions.
//    Checked bit for bit against IEEE division for the divisors the cost
//    and the simplex use (pi, 120 and every integer 1..64) on 2^32 random
//    dividends each, with no mismatch (tests/fastmath_check.cpp).
//  * self_ratio -- q / q of the one-bottom-type share: exactly 1 for every
//    finite non-zero q, NaN otherwise (IEEE 754 division), with no divide.
//
// The header compiles for the host too (g++), so the CPU test runs the very
// code the kernels run.
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define PHOTIC_FM_HD __host__ __device__ __forceinline__
#else
#define PHOTIC_FM_HD inline
#endif

namespace photic {
namespace fm {

// 2^(j/64), j = 0..63, as the double nearest it followed by the double
// nearest the remainder, from 60-digit decimal arithmetic.
#define PHOTIC_EXP2_TABLE \
  { 0x1.0000000000000p+0,  0x0.0p+0,  0x1.02c9a3e778061p+0, -0x1.19083535b085dp-56, \
    0x1.059b0d3158574p+0,  0x1.d73e2a475b465p-55,  0x1.0874518759bc8p+0,  0x1.186be4bb284ffp-57, \
    0x1.0b5586cf9890fp+0,  0x1.8a62e4adc610bp-54,  0x1.0e3ec32d3d1a2p+0,  0x1.03a1727c57b53p-59, \
    0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54,  0x1.1429aaea92de0p+0, -0x1.32fbf9af1369ep-54, \
    0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55,  0x1.1a35beb6fcb75p+0,  0x1.e5b4c7b4968e4p-55, \
    0x1.1d4873168b9aap+0,  0x1.e016e00a2643cp-54,  0x1.2063b88628cd6p+0,  0x1.dc775814a8495p-55, \
    0x1.2387a6e756238p+0,  0x1.9b07eb6c70573p-54,  0x1.26b4565e27cddp+0,  0x1.2bd339940e9d9p-55, \
    0x1.29e9df51fdee1p+0,  0x1.612e8afad1255p-55,  0x1.2d285a6e4030bp+0,  0x1.0024754db41d5p-54, \
    0x1.306fe0a31b715p+0,  0x1.6f46ad23182e4p-55,  0x1.33c08b26416ffp+0,  0x1.32721843659a6p-54, \
    0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54,  0x1.3a7db34e59ff7p+0, -0x1.5e436d661f5e3p-56, \
    0x1.3dea64c123422p+0,  0x1.ada0911f09ebcp-55,  0x1.4160a21f72e2ap+0, -0x1.ef3691c309278p-58, \
    0x1.44e086061892dp+0,  0x1.89b7a04ef80d0p-59,  0x1.486a2b5c13cd0p+0,  0x1.3c1a3b69062f0p-56, \
    0x1.4bfdad5362a27p+0,  0x1.d4397afec42e2p-56,  0x1.4f9b2769d2ca7p+0, -0x1.4b309d25957e3p-54, \
    0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55,  0x1.56f4736b527dap+0,  0x1.9bb2c011d93adp-54, \
    0x1.5ab07dd485429p+0,  0x1.6324c054647adp-54,  0x1.5e76f15ad2148p+0,  0x1.ba6f93080e65ep-54, \
    0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54,  0x1.6623882552225p+0, -0x1.bb60987591c34p-54, \
    0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54,  0x1.6dfb23c651a2fp+0, -0x1.bbe3a683c88abp-57, \
    0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55,  0x1.75feb564267c9p+0, -0x1.0245957316dd3p-54, \
    0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55,  0x1.7e2f336cf4e62p+0,  0x1.05d02ba15797ep-56, \
    0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54,  0x1.868d99b4492edp+0, -0x1.fc6f89bd4f6bap-54, \
    0x1.8ace5422aa0dbp+0,  0x1.6e9f156864b27p-54,  0x1.8f1ae99157736p+0,  0x1.5cc13a2e3976cp-55, \
    0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57,  0x1.97d829fde4e50p+0, -0x1.d185b7c1b85d1p-54, \
    0x1.9c49182a3f090p+0,  0x1.c7c46b071f2bep-56,  0x1.a0c667b5de565p+0, -0x1.359495d1cd533p-54, \
    0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54,  0x1.a9e6b5579fdbfp+0,  0x1.0fac90ef7fd31p-54, \
    0x1.ae89f995ad3adp+0,  0x1.7a1cd345dcc81p-54,  0x1.b33a2b84f15fbp+0, -0x1.2805e3084d708p-57, \
    0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56,  0x1.bcc1e904bc1d2p+0,  0x1.23dd07a2d9e84p-55, \
    0x1.c199bdd85529cp+0,  0x1.11065895048ddp-55,  0x1.c67f12e57d14bp+0,  0x1.2884dff483cadp-54, \
    0x1.cb720dcef9069p+0,  0x1.503cbd1e949dbp-56,  0x1.d072d4a07897cp+0, -0x1.cbc3743797a9cp-54, \
    0x1.d5818dcfba487p+0,  0x1.2ed02d75b3707p-55,  0x1.da9e603db3285p+0,  0x1.c2300696db532p-54, \
    0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54,  0x1.e502ee78b3ff6p+0,  0x1.39e8980a9cc8fp-55, \
    0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54,  0x1.efa1bee615a27p+0,  0x1.dc7f486a4b6b0p-54, \
    0x1.f50765b6e4540p+0,  0x1.9d3e12dd8a18bp-54,  0x1.fa7c1819e90d8p+0,  0x1.74853f3a5931ep-55}

#if defined(__CUDACC__)
static __device__ __align__(16) const double kExp2TabDev[128] = PHOTIC_EXP2_TABLE;
#endif
alignas(16) static const double kExp2TabHost[128] = PHOTIC_EXP2_TABLE;

PHOTIC_FM_HD int64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

PHOTIC_FM_HD double from_bits(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// k 2^52 (the exponent-field increment for a factor 2^k), for negative k too
PHOTIC_FM_HD int64_t shl52(int64_t k) { return (int64_t)((uint64_t)k << 52); }

// exp(x) in IEEE double (Tang's method, see the file header).  The result
// is scaled by adding m to the exponent field; only |x| >= 708 (where the
// result may be subnormal or overflow) and NaN take the slower branch.
PHOTIC_FM_HD double exp_t(double x) {
  const double kInv = 0x1.71547652b82fep+6;    // 64 / ln 2
  const double kShift = 0x1.8p52;              // t = x 64/ln2 + 1.5 2^52 rounds to an integer
  const double kL1 = 0x1.62e4200000000p-7;     // ln2/64 to 21 bits: n kL1 is exact
  const double kL2 = 0x1.fdf473de6af28p-28;    // ln2/64 - kL1
  const double t = fma(x, kInv, kShift);
  const double n = t - kShift;
  const int64_t ni = bits(t) - bits(kShift);   // n as an integer (|n| < 2^51)
  double r = fma(-n, kL1, x);
  r = fma(-n, kL2, r);
  const int j = (int)(ni & 63);
  const int64_t m = ni >> 6;                   // floor(n / 64)
#if defined(__CUDA_ARCH__)
  const double2 T = __ldg(reinterpret_cast<const double2 *>(kExp2TabDev) + j);
  const double th = T.x, tl = T.y;
#else
  const double th = kExp2TabHost[2 * j], tl = kExp2TabHost[2 * j + 1];
#endif
  const double c = fma(fma(fma(r, 1.0 / 120.0, 1.0 / 24.0), r, 1.0 / 6.0), r, 0.5);
  const double p = fma(r * r, c, r);           // exp(r) - 1
  const double y = fma(th, p, tl) + th;        // 2^(j/64) exp(r), in [0.99, 2)
  if ((bits(x) & 0x7fffffffffffffffLL) < 0x4086200000000000LL)  // |x| < 708
    return from_bits(bits(y) + shl52(m));
  if (x != x) return x + x;
  if (x < -746.0) return 0.0;
  if (x > 710.0) return from_bits(0x7ff0000000000000LL);
  // 2^m in two normal factors; the product rounds once (to a subnormal
  // below 2^-1022, to infinity above 2^1024)
  const int64_t m1 = m >> 1, m2 = m - m1;
  return from_bits(bits(y) + shl52(m1)) * from_bits(shl52(1023 + m2));
}

PHOTIC_FM_HD int ilog2(int n) {
#if defined(__CUDA_ARCH__)
  return 31 - __clz(n);
#else
  return 31 - __builtin_clz((unsigned)n);
#endif
}

// a / b for a positive normal b fixed in advance, inv = RN(1 / b)
// (Markstein's correction, see the file header).  A quotient that is zero,
// subnormal, infinite or NaN -- outside the correction's hypotheses, and
// never met by the cost or the simplex in practice -- is divided instead.
PHOTIC_FM_HD double div_by(double a, double b, double inv) {
  const double q = a * inv;
  const int64_t e = (bits(q) >> 52) & 0x7ff;
  if (e == 0 || e == 0x7ff) return a / b;
  const double r = fma(-q, b, a);
  return fma(r, inv, q);
}

// q / q: 1 for finite non-zero q, NaN for zero, infinite or NaN q.
PHOTIC_FM_HD double self_ratio(double q) {
  const int64_t a = bits(q) & 0x7fffffffffffffffLL;
  return (a == 0 || a >= 0x7ff0000000000000LL) ? from_bits(0x7ff8000000000000LL) : 1.0;
}

constexpr double kInvPi = 1.0 / 3.141592653589793;
constexpr double kInv120 = 1.0 / 120.0;

// a / n for a count n > 0: a power of two scales exactly (the product and
// the quotient are the same correctly rounded value), any other count is
// divided.
PHOTIC_FM_HD double div_count(double a, int n) {
  if ((n & (n - 1)) == 0) return a * from_bits(shl52(1023 - ilog2(n)));
  return a / (double)n;
}

}  // namespace fm
}  // namespace photic
