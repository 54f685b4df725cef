// Host check of the device Nelder-Mead state machine (photic_nm.cuh): the
// same source the kernels compile, built with g++, driven by the oracle's
// cost (po_cost, the restatement of samodel_error), against the oracle's
// nelmin (po_nelmin_pixel, the restatement of model/asa047.c:10-502) from
// the same start and step.  Every pixel must give the same minimiser, the
// same minimum, evaluation count, restart count and fault code, bit for
// bit.
//
//   nm_host_check <pixels> <seed>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#define __device__
#define __forceinline__ inline
#include "photic_fastmath.cuh"
#include "photic_nm.cuh"

extern "C" {
#include "photic_oracle.h"
}

namespace {

// The arithmetic of the FP64 policy of the inversion kernel
// (photic_gb300/csrc/photic_invert.cu, PrecF64).
struct HostF64 {
  using T = double;
  static T zero() { return 0.0; }
  static T one() { return 1.0; }
  static T add(T a, T b) { return a + b; }
  static T sub(T a, T b) { return a - b; }
  static T mul(T a, T b) { return a * b; }
  static T mul2(T a) { return 2.0 * a; }
  static T half(T a) { return a * 0.5; }
  static T scale2(T a, float c) { return a * (double)c; }
  static T div_n(T a, int n) { return photic::fm::div_by(a, (double)n, 1.0 / (double)n); }
  static bool lt(T a, T b) { return a < b; }
  static bool le(T a, T b) { return a <= b; }
  static T eps_step(T s) { return s * 1.0e-6; }
  static T eps_scale() { return 1.0e-6; }
  static long long trunc10(T y) {
    const double v = 10.0 * y;
    if (!(v > -9.2233720368547758e18 && v < 9.2233720368547758e18))
      return (long long)(-9223372036854775807LL - 1);
    return (long long)v;
  }
};

uint64_t mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
double unif(uint64_t &s, double lo, double hi) {
  s = mix(s);
  return lo + (hi - lo) * (double)(s >> 11) * 0x1.0p-53;
}

}  // namespace

int main(int argc, char **argv) {
  const int npix = argc > 1 ? atoi(argv[1]) : 200;
  const uint64_t seed = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  const int nb = 4;
  const double wl[4] = {443.0, 482.0, 561.0, 655.0};
  const double theta_sun = 35.0, theta_view = 0.0;
  std::vector<float> rrs_f((size_t)npix * nb);
  std::vector<double> truth((size_t)npix * 16);
  po_generate_single(seed, 0, npix, nb, wl, theta_sun, theta_view, 0.0, 2.0e-4, -9999.0f,
                     rrs_f.data(), truth.data());
  constexpr int N = 6;
  double V[(N + 1) * N], F[N + 1];
  int mismatches = 0, runs = 0;
  long long evals = 0;
  uint64_t s = seed * 7919 + 17;
  const double tolerances[3][3] = {{1.0e-10, 100, 2000}, {1.0e-2, 100, 5000}, {1.0e-6, 5, 300}};
  for (int p = 0; p < npix; p++) {
    double rrs[4];
    for (int b = 0; b < nb; b++) rrs[b] = rrs_f[(size_t)p * nb + b];
    const double tol[3] = {tolerances[p % 3][0], tolerances[p % 3][1], tolerances[p % 3][2]};
    double start[N] = {unif(s, 1.0, 40.0), unif(s, 5.0, 50.0), 1.0, unif(s, 0.5, 10.0),
                       unif(s, 0.5, 20.0), unif(s, 0.1, 5.0)};
    const double rel[N] = {1.25, 1.5, 0.5, 2.0, 2.0, 2.0};
    double step[N];
    for (int i = 0; i < N; i++) step[i] = rel[i] * start[i];
    // oracle
    double xo[N], yo;
    int io, ro, fo;
    po_nelmin_pixel(nb, wl, theta_sun, theta_view, rrs, start, step, tol[0], (int)tol[1],
                    (int)tol[2], xo, &yo, &io, &ro, &fo);
    // device state machine, one lane
    photic::NmLane<N, HostF64, 1> m;
    m.v = V;
    m.f = F;
    for (int i = 0; i < N; i++) {
      m.start[i] = start[i];
      m.step[i] = step[i];
    }
    m.begin(tol[0] * (double)N, (int)tol[1], (int)tol[2]);
    double rm[4], K[4];
    int guard = 0;
    for (;;) {
      const double y = po_cost(nb, wl, theta_sun, theta_view, 0.0, rrs, m.x, rm, K);
      if (m.step_machine(y)) break;
      if (++guard > 1000000) break;
    }
    runs++;
    evals += m.icount;
    bool same = m.icount == io && m.numres == ro && m.ifault == fo &&
                memcmp(&F[m.lo], &yo, sizeof yo) == 0;
    for (int i = 0; i < N; i++) same = same && memcmp(&m.xmin[i], &xo[i], sizeof xo[i]) == 0;
    if (!same) {
      if (mismatches < 5)
        printf("pixel %d: device icount %d numres %d ifault %d y %.17g / oracle %d %d %d %.17g\n",
               p, m.icount, m.numres, m.ifault, F[m.lo], io, ro, fo, yo);
      mismatches++;
    }
  }
  printf("nelmin runs %d, evaluations %lld, mismatches %d\n", runs, evals, mismatches);
  printf("%s\n", mismatches ? "FAIL" : "OK");
  return mismatches ? 1 : 0;
}
