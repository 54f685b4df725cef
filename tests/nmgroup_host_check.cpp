// Host check of the group-distributed Nelder-Mead state machine
// (photic_nmgroup.cuh) used by the temporal and region kernels: the same
// source, built with g++, with the G lanes of a group run one after the
// other at every step (each lane touches only its own coordinates of the
// shared simplex and its own copy of the vertex costs, so the order of the
// lanes within a step does not matter), against the oracle's nelmin
// (po_nelmin_fn, the restatement of model/asa047.c:10-502) from the same
// start and step.  Every run must give the same minimiser, minimum,
// evaluation count, restart count and fault code, bit for bit, and every
// lane must take the same decisions.
//
//   nmgroup_host_check <runs per case> <seed>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#define __device__
#define __forceinline__ inline
static inline float __double2float_rn(double x) { return (float)x; }
#include "photic_nmgroup.cuh"

extern "C" {
#include "photic_oracle.h"
}

namespace {

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

// The photic cost of one pixel (n = 6) through the oracle.
struct PixelCost {
  double rrs[4];
  static double eval(const double *x, void *ctx) {
    const PixelCost *c = (const PixelCost *)ctx;
    const double wl[4] = {443.0, 482.0, 561.0, 655.0};
    double rm[4], K[4];
    return po_cost(4, wl, 35.0, 0.0, 0.0, c->rrs, x, rm, K);
  }
};

// A smooth coupled cost in n variables with a valley, for the simplex
// sizes of the temporal and region fits.
struct ValleyCost {
  int n;
  double c[64], w[64];
  static double eval(const double *x, void *ctx) {
    const ValleyCost *v = (const ValleyCost *)ctx;
    double e = 0.0, s = 0.0;
    for (int i = 0; i < v->n; i++) {
      const double d = x[i] - v->c[i];
      e = e + v->w[i] * (d * d);
      s = s + x[i];
    }
    for (int i = 0; i + 1 < v->n; i++) {
      const double d = x[i + 1] - x[i] * x[i];
      e = e + 0.05 * (d * d);
    }
    return e + 0.01 * (s * s) / (double)v->n;
  }
};

struct Result {
  std::vector<double> xmin;
  double ynewlo = 0.0;
  int icount = 0, numres = 0, ifault = 0;
  bool lanes_agree = true;
};

// One nelmin call through G lanes of NmGroup<0, C, G, C * G>.
template <int C, int G>
Result run_group(int n, double (*fn)(const double *, void *), void *ctx, const double *start,
                 const double *step, double reqmin, int konvge, int kcount) {
  constexpr int CG = C * G;
  using M = photic::NmGroup<0, C, G, CG>;
  std::vector<double> V((size_t)(n + 1) * CG), Fall((size_t)(n + 1) * G), X(CG);
  std::vector<M> lane(G);
  for (int l = 0; l < G; l++) {
    M &m = lane[l];
    m.clear();
    m.nrt = n;
    m.gl = l;
    m.gmask = 0;
    m.V = V.data();
    m.Fv = Fall.data() + l;
    m.X = X.data();
    for (int t = 0; t < C; t++)
      if (m.own(t)) {
        m.start[t] = start[m.coord(t)];
        m.step[t] = step[m.coord(t)];
      }
    m.begin(reqmin * (double)n, konvge, kcount);
  }
  Result r;
  for (long guard = 0; guard < 10000000; guard++) {
    const double y = fn(X.data(), ctx);
    int done = -1;
    for (int l = 0; l < G; l++) {
      const int d = lane[l].step_machine(y) ? 1 : 0;
      if (done < 0) done = d;
      else if (d != done) r.lanes_agree = false;
    }
    if (done == 1) break;
  }
  r.xmin.assign(n, 0.0);
  for (int l = 0; l < G; l++)
    for (int t = 0; t < C; t++)
      if (lane[l].own(t)) r.xmin[lane[l].coord(t)] = lane[l].xmin[t];
  const M &m0 = lane[0];
  r.ynewlo = Fall[(size_t)m0.lo * G + 0];
  r.icount = m0.icount;
  r.numres = m0.numres;
  r.ifault = m0.ifault;
  for (int l = 1; l < G; l++) {
    const M &m = lane[l];
    if (m.icount != m0.icount || m.numres != m0.numres || m.ifault != m0.ifault || m.lo != m0.lo ||
        memcmp(&Fall[(size_t)m.lo * G + l], &r.ynewlo, sizeof(double)) != 0)
      r.lanes_agree = false;
  }
  return r;
}

}  // namespace

namespace {

int failures = 0, runs = 0;
long long evals = 0;

bool same_bits(double a, double b) { return memcmp(&a, &b, sizeof a) == 0; }

template <int C, int G>
void check(const char *label, int n, double (*fn)(const double *, void *), void *ctx,
           const double *start, const double *step, double reqmin, int konvge, int kcount) {
  double xo[64], yo;
  int io, ro, fo;
  po_nelmin_fn(fn, ctx, n, start, step, reqmin, konvge, kcount, xo, &yo, &io, &ro, &fo);
  const Result r = run_group<C, G>(n, fn, ctx, start, step, reqmin, konvge, kcount);
  bool ok = r.lanes_agree && r.icount == io && r.numres == ro && r.ifault == fo &&
            same_bits(r.ynewlo, yo);
  for (int i = 0; i < n; i++) ok = ok && same_bits(r.xmin[i], xo[i]);
  runs++;
  evals += r.icount;
  if (!ok) {
    if (failures < 8)
      printf("%s n=%d G=%d C=%d: group icount %d numres %d ifault %d y %.17g lanes %d / "
             "oracle %d %d %d %.17g\n",
             label, n, G, C, r.icount, r.numres, r.ifault, r.ynewlo, (int)r.lanes_agree, io, ro,
             fo, yo);
    failures++;
  }
}

}  // namespace

int main(int argc, char **argv) {
  const int nruns = argc > 1 ? atoi(argv[1]) : 20;
  const uint64_t seed = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  uint64_t s = seed * 104729 + 3;
  const double wl[4] = {443.0, 482.0, 561.0, 655.0};
  std::vector<float> rrs_f((size_t)nruns * 4);
  std::vector<double> truth((size_t)nruns * 16);
  po_generate_single(seed, 0, nruns, 4, wl, 35.0, 0.0, 0.0, 2.0e-4, -9999.0f, rrs_f.data(),
                     truth.data());
  const double rel[6] = {1.25, 1.5, 0.5, 2.0, 2.0, 2.0};
  for (int k = 0; k < nruns; k++) {
    // the photic cost, n = 6: one slot per lane (G = 8) and two slots (G = 4)
    PixelCost pc;
    for (int b = 0; b < 4; b++) pc.rrs[b] = rrs_f[(size_t)k * 4 + b];
    double start[64], step[64];
    const double st6[6] = {unif(s, 1.0, 40.0), unif(s, 5.0, 50.0), 1.0, unif(s, 0.5, 10.0),
                           unif(s, 0.5, 20.0), unif(s, 0.1, 5.0)};
    for (int i = 0; i < 6; i++) {
      start[i] = st6[i];
      step[i] = rel[i] * st6[i];
    }
    const double reqmin = k % 2 ? 1.0e-2 : 1.0e-10;
    const int kcount = k % 2 ? 5000 : 2000;
    check<1, 8>("pixel", 6, PixelCost::eval, &pc, start, step, reqmin, 100, kcount);
    check<2, 4>("pixel", 6, PixelCost::eval, &pc, start, step, reqmin, 100, kcount);
    // valley costs at the temporal (3 + 3k, 1 + 4k) and region (3R + 3)
    // simplex sizes
    const int sizes[6] = {9, 17, 21, 27, 30, 33};
    for (int si = 0; si < 6; si++) {
      ValleyCost vc;
      vc.n = sizes[si];
      for (int i = 0; i < vc.n; i++) {
        vc.c[i] = unif(s, -2.0, 2.0);
        vc.w[i] = unif(s, 0.5, 3.0);
        start[i] = unif(s, -3.0, 3.0);
        step[i] = unif(s, 0.2, 1.5);
      }
      const double rq = k % 3 == 0 ? 1.0e-10 : (k % 3 == 1 ? 1.0e-6 : 1.0e-2);
      const int kc = 400 + 40 * vc.n;
      // a group holds C * G >= n coordinates, as the kernels size it
      if (vc.n <= 32) check<1, 32>("valley", vc.n, ValleyCost::eval, &vc, start, step, rq, 5, kc);
      if (vc.n <= 32) check<2, 16>("valley", vc.n, ValleyCost::eval, &vc, start, step, rq, 5, kc);
      check<3, 16>("valley", vc.n, ValleyCost::eval, &vc, start, step, rq, 5, kc);
      if (vc.n <= 24) check<3, 8>("valley", vc.n, ValleyCost::eval, &vc, start, step, rq, 5, kc);
    }
  }
  printf("nelmin runs %d, evaluations %lld, mismatches %d\n", runs, evals, failures);
  printf("%s\n", failures ? "FAIL" : "OK");
  return failures ? 1 : 0;
}
