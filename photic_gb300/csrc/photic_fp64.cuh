// photic_fp64.cuh -- the HOPE forward model and the photic cost in IEEE
// double precision, written in the reference's association order.
//
// This translation unit family is compiled with --fmad=false, so no
// multiply-add pair below is fused: every product and sum is rounded
// separately, as in the reference built for x86-64.  Where fused
// multiply-adds are wanted (the FP32 and double-float paths) they are
// written as explicit fma calls.
//
// The exponentials and the divisions by fixed divisors (pi, 120, the band
// count) come from photic_fastmath.cuh: the divisions give the IEEE
// quotient bit for bit with a third of the FP64-pipe work, the exponential
// is within 1 ulp of the host libm's (the reference's) and equal to it on
// 97 % of arguments, against 94.6 % for CUDA's exp.
#pragma once
#include <stdint.h>

#include <type_traits>

#include "photic_fastmath.cuh"
#include "photic_params.h"

namespace photic {

constexpr double kPi = 3.141592653589793;  // model/common.h:19

// Measured-spectrum constants of one pixel and scene that do not change
// during the fit: the Y exponent depends only on the measured
// Rrs(440)/Rrs(490) (model/samodel.c:2897-2902), so pow(440/lambda, Y) is
// evaluated once per pixel instead of once per band evaluation.
template <int NB>
struct PixelF64 {
  double rrs[NB];
  double pw[NB];  // pow(440/lambda, Y)
  double mean;           // mean measured Rrs over the bands
  double r490, r550, r640;
};

// interp_1d at a pre-resolved segment (model/common.c:332-334).
template <int NB>
__device__ __forceinline__ double interp_plan(const InterpPlan &p, const double (&y)[NB]) {
  double y0 = y[0], y1 = y[0];
#pragma unroll
  for (int b = 0; b < NB; b++) {
    if (b == p.i0) y0 = y[b];
    if (b == p.i1) y1 = y[b];
  }
  if (p.exact) return y0;
  return y0 * p.one_minus_t + y1 * p.t;
}

// Per-pixel set-up: Rrs at 440..640 nm with the negative-440 guard
// (model/samodel.c:1785-1799), Y and the spectral mean.
template <int NB>
__device__ __forceinline__ void pixel_setup_f64(const FitParams &fp, const SceneConsts &sc,
                                                const double *r, PixelF64<NB> &px) {
  const int nb = fp.n_bands;
  double tot = 0.0;
#pragma unroll
  for (int b = 0; b < NB; b++) {
    px.rrs[b] = 0.0;
    if (b < nb) {
      px.rrs[b] = r[b];
      tot = tot + px.rrs[b];
    }
  }
  double r440 = interp_plan(fp.plan[0], px.rrs);
  px.r490 = interp_plan(fp.plan[1], px.rrs);
  px.r550 = interp_plan(fp.plan[2], px.rrs);
  px.r640 = interp_plan(fp.plan[3], px.rrs);
  if (r440 < 0.0) r440 = 0.0001;
  double chi = r440 / px.r490;
  double Y = 3.44 * (1.0 - 3.17 * fm::exp_t(-2.01 * chi));
  if (Y < 0.0) Y = 0.0;
  if (Y > 2.5) Y = 2.5;
#pragma unroll
  for (int b = 0; b < NB; b++)
    if (b < nb) px.pw[b] = pow(sc.ratio440[b], Y);
  px.mean = tot / (double)nb;
}

// Depth-dependent K penalty and very-high-K penalty
// (model/samodel.c:2696-2732) for one scene whose min K is K_min.
__device__ __forceinline__ double k_penalty_f64(const KPenalty &kp, double H, double K_min) {
  double e = 0.0;
  int c = -1;
  if (H < 1.0 && K_min < kp.k_thr[0]) c = 0;
  else if (H < 2.0 && K_min < kp.k_thr[1]) c = 1;
  else if (H < 3.0 && K_min < kp.k_thr[2]) c = 2;
  else if (H < 4.0 && K_min < kp.k_thr[3]) c = 3;
  else if (H < 5.0 && K_min < kp.k_thr[4]) c = 4;
  if (c >= 0) {
    double d = 1.0 / (0.01 + K_min) - kp.inv_t[c];
    e = e + 100.0 * (d * d);
  }
  return e;
}

struct CostDetailsF64 {
  double rrs_error, model_error, bottom_albedo, K_min, iod;
  double Rm[kMaxBands];
};

// What a plain evaluation can keep, besides its cost, so that the products
// at the kept optimum (model/samodel.c:2413, 1994-2079) follow from the same
// evaluation: the bands' bottom and total subsurface reflectances and the
// modelled Rrs, the Rrs error, K minimum and albedo.  NoKeep keeps nothing.
struct NoKeep {};
template <int NB>
struct BandKeep {
  double rrs_B[NB], rrs[NB], Rm[NB];
  double E, K_min, qB;
};

// Cost of x = (H, 100B, q, 100P, 100G, 100X) for one scene, one region,
// one bottom type: samodel_error (model/samodel.c:2432-2759) over
// samodel_Rrs (model/samodel.c:2846-2949).  With one region the depth and
// bottom continuity terms are identically zero and SAM is compiled out.
template <bool kDetails, int NB, class Keep = NoKeep>
__device__ __forceinline__ double cost_f64(const FitParams &fp, const SceneConsts &sc,
                                           const PixelF64<NB> &px, const double *x,
                                           CostDetailsF64 *det, Keep *keep = nullptr) {
  constexpr bool kKeep = !std::is_same<Keep, NoKeep>::value;
  const int nb = fp.n_bands;
  const double H = fabs(x[0]);
  const double B = 0.01 * fabs(x[1]);
  const double qa = fabs(x[2]);
  const double q = fm::self_ratio(qa);  // q / sum(q) with one bottom type
  const double P = 0.01 * fabs(x[3]);
  const double G = 0.01 * fabs(x[4]);
  const double X = 0.01 * fabs(x[5]);
  const double lnP = log(P);
  const double qB = q * B;
  double err = 0.0, K_min = 1.0e4, iod = 0.0;
#pragma unroll
  for (int b = 0; b < NB; b++) {
    if (b < nb) {
      double rho = qB * sc.refl[b];
      double a_phi = (sc.a0[b] + sc.a1[b] * lnP) * P;
      double a_g = G * sc.eS[b];
      double a = sc.aw[b] + a_phi + a_g;
      double bb = sc.bbw[b] + X * px.pw[b];
      double u = bb / (a + bb);
      double K = a + bb;
      if (K < 0.0) K = 0.0;
      if (K > 2.5) K = 2.5;
      double rrs_dp = (0.084 + 0.170 * u) * u;
      double DuC = 1.03 * sqrt(1.0 + 2.4 * u);
      double DuB = 1.04 * sqrt(1.0 + 5.4 * u);
      double M = sc.sec_sun + DuC * sc.sec_view;
      double rrs_C = rrs_dp * (1.0 - fm::exp_t(-M * K * H));
      M = sc.sec_sun + DuB * sc.sec_view;
      double rrs_B = fm::div_by(rho, kPi, fm::kInvPi) * fm::exp_t(-M * K * H);
      double rrs = rrs_C + rrs_B;
      double Rm = 0.5 * rrs / (1.0 - 1.5 * rrs);
      double d = Rm - px.rrs[b];
      err = err + d * d;
      if (__double2float_rn(K) != 0.0f && K < K_min) K_min = K;
      if (kDetails) {
        iod = iod + rrs_B / rrs;
        det->Rm[b] = Rm;
      }
      if constexpr (kKeep) {
        keep->rrs_B[b] = rrs_B;
        keep->rrs[b] = rrs;
        keep->Rm[b] = Rm;
      }
    }
  }
  const double E = 100.0 * sqrt(fm::div_count(err, nb)) / px.mean;
  double Ke = k_penalty_f64(fp.kp, H, K_min);
  if (K_min > 0.7) {
    double d = 4.0 * (K_min - 0.7);
    Ke = Ke + 100.0 * (d * d);
  }
  double model = 80.0 * E + 15.0 * Ke;
  model = fm::div_by(model, 120.0, fm::kInv120);
  if constexpr (kKeep) {
    keep->E = E;
    keep->K_min = K_min;
    keep->qB = qB;
  }
  if (kDetails) {
    det->rrs_error = E;
    det->model_error = model;
    det->bottom_albedo = qB;
    det->K_min = K_min == 1.0e4 ? 0.0 : K_min;
    det->iod = 100.0 * iod / (double)nb;
  }
  return model;
}

// The cold start of samodel_optimise_one_bottom_combination
// (model/samodel.c:2249-2353) for one region, one scene, one bottom type;
// the depth slot is filled per start.
template <int NB>
__device__ __forceinline__ void cold_start_f64(const FitParams &fp, const PixelF64<NB> &px,
                                               double *start, double *step) {
  start[1] = 100.0 * 4.0 * px.r490;
  step[1] = 1.5 * start[1];
  start[2] = 1.0;
  step[2] = 0.5 * start[2];
  start[3] = 100.0 * 0.072 * pow(px.r490 / px.r550, -1.7);
  start[4] = 1.5 * start[3];
  start[5] = 100.0 * 30.0 * fp.aw640 * px.r640;
  step[3] = 2.0 * start[3];
  step[4] = 2.0 * start[4];
  step[5] = 2.0 * start[5];
}

// samodel_Rrs (model/samodel.c:2846-2949) as the reference calls it: the
// physical parameters as given (fabs only where the reference takes it),
// Y from the caller's Rrs(440)/Rrs(490).  Returns Rrs; writes K.
__device__ __forceinline__ double forward_band_rho_f64(const SceneConsts &sc, int b, double P,
                                                       double G, double X, double rho, double H,
                                                       double Delta, double pw, double *K_out,
                                                       double *parts = nullptr) {
  const double a_phi = (sc.a0[b] + sc.a1[b] * log(fabs(P))) * fabs(P);
  const double a_g = fabs(G) * sc.eS[b];
  const double a = sc.aw[b] + a_phi + a_g;
  const double bb = sc.bbw[b] + X * pw;
  const double u = bb / (a + bb);
  double K = a + bb;
  if (K < 0.0) K = 0.0;
  if (K > 2.5) K = 2.5;
  *K_out = K;
  const double rrs_dp = (0.084 + 0.170 * u) * u;
  const double DuC = 1.03 * sqrt(1.0 + 2.4 * u);
  const double DuB = 1.04 * sqrt(1.0 + 5.4 * u);
  double M = sc.sec_sun + DuC * sc.sec_view;
  const double rrs_C = rrs_dp * (1.0 - fm::exp_t(-M * K * H));
  M = sc.sec_sun + DuB * sc.sec_view;
  const double rrs_B = fm::div_by(rho, kPi, fm::kInvPi) * fm::exp_t(-M * K * H);
  const double rrs = rrs_C + rrs_B;
  if (parts) {  // the intermediates samodel_Rrs stores in model_data
    parts[0] = rho;
    parts[1] = rrs_dp;
    parts[2] = rrs_B;
    parts[3] = rrs;
  }
  return 0.5 * rrs / (1.0 - 1.5 * rrs) + Delta;
}

// The same with one bottom type: rho = (q B) rho_sand(lambda).
__device__ __forceinline__ double forward_band_f64(const SceneConsts &sc, int b, double P,
                                                   double G, double X, double qB, double H,
                                                   double Delta, double pw, double *K_out,
                                                   double *parts = nullptr) {
  return forward_band_rho_f64(sc, b, P, G, X, qB * sc.refl[b], H, Delta, pw, K_out, parts);
}

// (long)(10 * y) of the local-minimum test (model/asa047.c:438-470).  C
// leaves the conversion of NaN or |v| >= 2^63 undefined; the x86-64
// instruction returns LONG_MIN there, and that result is used here so the
// outcome does not depend on the host the reference ran on.
__device__ __forceinline__ long long trunc10(double y) {
  double v = 10.0 * y;
  if (!(v > -9.2233720368547758e18 && v < 9.2233720368547758e18)) return (long long)(-9223372036854775807LL - 1);
  return (long long)v;
}

}  // namespace photic
