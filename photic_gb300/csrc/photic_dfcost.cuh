// photic_dfcost.cuh -- the photic cost in double-float arithmetic.
//
// Same model and the same sequence of operations as cost_f64
// (photic_fp64.cuh, after samodel_error / samodel_Rrs in
// model/samodel.c:2432-2949), evaluated in double-float (about 48 bits) on
// the FP32 pipes.  Results agree with the double-precision cost to a few
// 1e-14 relative; the Nelder-Mead decisions taken on them therefore agree
// with the FP64 reference except where two costs tie to that level.
#pragma once
#include <stdint.h>

#include "photic_df64.cuh"
#include "photic_dftab.h"
#include "photic_params.h"

namespace photic {

__device__ __forceinline__ df64 dp(const DfPair &p) { return df64{p.hi, p.lo}; }

// Compile-time double-float constant.
struct DfC {
  float hi, lo;
  __host__ __device__ constexpr DfC(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};
#define DFK(d) (df64{DfC(d).hi, DfC(d).lo})

__device__ __forceinline__ df64 dexp(df64 a) { return df_exp(a, kExpTabHi, kExpTabLo); }
__device__ __forceinline__ df64 dlog(df64 a) { return df_log(a, kExpTabHi, kExpTabLo); }

template <int NB>
struct PixelDF {
  df64 rrs[NB];
  df64 pw[NB];  // (440/lambda)^Y
  df64 mean;
  df64 r490, r550, r640;
};

template <int NB>
__device__ __forceinline__ df64 interp_plan_df(const InterpPlan &p, const DfPair &t,
                                               const DfPair &omt, const df64 (&y)[NB]) {
  df64 y0 = y[0], y1 = y[0];
#pragma unroll
  for (int b = 0; b < NB; b++) {
    if (b == p.i0) y0 = y[b];
    if (b == p.i1) y1 = y[b];
  }
  if (p.exact) return y0;
  return df_add(df_mul(y0, dp(omt)), df_mul(y1, dp(t)));
}

template <int NB>
__device__ __forceinline__ void pixel_setup_df(const FitParams &fp, const DfScene &ds,
                                               const float *r, PixelDF<NB> &px) {
  const int nb = fp.n_bands;
  df64 tot = df64{0.0f, 0.0f};
#pragma unroll
  for (int b = 0; b < NB; b++) {
    px.rrs[b] = df64{0.0f, 0.0f};
    if (b < nb) {
      px.rrs[b] = df64{r[b], 0.0f};
      tot = df_add_f(tot, r[b]);
    }
  }
  df64 r440 = interp_plan_df<NB>(fp.plan[0], ds.plan_t[0], ds.plan_omt[0], px.rrs);
  px.r490 = interp_plan_df<NB>(fp.plan[1], ds.plan_t[1], ds.plan_omt[1], px.rrs);
  px.r550 = interp_plan_df<NB>(fp.plan[2], ds.plan_t[2], ds.plan_omt[2], px.rrs);
  px.r640 = interp_plan_df<NB>(fp.plan[3], ds.plan_t[3], ds.plan_omt[3], px.rrs);
  if (df_lt(r440, df64{0.0f, 0.0f})) r440 = DFK(0.0001);
  df64 chi = df_div(r440, px.r490);
  df64 Y = df_mul(DFK(3.44), df_add_f(df_neg(df_mul(DFK(3.17), dexp(df_mul(DFK(-2.01), chi)))),
                                      1.0f));
  if (df_lt(Y, df64{0.0f, 0.0f})) Y = df64{0.0f, 0.0f};
  if (df_lt(df64{2.5f, 0.0f}, Y)) Y = df64{2.5f, 0.0f};
#pragma unroll
  for (int b = 0; b < NB; b++)
    if (b < nb) px.pw[b] = dexp(df_mul(Y, dp(ds.ln_ratio440[b])));
  px.mean = df_div_f(tot, (float)nb);
}

struct CostDetailsDF {
  df64 rrs_error, model_error, bottom_albedo, K_min, iod;
};

template <bool kDetails, int NB>
__device__ __forceinline__ df64 cost_df(const FitParams &fp, const DfScene &ds,
                                        const PixelDF<NB> &px, const df64 *x,
                                        CostDetailsDF *det) {
  const int nb = fp.n_bands;
  const df64 c001 = DFK(0.01);
  const df64 H = df_abs(x[0]);
  const df64 B = df_mul(c001, df_abs(x[1]));
  const float qa = fabsf(x[2].hi);
  // q / sum(q) with one bottom type: 1, or NaN when q is exactly zero
  const df64 qB = (qa == 0.0f || qa != qa) ? df64{__int_as_float(0x7fffffff), 0.0f} : B;
  const df64 P = df_mul(c001, df_abs(x[3]));
  const df64 G = df_mul(c001, df_abs(x[4]));
  const df64 X = df_mul(c001, df_abs(x[5]));
  const df64 lnP = dlog(P);
  df64 err = df64{0.0f, 0.0f}, K_min = df64{1.0e4f, 0.0f}, iod = df64{0.0f, 0.0f};
  // One band per trip: the double-float exp/div/sqrt sequences are long, and
  // unrolling the band loop multiplies the code beyond the instruction cache.
#pragma unroll 1
  for (int b = 0; b < nb; b++) {
    {
      df64 rho = df_mul(qB, dp(ds.refl[b]));
      df64 a_phi = df_mul(df_add(dp(ds.a0[b]), df_mul(dp(ds.a1[b]), lnP)), P);
      df64 a_g = df_mul(G, dp(ds.eS[b]));
      df64 a = df_add(df_add(dp(ds.aw[b]), a_phi), a_g);
      df64 bb = df_add(dp(ds.bbw[b]), df_mul(X, px.pw[b]));
      df64 apb = df_add(a, bb);
      df64 u = df_div(bb, apb);
      df64 K = apb;
      if (K.hi < 0.0f) K = df64{0.0f, 0.0f};
      if (df_lt(df64{2.5f, 0.0f}, K)) K = df64{2.5f, 0.0f};
      df64 rrs_dp = df_mul(df_add(DFK(0.084), df_mul(DFK(0.170), u)), u);
      df64 DuC = df_mul(DFK(1.03), df_sqrt(df_add_f(df_mul(DFK(2.4), u), 1.0f)));
      df64 DuB = df_mul(DFK(1.04), df_sqrt(df_add_f(df_mul(DFK(5.4), u), 1.0f)));
      df64 KH = df_mul(K, H);
      df64 M = df_add(dp(ds.sec_sun), df_mul(DuC, dp(ds.sec_view)));
      df64 e1 = dexp(df_neg(df_mul(M, KH)));
      df64 rrs_C = df_mul(rrs_dp, df_add_f(df_neg(e1), 1.0f));
      M = df_add(dp(ds.sec_sun), df_mul(DuB, dp(ds.sec_view)));
      df64 e2 = dexp(df_neg(df_mul(M, KH)));
      df64 rrs_B = df_mul(df_mul(rho, DFK(1.0 / 3.141592653589793)), e2);
      df64 rrs = df_add(rrs_C, rrs_B);
      df64 Rm = df_div(df_mul_f(rrs, 0.5f), df_add_f(df_neg(df_mul_f(rrs, 1.5f)), 1.0f));
      df64 d = df_sub(Rm, px.rrs[b]);
      err = df_add(err, df_mul(d, d));
      if (K.hi != 0.0f && df_lt(K, K_min)) K_min = K;
      if (kDetails) iod = df_add(iod, df_div(rrs_B, rrs));
    }
  }
  const df64 E = df_div(df_mul_f(df_sqrt(df_div_f(err, (float)nb)), 100.0f), px.mean);
  df64 Ke = df64{0.0f, 0.0f};
  {
    int c = -1;
    // thresholds compared in double-float
    if (df_lt(H, df64{1.0f, 0.0f}) && df_lt(K_min, dp(ds.k_thr[0]))) c = 0;
    else if (df_lt(H, df64{2.0f, 0.0f}) && df_lt(K_min, dp(ds.k_thr[1]))) c = 1;
    else if (df_lt(H, df64{3.0f, 0.0f}) && df_lt(K_min, dp(ds.k_thr[2]))) c = 2;
    else if (df_lt(H, df64{4.0f, 0.0f}) && df_lt(K_min, dp(ds.k_thr[3]))) c = 3;
    else if (df_lt(H, df64{5.0f, 0.0f}) && df_lt(K_min, dp(ds.k_thr[4]))) c = 4;
    if (c >= 0) {
      DfPair it = ds.inv_t[0];
#pragma unroll
      for (int i = 1; i < 5; i++)
        if (i == c) it = ds.inv_t[i];
      df64 dd = df_sub(df_div(df64{1.0f, 0.0f}, df_add(DFK(0.01), K_min)), dp(it));
      Ke = df_mul_f(df_mul(dd, dd), 100.0f);
    }
    if (df_lt(DFK(0.7), K_min)) {
      df64 dd = df_mul_f(df_sub(K_min, DFK(0.7)), 4.0f);
      Ke = df_add(Ke, df_mul_f(df_mul(dd, dd), 100.0f));
    }
  }
  df64 model = df_add(df_mul_f(E, 80.0f), df_mul_f(Ke, 15.0f));
  model = df_div_f(model, 120.0f);
  if (kDetails) {
    det->rrs_error = E;
    det->model_error = model;
    det->bottom_albedo = qB;
    det->K_min = (K_min.hi == 1.0e4f) ? df64{0.0f, 0.0f} : K_min;
    det->iod = df_div_f(df_mul_f(iod, 100.0f), (float)nb);
  }
  return model;
}

template <int NB>
__device__ __forceinline__ void cold_start_df(const FitParams &fp, const DfScene &ds,
                                              const PixelDF<NB> &px, df64 *start, df64 *step) {
  (void)fp;
  start[1] = df_mul_f(px.r490, 400.0f);
  step[1] = df_mul_f(start[1], 1.5f);
  start[2] = df64{1.0f, 0.0f};
  step[2] = df64{0.5f, 0.0f};
  // 100 * 0.072 * (r490 / r550)^-1.7
  start[3] = df_mul(DFK(100.0 * 0.072), dexp(df_mul(DFK(-1.7), dlog(df_div(px.r490, px.r550)))));
  start[4] = df_mul_f(start[3], 1.5f);
  start[5] = df_mul(dp(ds.x_start_coef), px.r640);
  step[3] = df_mul_f(start[3], 2.0f);
  step[4] = df_mul_f(start[4], 2.0f);
  step[5] = df_mul_f(start[5], 2.0f);
}

}  // namespace photic
