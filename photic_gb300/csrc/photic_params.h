// photic_params.h -- kernel-parameter structs shared by the host set-up
// (photic_host.cpp) and the device code.  Everything a kernel needs is
// passed by value in these structs (the per-band constants of at most 8
// bands fit easily in the kernel-parameter space), so concurrent calls on
// different streams with different configurations never share state.
#pragma once
#include <stdint.h>

namespace photic {

constexpr int kMaxBands = 8;
constexpr int kMaxScenes = 8;
constexpr int kMaxHStarts = 32;
constexpr int kNRefTargets = 5;  // Rrs at 440, 490, 550, 640, 750 nm

// Linear interpolation at a fixed target wavelength, resolved on the host
// from the band wavelengths exactly as interp_1d (model/common.c:298-335)
// chooses its segment: the measured value at band i0 (exact match), or
// y[i0] * (1 - t) + y[i1] * t.
struct InterpPlan {
  int32_t exact;  // 1: return y[i0]
  int32_t i0, i1;
  double t, one_minus_t;
};

// Constants of one scene at its band wavelengths (samodel():521-618).
struct SceneConsts {
  double a0[kMaxBands], a1[kMaxBands], aw[kMaxBands], bbw[kMaxBands];
  double refl[kMaxBands];     // sand bottom reflectance
  double refl_k[3][kMaxBands];  // sand, seagrass, coral (model/samodel.c:464-475)
  double wl[kMaxBands];
  double eS[kMaxBands];       // exp(-0.015 * (lambda - 440)), host libm
  double ratio440[kMaxBands]; // 440 / lambda
  double sec_sun, sec_view, h_tide;
};

// K-penalty constants of samodel_error (model/samodel.c:2696-2732):
// thresholds on min K and 1 / (0.01 + target) for each depth band.
struct KPenalty {
  double k_thr[5];    // K_min thresholds for H < 1, 2, 3, 4, 5
  double inv_t[5];    // 1.0 / (0.01 + target)
};

// A double split into two floats (hi = fl(d), lo = fl(d - hi)), the
// host-side form of the device's double-float constants.
struct DfPair {
  float hi, lo;
};

// Double-float copies of the constants the cost needs (filled on the host
// from the double-precision SceneConsts / FitParams).
struct DfScene {
  DfPair a0[kMaxBands], a1[kMaxBands], aw[kMaxBands], bbw[kMaxBands];
  DfPair refl[kMaxBands], eS[kMaxBands];
  DfPair ln_ratio440[kMaxBands];  // log(440 / lambda)
  DfPair sec_sun, sec_view;
  DfPair plan_t[kNRefTargets], plan_omt[kNRefTargets];
  DfPair x_start_coef;            // 100 * 30 * a_w(640)
  DfPair k_thr[5], inv_t[5];
  DfPair reqmin_n;                // reqmin * n
  DfPair hstarts[kMaxHStarts];
};

struct FitParams {
  int32_t n_bands;
  int32_t kcount, konvge;
  int32_t n_hstarts;
  int32_t layout;
  float nodata;
  double reqmin;
  double early_exit_per_scene;
  double aw640;
  double seed_step_scale;
  double hstarts[kMaxHStarts];
  InterpPlan plan[kNRefTargets];
  KPenalty kp;
};

}  // namespace photic
