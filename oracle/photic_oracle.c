/*
 * photic_oracle.c -- CPU restatement of photic's per-pixel inversion.
 *
 * TEST INFRASTRUCTURE ONLY (see photic_oracle.h).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load this library, and
 * only as the checker or as the timed CPU baseline, never as the product.
 *
 * Every routine below states which reference lines it follows.  The
 * arithmetic is written in the same association order as the reference so
 * that, built with the same compiler flags and libm, it reproduces the
 * reference's results bit for bit (checked against oracle/_ref by
 * tests/test_oracle_vs_reference.py).  The one deliberate departure is the
 * double -> long truncation inside nelmin's local-minimum test
 * (model/asa047.c:438,445,460), whose result for NaN or |x| >= 2^63 is
 * undefined in C: it is pinned here to the x86-64 behaviour (LONG_MIN) so
 * that the oracle agrees with itself on every host.
 */
#include "photic_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#if _OPENMP
#include <omp.h>
#endif

#define PO_PI 3.141592653589793 /* model/common.h:19 */

/* ------------------------------------------------------------------------
 * Spectral tables on the 41-point 400..800 nm grid.  Values are the
 * published tables the reference tabulates in model/samodel.c:105-287:
 * pure-water absorption (Pope & Fry 1997), pure-water backscatter
 * (Morel 1974), Lee's a0/a1 phytoplankton coefficients (Lee 1994) and the
 * eight HYDROLIGHT-averaged bottom reflectance spectra.  They must be equal
 * to the reference's numbers for parity, so they are data, not design.
 * ---------------------------------------------------------------------- */
#define PO_NREF 41
static const double po_ref_wl[PO_NREF] = {
    400, 410, 420, 430, 440, 450, 460, 470, 480, 490, 500, 510, 520, 530,
    540, 550, 560, 570, 580, 590, 600, 610, 620, 630, 640, 650, 660, 670,
    680, 690, 700, 710, 720, 730, 740, 750, 760, 770, 780, 790, 800};
static const double po_aw[PO_NREF] = {
    0.00663, 0.00473, 0.00454, 0.00495, 0.00635, 0.00922, 0.00979, 0.0106, 0.0127,
    0.015,   0.0204,  0.0325,  0.0409,  0.0434,  0.0474,  0.0565,  0.0619, 0.0695,
    0.0896,  0.1351,  0.2224,  0.2644,  0.2755,  0.2916,  0.3108,  0.34,   0.41,
    0.439,   0.465,   0.516,   0.624,   0.827,   1.231,   1.65768, 2.38147, 2.47014,
    2.5045,  2.47509, 2.35431, 2.17654, 2.01226};
static const double po_bbw[PO_NREF] = {
    0.0038,      0.00341552,  0.00307784,  0.00278035,  0.00251749,  0.00228457,
    0.00207763,  0.0018933,   0.0017287,   0.00158138,  0.00144921,  0.00133039,
    0.00122334,  0.00112671,  0.0010393,   0.000960099, 0.000888199, 0.000822817,
    0.000763262, 0.000708928, 0.000659279, 0.000613844, 0.000572204, 0.000533988,
    0.000498868, 0.000466549, 0.00043677,  0.000409298, 0.000383923, 0.000360458,
    0.000338734, 0.000318601, 0.000299921, 0.000282571, 0.000266441, 0.000251431,
    0.000237448, 0.00022441,  0.000212243, 0.000200879, 0.000190254};
static const double po_a0[PO_NREF] = {
    0.684266, 0.778234, 0.86369,  0.960272, 1,        0.96339,  0.931107, 0.869651, 0.788982,
    0.755811, 0.733335, 0.691062, 0.632722, 0.568079, 0.504551, 0.426236, 0.343342, 0.294978,
    0.278405, 0.259509, 0.238935, 0.274531, 0.319712, 0.342135, 0.333133, 0.350196, 0.560974,
    0.843456, 0.74852,  0.4,      0.15,     0.06,     0.026,    0.013,    0.013,    0.013,
    0.013,    0.013,    0.013,    0.013,    0.013};
static const double po_a1[PO_NREF] = {
    0.0205345, 0.0129366, 0.0064013, 0.00168429, 0,         0.00602146, 0.0109083,
    0.0157169, 0.0152315, 0.0255969, 0.0559074,  0.0865174, 0.098141,   0.0968975,
    0.0899322, 0.0780758, 0.0658936, 0.0596445,  0.0581118, 0.0539721,  0.0494872,
    0.057845,  0.0673832, 0.0717643, 0.0684625,  0.0713488, 0.112818,   0.159471,
    0.138835,  0.0811786, 0.03,      0.012,      0.0054,    0.0028,     0.0028,
    0.0028,    0.0028,    0.0028,    0.0028,     0.0028,    0.0028};
/* Bottom table order: sand, seagrass, coral, macrophytes, dark sediment,
 * coral sand, green algae, red algae (model/samodel.c:464-475). */
static const double po_bottom[PO_N_BOTTOM_TYPES][PO_NREF] = {
    {0.634432, 0.654965, 0.682443, 0.712079, 0.74123,  0.769656, 0.802245, 0.827992, 0.854624,
     0.878036, 0.89898,  0.924542, 0.94899,  0.965671, 0.982481, 1.,       1.01237,  1.02994,
     1.04658,  1.07139,  1.08139,  1.08884,  1.09447,  1.09916,  1.10557,  1.10758,  1.101,
     1.08464,  1.08658,  1.12477,  1.17063,  1.20125,  1.21407,  1.22691,  1.23186,  1.24098,
     1.24708,  1.25257,  1.25607,  1.26361,  1.26789},
    {0.542201, 0.538755, 0.543345, 0.550218, 0.550218, 0.562483, 0.606813, 0.607225, 0.63619,
     0.650873, 0.670997, 0.735138, 0.808387, 0.887508, 0.949743, 1.,       1.03488,  1.04312,
     1.03199,  1.00882,  0.95964,  0.903696, 0.85915,  0.848253, 0.830917, 0.807567, 0.785207,
     0.839027, 1.09213,  1.68562,  2.5015,   4.15478,  5.11731,  5.77383,  6.02484,  6.11441,
     6.16467,  6.22648,  6.27581,  6.29811,  6.34481},
    {0.437155, 0.381353, 0.353904, 0.339709, 0.358934, 0.382172, 0.390592, 0.407088, 0.462696,
     0.522577, 0.60409,  0.707443, 0.764575, 0.826841, 0.892756, 1.,       1.15687,  1.3644,
     1.44365,  1.40967,  1.48473,  1.53551,  1.41572,  1.32706,  1.25349,  1.20397,  0.955824,
     0.643935, 0.669901, 1.38703,  2.42848,  3.3846,   3.6429,   3.89712,  4.10336,  4.23733,
     4.32766,  4.37486,  4.43428,  4.47756,  4.52468},
    {0.443737, 0.401082, 0.382427, 0.382427, 0.382427, 0.382427, 0.402497, 0.409674, 0.443211,
     0.44772,  0.494445, 0.620241, 0.755823, 0.882367, 0.973539, 1.,       1.09947,  1.09321,
     1.11723,  1.09127,  1.06283,  1.03064,  0.919521, 0.896435, 0.839186, 0.769511, 0.645607,
     0.60577,  0.743085, 1.1217,   2.17169,  3.27124,  3.47565,  3.3989,   3.48151,  3.59713,
     3.65614,  3.65521,  3.67159,  3.6131,   3.58176},
    {0.57054,  0.564806, 0.583536, 0.596254, 0.616995, 0.640224, 0.669295, 0.691865, 0.722327,
     0.740098, 0.765618, 0.801745, 0.850374, 0.901024, 0.943913, 1.,       1.05834,  1.10294,
     1.13346,  1.17132,  1.20427,  1.20038,  1.16874,  1.16074,  1.14623,  1.14875,  1.03881,
     0.903713, 0.894767, 1.05454,  1.30921,  1.49551,  1.58863,  1.64064,  1.65234,  1.66933,
     1.68055,  1.69243,  1.70471,  1.72121,  1.72876},
    {0.616201, 0.636915, 0.659543, 0.685341, 0.71562,  0.742639, 0.769601, 0.792999, 0.818446,
     0.840791, 0.86273,  0.890834, 0.912898, 0.940877, 0.970795, 1.,       1.03073,  1.05991,
     1.08887,  1.1141,   1.13666,  1.15865,  1.18297,  1.20189,  1.22277,  1.23953,  1.25598,
     1.27532,  1.29161,  1.31127,  1.3302,   1.348,    1.36099,  1.37632,  1.38579,  1.39478,
     1.40298,  1.41371,  1.42261,  1.43402,  1.44206},
    {0.16848,  0.188393, 0.188646, 0.17936,  0.170655, 0.190607, 0.220843, 0.241126, 0.262068,
     0.294282, 0.357834, 0.516557, 0.717781, 0.898626, 0.975598, 1.,       1.00009,  0.946152,
     0.874696, 0.829798, 0.807546, 0.763138, 0.701775, 0.673854, 0.606387, 0.524554, 0.426766,
     0.3044,   0.284069, 0.48541,  0.912011, 1.33421,  1.52307,  1.61754,  1.65643,  1.66741,
     1.66741,  1.66741,  1.66741,  1.66741,  1.66298},
    {1.25032,  1.13331,  1.06326,  1.00005,  0.925705, 0.983453, 1.,       1.,       0.975044,
     0.877564, 0.877766, 0.987416, 1.04918,  1.03747,  1.,       1.,       1.01387,  1.16916,
     1.56137,  2.08995,  2.44941,  2.40749,  2.30252,  2.33337,  2.48719,  2.53279,  2.21543,
     1.72598,  1.80604,  2.72284,  4.35056,  5.67543,  6.32734,  6.72766,  6.90232,  6.98939,
     7.04997,  7.09008,  7.11525,  7.09872,  7.04973}};

/* ------------------------------------------------------------------------
 * Tolerant comparisons in single precision (model/common.c:392-406) and
 * piecewise-linear interpolation with end-segment extrapolation
 * (interp_1d, model/common.c:298-335).  The float arguments are part of the
 * behaviour: doubles are rounded to float before comparing.
 * ---------------------------------------------------------------------- */
static int f_close(float a, float b, float eps) {
  double big = fabs(a) < fabs(b) ? fabs(b) : fabs(a);
  return fabs(a - b) <= big * eps;
}
static int f_le(float a, float b, float eps) { return a < b || f_close(a, b, eps); }
static int f_ge(float a, float b, float eps) { return a > b || f_close(a, b, eps); }

double po_interp_1d(const double *X, const double *Y, int n, double x) {
  double x0 = 0.0, x1 = 1.0, y0 = 0.0, y1 = 0.0, t;
  int i;
  if (f_close(x, X[0], 1.0e-5)) return Y[0];
  if (f_close(x, X[n - 1], 1.0e-5)) return Y[n - 1];
  if (X[0] < X[n - 1] && x < X[0]) {
    x0 = X[0]; x1 = X[1]; y0 = Y[0]; y1 = Y[1];
  } else if (X[n - 1] > X[0] && x > X[n - 1]) {
    x0 = X[n - 2]; x1 = X[n - 1]; y0 = Y[n - 2]; y1 = Y[n - 1];
  } else {
    for (i = 0; i + 1 < n; i++) {
      int up = f_le(X[i], x, 1.0e-5) && f_ge(X[i + 1], x, 1.0e-5);
      int down = f_ge(X[i], x, 1.0e-5) && f_le(X[i + 1], x, 1.0e-5);
      if (up || down) {
        x0 = X[i]; x1 = X[i + 1]; y0 = Y[i]; y1 = Y[i + 1];
        break;
      }
    }
  }
  t = (x - x0) / (x1 - x0);
  return y0 * (1.0 - t) + y1 * t;
}

/* ------------------------------------------------------------------------
 * Scene constants: band-wavelength interpolation of the tables and the
 * subsurface angle secants, as samodel() prepares them
 * (model/samodel.c:505, 534-548, 550-618).
 * ---------------------------------------------------------------------- */
typedef struct {
  int n_bands;
  double wl[PO_MAX_BANDS];
  double a0[PO_MAX_BANDS], a1[PO_MAX_BANDS], aw[PO_MAX_BANDS], bbw[PO_MAX_BANDS];
  double refl[PO_N_BOTTOM_TYPES][PO_MAX_BANDS];
  double sec_sun, sec_view, h_tide, aw640;
} po_scene;

static void scene_init(po_scene *sc, int n_bands, const double *wl, double theta_sun_deg,
                       double theta_view_deg, double h_tide) {
  int b, k;
  double th;
  sc->n_bands = n_bands;
  th = theta_view_deg;
  th *= PO_PI / 180.0;
  sc->sec_view = 1.0 / cos(th);
  th = theta_sun_deg;
  th *= PO_PI / 180.0;
  sc->sec_sun = 1.0 / cos(th);
  sc->h_tide = h_tide;
  sc->aw640 = po_interp_1d(po_ref_wl, po_aw, PO_NREF, 640.0);
  for (b = 0; b < n_bands; b++) {
    double l = wl[b];
    sc->wl[b] = l;
    sc->a0[b] = po_interp_1d(po_ref_wl, po_a0, PO_NREF, l);
    sc->a1[b] = po_interp_1d(po_ref_wl, po_a1, PO_NREF, l);
    sc->bbw[b] = po_interp_1d(po_ref_wl, po_bbw, PO_NREF, l);
    sc->aw[b] = po_interp_1d(po_ref_wl, po_aw, PO_NREF, l);
    for (k = 0; k < PO_N_BOTTOM_TYPES; k++)
      sc->refl[k][b] = po_interp_1d(po_ref_wl, po_bottom[k], PO_NREF, l);
  }
}

void po_band_constants(int n_bands, const double *wl, double theta_sun_deg,
                       double theta_view_deg, double *out) {
  po_scene sc;
  int b;
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, 0.0);
  for (b = 0; b < n_bands; b++) {
    out[b * 8 + 0] = sc.a0[b];
    out[b * 8 + 1] = sc.a1[b];
    out[b * 8 + 2] = sc.aw[b];
    out[b * 8 + 3] = sc.bbw[b];
    out[b * 8 + 4] = sc.refl[0][b];
    out[b * 8 + 5] = sc.sec_sun;
    out[b * 8 + 6] = sc.sec_view;
    out[b * 8 + 7] = sc.aw640;
  }
}

/* ------------------------------------------------------------------------
 * One pixel: its scenes, measured spectra, the interpolated Rrs at
 * 440/490/550/640/750 nm, and the per-evaluation side outputs the
 * reference keeps in model_data.
 * ---------------------------------------------------------------------- */
enum { PO_LAYOUT_REFERENCE = 0, PO_LAYOUT_PER_SCENE_B = 1 };

typedef struct {
  int n_scenes, n_bands, n_bottoms, layout;
  const po_scene *sc[PO_MAX_SCENES];
  double rrs[PO_MAX_SCENES][PO_MAX_BANDS];
  double r440[PO_MAX_SCENES], r490[PO_MAX_SCENES], r550[PO_MAX_SCENES];
  double r640[PO_MAX_SCENES], r750[PO_MAX_SCENES];
  /* side outputs of the latest cost evaluation */
  double Rm[PO_MAX_SCENES][PO_MAX_BANDS], rrs_mod[PO_MAX_SCENES][PO_MAX_BANDS];
  double rrs_bot[PO_MAX_SCENES][PO_MAX_BANDS], K[PO_MAX_SCENES][PO_MAX_BANDS];
  double bottom_albedo, rrs_error, model_error;
} po_pixel;

static int n_params_of(const po_pixel *px) {
  if (px->layout == PO_LAYOUT_PER_SCENE_B) return 1 + 4 * px->n_scenes;
  return 1 + 2 * px->n_bottoms + 3 * px->n_scenes; /* model/samodel.c:1833-1855 */
}

/* Rrs(440..750) of each scene from its measured bands, with the
 * negative-440 guard (model/samodel.c:1785-1799). */
static void pixel_reference_rrs(po_pixel *px) {
  int s;
  for (s = 0; s < px->n_scenes; s++) {
    const double *wl = px->sc[s]->wl;
    int n = px->n_bands;
    px->r440[s] = po_interp_1d(wl, px->rrs[s], n, 440.0);
    px->r490[s] = po_interp_1d(wl, px->rrs[s], n, 490.0);
    px->r550[s] = po_interp_1d(wl, px->rrs[s], n, 550.0);
    px->r640[s] = po_interp_1d(wl, px->rrs[s], n, 640.0);
    px->r750[s] = po_interp_1d(wl, px->rrs[s], n, 750.0);
    if (px->r440[s] < 0.0) px->r440[s] = 0.0001;
  }
}

/* HOPE forward model for one band (samodel_Rrs, model/samodel.c:2846-2949).
 * rho is the already mixed bottom term sum_i q_i B_i rho_i(lambda). */
static double hope_band(const po_scene *sc, int b, double P, double G, double X, double rho,
                        double H, double Delta, double r440, double r490, double *K_out,
                        double *rrs_bottom, double *rrs_total) {
  const double S = 0.015;
  double a_phi, a_g, a, chi, Y, b_p, bb, u, K, rrs_dp, DuC, DuB, M, rrs_C, rrs_B, rrs;
  double lambda = sc->wl[b];
  a_phi = (sc->a0[b] + sc->a1[b] * log(fabs(P))) * fabs(P);
  a_g = fabs(G) * exp(-S * (lambda - 440.0));
  a = sc->aw[b] + a_phi + a_g;
  chi = r440 / r490;
  Y = 3.44 * (1.0 - 3.17 * exp(-2.01 * chi));
  if (Y < 0.0) Y = 0.0;
  if (Y > 2.5) Y = 2.5;
  b_p = X * pow(440.0 / lambda, Y);
  bb = sc->bbw[b] + b_p;
  u = bb / (a + bb);
  K = a + bb;
  if (K < 0.0) K = 0.0;
  if (K > 2.5) K = 2.5;
  *K_out = K;
  rrs_dp = (0.084 + 0.170 * u) * u;
  DuC = 1.03 * sqrt(1.0 + 2.4 * u);
  DuB = 1.04 * sqrt(1.0 + 5.4 * u);
  M = sc->sec_sun + DuC * sc->sec_view;
  rrs_C = rrs_dp * (1.0 - exp(-M * K * H));
  M = sc->sec_sun + DuB * sc->sec_view;
  rrs_B = rho / PO_PI * exp(-M * K * H);
  *rrs_bottom = rrs_B;
  rrs = rrs_C + rrs_B;
  *rrs_total = rrs;
  return 0.5 * rrs / (1.0 - 1.5 * rrs) + Delta;
}

/* Cost of one parameter vector (samodel_error, model/samodel.c:2432-2759)
 * for a single spatial region.  With one region the depth- and
 * bottom-continuity terms (model/samodel.c:2598-2692) compare each value
 * with itself and are identically zero, and SAM is compiled out (SAM 0,
 * model/samodel.c:96), so the weighted sum reduces to the spectral and K
 * terms; both are restated here in the reference's operation order. */
static double pixel_cost(const double *x, void *ctx) {
  po_pixel *px = (po_pixel *)ctx;
  const int nb = px->n_bottoms;
  double err = 0.0, tot = 0.0, H, rrs_error, K_error, K_min = 1.0e4, model;
  int s, b, k, nobs = 0;

  H = fabs(x[0]);
  for (s = 0; s < px->n_scenes; s++) {
    const po_scene *sc = px->sc[s];
    double P, G, X, B[PO_N_BOTTOM_TYPES], q[PO_N_BOTTOM_TYPES], q_sum = 0.0;
    int nbs;
    if (px->layout == PO_LAYOUT_PER_SCENE_B) {
      B[0] = 0.01 * fabs(x[1 + 4 * s]);
      P = 0.01 * fabs(x[1 + 4 * s + 1]);
      G = 0.01 * fabs(x[1 + 4 * s + 2]);
      X = 0.01 * fabs(x[1 + 4 * s + 3]);
      q[0] = 1.0;
      nbs = 1;
    } else {
      int off = 1 + 2 * nb;
      P = 0.01 * fabs(x[off + 3 * s]);
      G = 0.01 * fabs(x[off + 3 * s + 1]);
      X = 0.01 * fabs(x[off + 3 * s + 2]);
      for (k = 0; k < nb; k++) B[k] = 0.01 * fabs(x[1 + k]);
      for (k = 0; k < nb; k++) {
        q[k] = fabs(x[1 + nb + k]);
        q_sum += q[k];
      }
      for (k = 0; k < nb; k++) q[k] /= q_sum;
      nbs = nb;
    }
    for (b = 0; b < px->n_bands; b++) {
      double rho = 0.0, albedo = 0.0, Rm, d;
      for (k = 0; k < nbs; k++) {
        albedo += q[k] * B[k];
        rho += q[k] * B[k] * sc->refl[k][b];
      }
      px->bottom_albedo = albedo;
      Rm = hope_band(sc, b, P, G, X, rho, H, 0.0, px->r440[s], px->r490[s], &px->K[s][b],
                     &px->rrs_bot[s][b], &px->rrs_mod[s][b]);
      px->Rm[s][b] = Rm;
      d = Rm - px->rrs[s][b];
      err += pow(d, 2.0);
      tot += px->rrs[s][b];
      nobs++;
    }
  }
  rrs_error = 100.0 * sqrt(err / (double)nobs) / (tot / (double)nobs);
  px->rrs_error = rrs_error;

  /* Shallow/low-K and very-high-K penalties, model/samodel.c:2696-2732. */
  {
    const double mean_c = 0.275, min_c = 0.185;
    K_error = 0.0;
    for (s = 0; s < px->n_scenes; s++) {
      K_min = 1.0e4;
      for (b = 0; b < px->n_bands; b++)
        if (!f_close((float)px->K[s][b], 0.0f, 1.0e-6f) && px->K[s][b] < K_min) K_min = px->K[s][b];
      if (H < 1.0 && K_min < mean_c) {
        K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + min_c), 2);
      } else if (H < 2.0 && K_min < 0.5 * (1.5 * min_c + 0.5 * mean_c)) {
        K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.5 * min_c + 0.5 * mean_c)), 2);
      } else if (H < 3.0 && K_min < 0.5 * (1.25 * min_c + 0.75 * mean_c)) {
        K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.25 * min_c + 0.75 * mean_c)), 2);
      } else if (H < 4.0 && K_min < 0.5 * (1.5 * min_c + 0.5 * mean_c)) {
        K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.5 * min_c + 0.5 * mean_c)), 2);
      } else if (H < 5.0 && K_min < 0.5 * (1.75 * min_c + 0.25 * mean_c)) {
        K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.75 * min_c + 0.25 * mean_c)), 2);
      }
    }
    /* uses the last scene's K_min, as the reference does */
    if (K_min > 0.7) K_error += 100.0 * pow(4.0 * (K_min - 0.7), 2);
  }
  /* weights 80/15/10/15 (model/samodel.c:2736-2744); depth/bottom terms 0 */
  model = 80.0 * rrs_error + 15.0 * K_error;
  model /= 120.0;
  px->model_error = model;
  return model;
}

/* ------------------------------------------------------------------------
 * Nelder-Mead, AS 47 as modified in model/asa047.c:10-502: reflection 1,
 * expansion 2, contraction 1/2, shrink towards the best vertex; variance
 * test every konvge iterations against reqmin*n; then the +/- eps*step
 * local-minimum probe on (long)(10*y) truncated costs, restarting from the
 * probe point with a 1e-6 scaled simplex when it fails.
 * ---------------------------------------------------------------------- */
typedef double (*po_fn)(const double *x, void *ctx);

/* (long)(10*y) with the x86-64 result for NaN and out-of-range values. */
static long trunc_to_long(double v) {
  if (!(v > -9.2233720368547758e18 && v < 9.2233720368547758e18)) return LONG_MIN;
  return (long)v;
}

static void po_nelmin(po_fn fn, void *ctx, int n, double *start, double *xmin, double *ynewlo,
                      double reqmin, const double *step, int konvge, int kcount, int *icount,
                      int *numres, int *ifault) {
  const double grow = 2.0, shrink = 0.5, eps = 1.0e-6;
  double v[(PO_MAX_PARAMS + 1) * PO_MAX_PARAMS], f[PO_MAX_PARAMS + 1];
  double cen[PO_MAX_PARAMS], refl[PO_MAX_PARAMS], trial[PO_MAX_PARAMS];
  double scale = 1.0, fr, ft, fmean, var, delta, ylo;
  const double nd = (double)n, n1d = (double)(n + 1), var_limit = reqmin * nd;
  int i, j, lo, hi, countdown = konvge;
  long floor_lo, floor_probe;

  if (reqmin <= 0.0 || n < 1 || konvge < 1) {
    *ifault = 1;
    return;
  }
  *icount = 0;
  *numres = 0;
  for (;;) {
    /* Simplex: vertex n is the start point, vertex j moves coordinate j. */
    for (i = 0; i < n; i++) v[n * n + i] = start[i];
    f[n] = fn(start, ctx);
    (*icount)++;
    for (j = 0; j < n; j++) {
      double keep = start[j];
      start[j] = start[j] + step[j] * scale;
      for (i = 0; i < n; i++) v[j * n + i] = start[i];
      f[j] = fn(start, ctx);
      (*icount)++;
      start[j] = keep;
    }
    /* ylo is kept apart from f[lo]: when every vertex ties, hi == lo and
     * the reference keeps comparing against the old best value. */
    ylo = f[0];
    lo = 0;
    for (j = 1; j <= n; j++)
      if (f[j] < ylo) {
        ylo = f[j];
        lo = j;
      }

    for (;;) {
      if (kcount <= *icount) break;
      hi = 0;
      for (j = 1; j <= n; j++)
        if (f[hi] < f[j]) hi = j;
      *ynewlo = f[hi];
      for (i = 0; i < n; i++) {
        double z = 0.0;
        for (j = 0; j <= n; j++) z = z + v[j * n + i];
        z = z - v[hi * n + i];
        cen[i] = z / nd;
      }
      for (i = 0; i < n; i++) refl[i] = cen[i] + 1.0 * (cen[i] - v[hi * n + i]);
      fr = fn(refl, ctx);
      (*icount)++;

      if (fr < ylo) {
        for (i = 0; i < n; i++) trial[i] = cen[i] + grow * (refl[i] - cen[i]);
        ft = fn(trial, ctx);
        (*icount)++;
        if (fr < ft) {
          for (i = 0; i < n; i++) v[hi * n + i] = refl[i];
          f[hi] = fr;
        } else {
          for (i = 0; i < n; i++) v[hi * n + i] = trial[i];
          f[hi] = ft;
        }
      } else {
        int worse = 0;
        for (j = 0; j <= n; j++)
          if (fr < f[j]) worse++;
        if (worse > 1) {
          for (i = 0; i < n; i++) v[hi * n + i] = refl[i];
          f[hi] = fr;
        } else if (worse == 0) {
          for (i = 0; i < n; i++) trial[i] = cen[i] + shrink * (v[hi * n + i] - cen[i]);
          ft = fn(trial, ctx);
          (*icount)++;
          if (f[hi] < ft) {
            /* shrink every vertex towards the best one */
            for (j = 0; j <= n; j++) {
              for (i = 0; i < n; i++) {
                v[j * n + i] = (v[j * n + i] + v[lo * n + i]) * 0.5;
                xmin[i] = v[j * n + i];
              }
              f[j] = fn(xmin, ctx);
              (*icount)++;
            }
            ylo = f[0];
            lo = 0;
            for (j = 1; j <= n; j++)
              if (f[j] < ylo) {
                ylo = f[j];
                lo = j;
              }
            continue;
          }
          for (i = 0; i < n; i++) v[hi * n + i] = trial[i];
          f[hi] = ft;
        } else {
          for (i = 0; i < n; i++) trial[i] = cen[i] + shrink * (refl[i] - cen[i]);
          ft = fn(trial, ctx);
          (*icount)++;
          if (ft <= fr) {
            for (i = 0; i < n; i++) v[hi * n + i] = trial[i];
            f[hi] = ft;
          } else {
            for (i = 0; i < n; i++) v[hi * n + i] = refl[i];
            f[hi] = fr;
          }
        }
      }
      if (f[hi] < ylo) {
        ylo = f[hi];
        lo = hi;
      }
      countdown--;
      if (countdown > 0) continue;
      if (*icount <= kcount) {
        countdown = konvge;
        fmean = 0.0;
        for (j = 0; j <= n; j++) fmean = fmean + f[j];
        fmean = fmean / n1d;
        var = 0.0;
        for (j = 0; j <= n; j++) var = var + pow(f[j] - fmean, 2);
        if (var <= var_limit) break;
      }
    }

    for (i = 0; i < n; i++) xmin[i] = v[lo * n + i];
    *ynewlo = f[lo];
    floor_lo = trunc_to_long(10.0 * f[lo]);
    if (kcount < *icount) {
      *ifault = 2;
      break;
    }
    *ifault = 0;
    for (i = 0; i < n; i++) {
      delta = step[i] * eps;
      xmin[i] = xmin[i] + delta;
      floor_probe = trunc_to_long(10.0 * fn(xmin, ctx));
      (*icount)++;
      if (floor_probe < floor_lo) {
        *ifault = 2;
        break;
      }
      xmin[i] = xmin[i] - delta - delta;
      floor_probe = trunc_to_long(10.0 * fn(xmin, ctx));
      (*icount)++;
      if (floor_probe < floor_lo) {
        *ifault = 2;
        break;
      }
      xmin[i] = xmin[i] + delta;
    }
    if (*ifault == 0) break;
    for (i = 0; i < n; i++) start[i] = xmin[i];
    scale = eps;
    (*numres)++;
  }
}

/* ------------------------------------------------------------------------
 * Per-pixel driver (samodel_optimise + _one_bottom_combination, cold start,
 * no empirical depth, model/samodel.c:1768-2115 and :2119-2427), or a
 * single fit from a caller-given start vector (seeded).
 * ---------------------------------------------------------------------- */
typedef struct {
  double reqmin;
  int konvge, kcount;
  int n_hstarts;
  const double *hstarts;
  double seed_step_scale;
} po_fit;

static void cold_start(const po_pixel *px, double H0, double *start, double *step) {
  const int nb = px->n_bottoms, ns = px->n_scenes;
  double m490 = 0.0;
  int s, k;
  start[0] = H0;
  step[0] = 1.25 * start[0];
  for (s = 0; s < ns; s++) m490 += px->r490[s];
  m490 /= (double)1 * ns;
  if (px->layout == PO_LAYOUT_PER_SCENE_B) {
    for (s = 0; s < ns; s++) {
      double r490 = (0.0 + px->r490[s]) / (double)1;
      double r550 = (0.0 + px->r550[s]) / (double)1;
      double r640 = (0.0 + px->r640[s]) / (double)1;
      double *z = start + 1 + 4 * s, *d = step + 1 + 4 * s;
      z[0] = 100.0 * 4.0 * r490;
      d[0] = 1.5 * z[0];
      z[1] = 100.0 * 0.072 * pow(r490 / r550, -1.7);
      z[2] = 1.5 * z[1];
      z[3] = 100.0 * 30.0 * px->sc[s]->aw640 * r640;
      d[1] = 2.0 * z[1];
      d[2] = 2.0 * z[2];
      d[3] = 2.0 * z[3];
    }
    return;
  }
  for (k = 0; k < nb; k++) {
    start[1 + k] = 100.0 * 4.0 * m490;
    step[1 + k] = 1.5 * start[1 + k];
  }
  for (k = 0; k < nb; k++) {
    start[1 + nb + k] = 1.0;
    step[1 + nb + k] = 0.5 * start[1 + nb + k];
  }
  for (s = 0; s < ns; s++) {
    int o = 1 + 2 * nb + 3 * s;
    double r490 = (0.0 + px->r490[s]) / (double)1;
    double r550 = (0.0 + px->r550[s]) / (double)1;
    double r640 = (0.0 + px->r640[s]) / (double)1;
    start[o] = 100.0 * 0.072 * pow(r490 / r550, -1.7);
    start[o + 1] = 1.5 * start[o];
    start[o + 2] = 100.0 * 30.0 * px->sc[s]->aw640 * r640;
    step[o] = 2.0 * start[o];
    step[o + 1] = 2.0 * start[o + 1];
    step[o + 2] = 2.0 * start[o + 2];
  }
}

/* Steps of a seeded start: the cold start's relative steps times a scale
 * (1 reproduces the reference's hot-start steps, model/samodel.c:2286-2309). */
static void seeded_start(const po_pixel *px, const double *seed, double scale, double *start,
                         double *step) {
  int n = n_params_of(px), i;
  double rel_ref[6] = {1.25, 1.5, 0.5, 2.0, 2.0, 2.0};
  for (i = 0; i < n; i++) {
    double rel = (i < 6) ? rel_ref[i] : 2.0;
    start[i] = seed[i];
    step[i] = (rel * scale) * start[i];
  }
}

/* fit_pixel, also handing back the kept vector (signed, as nelmin left it)
 * when best_out is given. */
static void fit_pixel_ex(po_pixel *px, const po_fit *fit, const double *seed, double *o,
                         double *best_out);

static void fit_pixel(po_pixel *px, const po_fit *fit, const double *seed, double *o) {
  fit_pixel_ex(px, fit, seed, o, NULL);
}

static void fit_pixel_ex(po_pixel *px, const po_fit *fit, const double *seed, double *o,
                         double *best_out) {
  const int n = n_params_of(px);
  double start[PO_MAX_PARAMS], step[PO_MAX_PARAMS], xm[PO_MAX_PARAMS], best[PO_MAX_PARAMS];
  double lowest = 1.0e4, y = 0.0;
  int icount = 0, numres = 0, ifault = 0, k, s, b, nst;
  long total = 0;
  int kept_evals = 0, kept_res = 0, kept_start = 0, kept_fault = 0, converged = 0;

  pixel_reference_rrs(px);
  memset(best, 0, sizeof best);
  nst = seed ? 1 : fit->n_hstarts;
  for (k = 0; k < nst; k++) {
    if (seed)
      seeded_start(px, seed, fit->seed_step_scale, start, step);
    else
      cold_start(px, fit->hstarts[k], start, step);
    po_nelmin(pixel_cost, px, n, start, xm, &y, fit->reqmin, step, fit->konvge, fit->kcount,
              &icount, &numres, &ifault);
    total += icount;
    if (y < lowest) {
      lowest = y;
      memcpy(best, xm, n * sizeof(double));
      kept_evals = icount;
      kept_res = numres;
      kept_start = k;
      kept_fault = ifault;
      converged = (ifault == 0);
      if (lowest < 2.5 * ((float)px->n_scenes)) break; /* model/samodel.c:2404 */
    }
  }
  /* Recompute the model at the kept optimum (model/samodel.c:2413). */
  pixel_cost(best, px);

  /* Post-fit products (model/samodel.c:1994-2079) for one region. */
  {
    double K_min = 1.0e10, iod = 0.0, nobs = 0.0, depth;
    int found = 0;
    for (s = 0; s < px->n_scenes; s++)
      for (b = 0; b < px->n_bands; b++)
        if (!f_close((float)px->K[s][b], (float)0.0, 1.0e-4f) && px->K[s][b] < K_min) {
          K_min = px->K[s][b];
          found = 1;
        }
    if (!found) K_min = 0.0;
    depth = 0.0;
    depth += sqrt(1.0) * fabs(best[0]);
    depth /= sqrt(1.0) + 1.0 - 1.0;
    for (s = 0; s < px->n_scenes; s++)
      for (b = 0; b < px->n_bands; b++) {
        iod += px->rrs_bot[s][b] / px->rrs_mod[s][b];
        nobs += 1.0;
      }
    iod = 100.0 * iod / nobs;
    o[0] = depth;
    o[1] = px->bottom_albedo;
    o[2] = px->model_error;
    o[3] = px->rrs_error;
    o[4] = K_min;
    o[5] = iod;
  }
  o[6] = (double)kept_evals;
  o[7] = (double)total;
  o[8] = converged ? 1.0 : 0.0;
  o[9] = 0.0;
  o[10] = (double)px->n_scenes;
  for (s = 0; s < px->n_scenes; s++) {
    int idx = (px->layout == PO_LAYOUT_PER_SCENE_B) ? 1 + 4 * s + 1 : 1 + 2 * px->n_bottoms + 3 * s;
    o[11 + s] = 0.01 * fabs(best[idx]);
    o[19 + s] = 0.01 * fabs(best[idx + 1]);
    o[27 + s] = 0.01 * fabs(best[idx + 2]);
  }
  o[35] = (double)kept_res;
  o[36] = (double)kept_start;
  o[37] = (double)kept_fault;
  if (best_out) memcpy(best_out, best, n * sizeof(double));
}

/* Mask test of model/samodel.c:937-941: nodata or negative in any band. */
static int masked(const float *r, int n, float nodata) {
  int b;
  for (b = 0; b < n; b++)
    if (f_close(r[b], nodata, 1.0e-6f) || r[b] < 0.0) return 1;
  return 0;
}

static const double po_default_hstarts[8] = {40.0, 30.0, 20.0, 15.0, 10.0, 7.5, 2.5, 1.0};

int po_nout(void) { return PO_NOUT; }

int po_invert_batch(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                    double h_tide, const float *rrs, int64_t npix, float nodata, double reqmin,
                    int konvge, int kcount, int n_hstarts, const double *hstarts,
                    const double *seeds, double seed_step_scale, int nthreads, double *out) {
  po_scene sc;
  po_fit fit;
  int64_t p;
  if (n_bands < 2 || n_bands > PO_MAX_BANDS) return 1;
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, h_tide);
  fit.seed_step_scale = seed_step_scale;
  fit.reqmin = reqmin;
  fit.konvge = konvge;
  fit.kcount = kcount;
  fit.n_hstarts = (n_hstarts > 0 && hstarts) ? n_hstarts : 8;
  fit.hstarts = (n_hstarts > 0 && hstarts) ? hstarts : po_default_hstarts;
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 8)
#endif
  for (p = 0; p < npix; p++) {
    const float *r = rrs + p * n_bands;
    double *o = out + p * PO_NOUT;
    const double *seed = NULL;
    po_pixel px;
    int b;
    memset(o, 0, PO_NOUT * sizeof(double));
    if (masked(r, n_bands, nodata)) {
      o[9] = 1.0;
      continue;
    }
    memset(&px, 0, sizeof px);
    px.n_scenes = 1;
    px.n_bands = n_bands;
    px.n_bottoms = 1;
    px.layout = PO_LAYOUT_REFERENCE;
    px.sc[0] = &sc;
    for (b = 0; b < n_bands; b++) px.rrs[0][b] = r[b];
    if (seeds && !isnan(seeds[p * 6])) seed = seeds + p * 6;
    fit_pixel(&px, &fit, seed, o);
  }
  return 0;
}

int po_joint_invert_batch(int n_bands, const double *wl, double theta_view_deg, double h_tide,
                          const int32_t *scene_offsets, const double *theta_sun_deg,
                          const float *rrs, int64_t npix, float nodata, int layout,
                          double reqmin, int konvge, int kcount, int n_hstarts,
                          const double *hstarts, int nthreads, double *out) {
  po_fit fit;
  int64_t p;
  if (n_bands < 2 || n_bands > PO_MAX_BANDS) return 1;
  fit.seed_step_scale = 1.0;
  fit.reqmin = reqmin;
  fit.konvge = konvge;
  fit.kcount = kcount;
  fit.n_hstarts = (n_hstarts > 0 && hstarts) ? n_hstarts : 8;
  fit.hstarts = (n_hstarts > 0 && hstarts) ? hstarts : po_default_hstarts;
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (p = 0; p < npix; p++) {
    int o0 = scene_offsets[p], k = scene_offsets[p + 1] - scene_offsets[p], s, b, m = 0;
    double *o = out + p * PO_NOUT;
    po_scene sc[PO_MAX_SCENES];
    po_pixel px;
    memset(o, 0, PO_NOUT * sizeof(double));
    if (k < 1 || k > PO_MAX_SCENES) {
      o[9] = 2.0;
      continue;
    }
    for (s = 0; s < k; s++) m |= masked(rrs + (size_t)(o0 + s) * n_bands, n_bands, nodata);
    if (m) {
      o[9] = 1.0;
      continue;
    }
    memset(&px, 0, sizeof px);
    px.n_scenes = k;
    px.n_bands = n_bands;
    px.n_bottoms = 1;
    px.layout = layout;
    for (s = 0; s < k; s++) {
      scene_init(&sc[s], n_bands, wl, theta_sun_deg[o0 + s], theta_view_deg, h_tide);
      px.sc[s] = &sc[s];
      for (b = 0; b < n_bands; b++) px.rrs[s][b] = rrs[(size_t)(o0 + s) * n_bands + b];
    }
    fit_pixel(&px, &fit, NULL, o);
  }
  return 0;
}

double po_cost(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
               double h_tide, const double *rrs_measured, const double *params,
               double *rrs_modelled, double *K_out) {
  po_scene sc;
  po_pixel px;
  double c;
  int b;
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, h_tide);
  memset(&px, 0, sizeof px);
  px.n_scenes = 1;
  px.n_bands = n_bands;
  px.n_bottoms = 1;
  px.sc[0] = &sc;
  for (b = 0; b < n_bands; b++) px.rrs[0][b] = rrs_measured[b];
  pixel_reference_rrs(&px);
  c = pixel_cost(params, &px);
  for (b = 0; b < n_bands; b++) {
    rrs_modelled[b] = px.Rm[0][b];
    K_out[b] = px.K[0][b];
  }
  return c;
}

/* nelmin (model/asa047.c:10-502) over a caller's cost, n <= PO_MAX_PARAMS:
 * lets the tests run the device state machines against this restatement
 * at any simplex size.  start is not modified. */
void po_nelmin_fn(double (*fn)(const double *x, void *ctx), void *ctx, int n,
                  const double *start_in, const double *step, double reqmin, int konvge,
                  int kcount, double *xmin, double *ynewlo, int *icount, int *numres,
                  int *ifault) {
  double start[PO_MAX_PARAMS];
  memcpy(start, start_in, (size_t)n * sizeof(double));
  po_nelmin(fn, ctx, n, start, xmin, ynewlo, reqmin, step, konvge, kcount, icount, numres,
            ifault);
}

void po_nelmin_pixel(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                     const double *rrs_measured, const double *start_in, const double *step,
                     double reqmin, int konvge, int kcount, double *xmin, double *ynewlo,
                     int *icount, int *numres, int *ifault) {
  po_scene sc;
  po_pixel px;
  double start[PO_MAX_PARAMS];
  int b;
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, 0.0);
  memset(&px, 0, sizeof px);
  px.n_scenes = 1;
  px.n_bands = n_bands;
  px.n_bottoms = 1;
  px.sc[0] = &sc;
  for (b = 0; b < n_bands; b++) px.rrs[0][b] = rrs_measured[b];
  pixel_reference_rrs(&px);
  memcpy(start, start_in, 6 * sizeof(double));
  po_nelmin(pixel_cost, &px, 6, start, xmin, ynewlo, reqmin, step, konvge, kcount, icount, numres,
            ifault);
}

/* ------------------------------------------------------------------------
 * Synthetic scenes.  Counter-based Philox4x32-10 (Salmon et al., SC'11)
 * keyed by the 64-bit seed, with the pixel index and a draw index in the
 * counter, so any pixel can be regenerated alone and the CUDA generator in
 * photic_gb300/csrc produces the same uniforms.  Truth follows the
 * synthetic prior of the plain-method workload: H~U(0.5,25) m,
 * P~logU(0.005,0.1), G~logU(0.005,0.2), X~logU(0.001,0.05),
 * B~U(0.05,0.5) on the sand spectrum; Rrs from the forward model with the
 * spectral-shape exponent Y made self-consistent by fixed-point iteration
 * (Y depends on the measured Rrs440/Rrs490, model/samodel.c:2898-2901),
 * plus Gaussian noise.  This generator is new: the reference has none.
 * ---------------------------------------------------------------------- */
void po_philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                   uint32_t *out4) {
  int r;
  for (r = 0; r < 10; r++) {
    uint64_t m0 = (uint64_t)0xD2511F53u * c0, m1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(m1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)m1;
    uint32_t n2 = (uint32_t)(m0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)m0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out4[0] = c0; out4[1] = c1; out4[2] = c2; out4[3] = c3;
}

static void draw4(uint64_t seed, uint64_t idx, uint32_t block, uint32_t stream, double *u) {
  uint32_t w[4];
  int i;
  po_philox4x32((uint32_t)idx, (uint32_t)(idx >> 32), block, stream, (uint32_t)seed,
                (uint32_t)(seed >> 32), w);
  for (i = 0; i < 4; i++) u[i] = ((double)w[i] + 0.5) * 2.3283064365386963e-10; /* 2^-32 */
}

static double log_uniform(double u, double lo, double hi) {
  return exp(log(lo) + u * (log(hi) - log(lo)));
}

/* Fixed-point synthesis of one scene's spectrum for truth (H,P,G,X,B). */
static void synthesise(const po_scene *sc, double H, double P, double G, double X, double B,
                       double *rrs) {
  po_pixel px;
  double x[6];
  int it, b;
  memset(&px, 0, sizeof px);
  px.n_scenes = 1;
  px.n_bands = sc->n_bands;
  px.n_bottoms = 1;
  px.sc[0] = sc;
  x[0] = H; x[1] = 100.0 * B; x[2] = 1.0; x[3] = 100.0 * P; x[4] = 100.0 * G; x[5] = 100.0 * X;
  for (b = 0; b < sc->n_bands; b++) px.rrs[0][b] = 0.01;
  for (it = 0; it < 30; it++) {
    pixel_reference_rrs(&px);
    pixel_cost(x, &px);
    for (b = 0; b < sc->n_bands; b++) px.rrs[0][b] = px.Rm[0][b];
  }
  for (b = 0; b < sc->n_bands; b++) rrs[b] = px.rrs[0][b];
}

static void add_noise(uint64_t seed, uint64_t idx, uint32_t stream, int n_bands, double sigma,
                      double *rrs) {
  int b;
  for (b = 0; b < n_bands; b += 2) {
    double u[4], r, a;
    draw4(seed, idx, 2u + (uint32_t)(b / 4), stream, u);
    r = sqrt(-2.0 * log(u[(b % 4)]));
    a = 2.0 * PO_PI * u[(b % 4) + 1];
    rrs[b] += sigma * r * cos(a);
    if (b + 1 < n_bands) rrs[b + 1] += sigma * r * sin(a);
  }
}

static void apply_mask(double u_mask, double u_kind, double mask_frac, int n_bands, float nodata,
                       float *r) {
  int b;
  if (u_mask >= mask_frac) return;
  if (u_kind < 0.5) {
    for (b = 0; b < n_bands; b++) r[b] = nodata;
  } else {
    r[n_bands - 1] = -fabsf(r[n_bands - 1]) - 1.0e-3f;
  }
}

void po_generate_single(uint64_t seed, int64_t pix0, int64_t npix, int n_bands, const double *wl,
                        double theta_sun_deg, double theta_view_deg, double mask_frac,
                        double noise_sigma, float nodata, float *rrs_out, double *truth_out) {
  po_scene sc;
  int64_t i;
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, 0.0);
#if _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (i = 0; i < npix; i++) {
    uint64_t p = (uint64_t)(pix0 + i);
    double u0[4], u1[4], H, P, G, X, B, r[PO_MAX_BANDS];
    int b;
    draw4(seed, p, 0u, 0u, u0);
    draw4(seed, p, 1u, 0u, u1);
    H = 0.5 + 24.5 * u0[0];
    P = log_uniform(u0[1], 0.005, 0.1);
    G = log_uniform(u0[2], 0.005, 0.2);
    X = log_uniform(u0[3], 0.001, 0.05);
    B = 0.05 + 0.45 * u1[0];
    synthesise(&sc, H, P, G, X, B, r);
    add_noise(seed, p, 0u, n_bands, noise_sigma, r);
    for (b = 0; b < n_bands; b++) rrs_out[i * n_bands + b] = (float)r[b];
    apply_mask(u1[1], u1[2], mask_frac, n_bands, nodata, rrs_out + i * n_bands);
    if (truth_out) {
      truth_out[i * 5 + 0] = H;
      truth_out[i * 5 + 1] = P;
      truth_out[i * 5 + 2] = G;
      truth_out[i * 5 + 3] = X;
      truth_out[i * 5 + 4] = B;
    }
  }
}

void po_joint_counts(uint64_t seed, int64_t npix, int kmin, int kmax, int32_t *counts) {
  int64_t p;
  for (p = 0; p < npix; p++) {
    double u[4];
    int k;
    draw4(seed, (uint64_t)p, 0u, 1u, u);
    k = kmin + (int)(u[0] * (double)(kmax - kmin + 1));
    if (k > kmax) k = kmax;
    counts[p] = k;
  }
}

void po_generate_joint(uint64_t seed, int64_t npix, int n_bands, const double *wl,
                       double theta_view_deg, double theta_sun_min, double theta_sun_max,
                       double mask_frac, double noise_sigma, float nodata,
                       const int32_t *scene_offsets, double *theta_sun_out, float *rrs_out,
                       double *truth_out) {
  int64_t p;
#if _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (p = 0; p < npix; p++) {
    int o0 = scene_offsets[p], k = scene_offsets[p + 1] - o0, s, b;
    double uH[4], H;
    draw4(seed, (uint64_t)p, 1u, 1u, uH);
    H = 0.5 + 24.5 * uH[0];
    for (s = 0; s < k; s++) {
      uint64_t obs = (uint64_t)(o0 + s);
      double u0[4], u1[4], r[PO_MAX_BANDS], P, G, X, B, th;
      po_scene sc;
      draw4(seed, obs, 0u, 2u, u0);
      draw4(seed, obs, 1u, 2u, u1);
      P = log_uniform(u0[0], 0.005, 0.1);
      G = log_uniform(u0[1], 0.005, 0.2);
      X = log_uniform(u0[2], 0.001, 0.05);
      B = 0.05 + 0.45 * u0[3];
      th = theta_sun_min + (theta_sun_max - theta_sun_min) * u1[0];
      theta_sun_out[obs] = th;
      scene_init(&sc, n_bands, wl, th, theta_view_deg, 0.0);
      synthesise(&sc, H, P, G, X, B, r);
      add_noise(seed, obs, 2u, n_bands, noise_sigma, r);
      for (b = 0; b < n_bands; b++) rrs_out[obs * n_bands + b] = (float)r[b];
      if (s == 0) apply_mask(uH[1], uH[2], mask_frac, n_bands, nodata, rrs_out + obs * n_bands);
      if (truth_out) {
        truth_out[obs * 5 + 0] = H;
        truth_out[obs * 5 + 1] = P;
        truth_out[obs * 5 + 2] = G;
        truth_out[obs * 5 + 3] = X;
        truth_out[obs * 5 + 4] = B;
      }
    }
  }
}

/* ---- depth uncertainty (model/samodel.c:1368-1479) ------------------------
 * The reference's estimate with its random draws replaced by Philox draws
 * keyed by seed (the GPU uses the same stream): sample g = k * n_samples + s
 * of interval k probes pixel (w0 * npix) >> 32 of counter (g, trial, 0xD5),
 * and moves every band by n * r_sigma[b], n = +/- u1 (sign from u0) of
 * counter (g, 0xFFFFFFFF, 0xD6).  Refits are independent cold starts.
 * With sample_depth_in the refits are skipped and those depths are used. */
#define PO_DS_MAX 120

static int po_approx_f(float a, float b, float eps) {
  float d = fabsf(a - b);
  return d <= ((fabsf(a) < fabsf(b) ? fabsf(b) : fabsf(a)) * eps);
}

/* The deepest fitted depth's interval count (model/samodel.c:1383-1387). */
static int ds_intervals_host(const float *depth, int64_t npix, double interval) {
  float mx = 0.0f;
  double m;
  int64_t p;
  int n_int;
  for (p = 0; p < npix; p++) {
    float v = depth[p];
    if (!(v > 0.0f) || po_approx_f(v, 0.0f, 1.0e-4f)) continue;
    if (v > mx) mx = v;
  }
  m = interval * (double)((int)mx / interval);
  if (m > 30.0) m = 30.0;
  n_int = (int)(m / interval);
  return n_int > PO_DS_MAX ? PO_DS_MAX : n_int;
}

/* The samples: per (interval, sample) a pixel of the interval found by up
 * to n_trials uniform probes (-1: none) and the draw n of frand2(1.0)
 * (model/samodel.c:1402-1424, model/common.c:220), from Philox. */
static void ds_select_host(const float *depth, int64_t npix, int n_samples, uint64_t seed,
                           int n_int, double interval, int32_t *sample_pixel, float *sample_n) {
  const int64_t ns = (int64_t)PO_DS_MAX * n_samples;
  const int n_trials = (int)sqrt((double)npix);
  int64_t g;
  for (g = 0; g < ns; g++) {
    int64_t found = -1;
    int t2, k = (int)(g / n_samples);
    if (k < n_int) {
      double d = k * interval;
      for (t2 = 0; t2 < n_trials && found < 0; t2++) {
        uint32_t w[4];
        int64_t q;
        po_philox4x32((uint32_t)g, (uint32_t)(g >> 32), (uint32_t)t2, 0xD5u, (uint32_t)seed,
                      (uint32_t)(seed >> 32), w);
        q = (int64_t)(((uint64_t)w[0] * (uint64_t)npix) >> 32);
        if (depth[q] > d && depth[q] < d + interval) found = q;
      }
    }
    sample_pixel[g] = (int32_t)found;
    sample_n[g] = 0.0f;
    if (found >= 0) {
      uint32_t w[4];
      double u0, u1;
      po_philox4x32((uint32_t)g, (uint32_t)(g >> 32), 0xFFFFFFFFu, 0xD6u, (uint32_t)seed,
                    (uint32_t)(seed >> 32), w);
      u0 = ((double)w[0] + 0.5) * 2.3283064365386963e-10;
      u1 = ((double)w[1] + 0.5) * 2.3283064365386963e-10;
      sample_n[g] = u0 < 0.5 ? (float)u1 : -1.0f * (float)u1;
    }
  }
}

/* vec_mean2_double / vec_stddev_double of each interval's non-zero
 * refitted depths (model/common.c:877-940) and the map (:1462-1476). */
static void ds_finish_host(const double *sample_depth, int n_samples, int n_int, double interval,
                           const float *depth, int64_t npix, double *table, float *depth_sigma) {
  int64_t p;
  int k;
  for (k = 0; k < PO_DS_MAX; k++) {
    double sigma = 0.0;
    if (k < n_int) {
      const double *v = sample_depth + (int64_t)k * n_samples;
      double total = 0.0, mean, sumdev = 0.0;
      int s, count = 0;
      for (s = 0; s < n_samples; s++)
        if (!po_approx_f((float)v[s], 0.0f, 1.0e-4f)) {
          total += v[s];
          count++;
        }
      if (count > 0) {
        mean = (double)(float)(total / (double)count);
        for (s = 0; s < n_samples; s++)
          if (!po_approx_f((float)v[s], 0.0f, 1.0e-4f)) sumdev += pow(v[s] - mean, 2);
        sigma = sqrt(sumdev / (double)count);
      }
    }
    table[k] = sigma;
  }
  for (p = 0; p < npix; p++) {
    float s = 0.0f, dp = depth[p];
    if (dp > 0.0f) {
      double d = 0.0;
      for (k = 0; k < n_int; k++, d += interval)
        if (dp > d && dp <= d + interval) {
          s = (float)table[k];
          break;
        }
    }
    depth_sigma[p] = s;
  }
}

int po_depth_sigma(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                   const float *rrs, int64_t npix, const float *depth, const double *r_sigma,
                   int n_samples, uint64_t seed, double reqmin, int konvge, int kcount,
                   int nthreads, const double *sample_depth_in, int32_t *sample_pixel,
                   double *sample_depth, double *table, float *depth_sigma) {
  const double interval = 0.25;
  const int64_t ns = (int64_t)PO_DS_MAX * n_samples;
  const int n_int = ds_intervals_host(depth, npix, interval);
  int64_t g;
  float *srrs = (float *)malloc((size_t)ns * n_bands * sizeof(float));
  float *sn = (float *)malloc((size_t)ns * sizeof(float));
  if (!srrs || !sn) {
    free(srrs);
    free(sn);
    return 1;
  }
  ds_select_host(depth, npix, n_samples, seed, n_int, interval, sample_pixel, sn);
  for (g = 0; g < ns; g++) {
    const int64_t found = sample_pixel[g];
    int b;
    for (b = 0; b < n_bands; b++) {
      double v;
      if (found < 0) {
        srrs[g * n_bands + b] = -9999.0f;
        continue;
      }
      v = (double)rrs[found * n_bands + b];
      if (!po_approx_f(sn[g], 0.0f, 1.0e-6f)) v += (double)sn[g] * r_sigma[b];
      srrs[g * n_bands + b] = (float)v;
    }
  }
  free(sn);
  if (sample_depth_in) {
    memcpy(sample_depth, sample_depth_in, (size_t)ns * sizeof(double));
  } else {
    double *out = (double *)malloc((size_t)ns * PO_NOUT * sizeof(double));
    if (!out) {
      free(srrs);
      return 1;
    }
    if (po_invert_batch(n_bands, wl, theta_sun_deg, theta_view_deg, 0.0, srrs, ns, -9999.0f,
                        reqmin, konvge, kcount, 0, NULL, NULL, 1.0, nthreads, out)) {
      free(out);
      free(srrs);
      return 1;
    }
    for (g = 0; g < ns; g++) sample_depth[g] = out[g * PO_NOUT + 0];
    free(out);
  }
  free(srrs);
  ds_finish_host(sample_depth, n_samples, n_int, interval, depth, npix, table, depth_sigma);
  return 0;
}

/* ---- regions, bottom mixtures and scenes (model/samodel.c:1768-2115) ----
 * The general fit of samodel_optimise: each pixel alone (n_spatial = 1) or
 * together with its 3 x 3 neighbourhood (n_spatial = 2; extract_Rrs_data,
 * model/samodel.c:2957-3027: indexes clamped at the grid's edges,
 * neighbours with a nodata band in any scene left out; smoothing radius 1),
 * over n_scenes scenes of the same bands (each with its own sun zenith),
 * with n_bottoms bottom types (sand, seagrass, coral: the first entries of
 * the reference's bottom table, model/samodel.c:464-475).  Every region has
 * its own depth and, per bottom type, its own albedo and mixing weight q;
 * every scene its own P, G, X; the cost adds the depth- and
 * bottom-continuity terms (model/samodel.c:2594-2692).  With an empirical
 * depth the pixel takes that single depth start, and a pixel deeper than
 * 8 m is fitted with sand alone (model/samodel.c:1781, 1826-1830,
 * 2208-2231; the bottom-type count is restored after the pixel,
 * model/samodel.c:2104). */
#define PO_MAX_REGIONS 9
#define PO_MAX_MIX 3

typedef struct {
  int R, S, origin, n_bands, nb;
  const po_scene *sc[PO_MAX_SCENES];
  double rrs[PO_MAX_REGIONS][PO_MAX_SCENES][PO_MAX_BANDS];
  double r440[PO_MAX_REGIONS][PO_MAX_SCENES], r490[PO_MAX_REGIONS][PO_MAX_SCENES];
  double r550[PO_MAX_REGIONS][PO_MAX_SCENES], r640[PO_MAX_REGIONS][PO_MAX_SCENES];
  double r750[PO_MAX_REGIONS][PO_MAX_SCENES];
  double K[PO_MAX_SCENES][PO_MAX_BANDS]; /* md->K[scene][band]: the last region's */
  double rrs_mod[PO_MAX_REGIONS][PO_MAX_SCENES][PO_MAX_BANDS];
  double rrs_bot[PO_MAX_REGIONS][PO_MAX_SCENES][PO_MAX_BANDS];
  double Rm[PO_MAX_REGIONS][PO_MAX_SCENES][PO_MAX_BANDS]; /* md->Rrs_modelled */
  double bottom_albedo, rrs_error, model_error;
} po_rpixel;

static int region_n_params(const po_rpixel *px) {
  return px->R + 2 * px->nb * px->R + 3 * px->S; /* model/samodel.c:1806-1855 */
}

static double k_penalty(double H, double K_min) {
  const double mean_c = 0.275, min_c = 0.185;
  double K_error = 0.0;
  if (H < 1.0 && K_min < mean_c) {
    K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + min_c), 2);
  } else if (H < 2.0 && K_min < 0.5 * (1.5 * min_c + 0.5 * mean_c)) {
    K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.5 * min_c + 0.5 * mean_c)), 2);
  } else if (H < 3.0 && K_min < 0.5 * (1.25 * min_c + 0.75 * mean_c)) {
    K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.25 * min_c + 0.75 * mean_c)), 2);
  } else if (H < 4.0 && K_min < 0.5 * (1.5 * min_c + 0.5 * mean_c)) {
    K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.5 * min_c + 0.5 * mean_c)), 2);
  } else if (H < 5.0 && K_min < 0.5 * (1.75 * min_c + 0.25 * mean_c)) {
    K_error += 100.0 * pow(1.0 / (0.01 + K_min) - 1.0 / (0.01 + 0.5 * (1.75 * min_c + 0.25 * mean_c)), 2);
  }
  return K_error;
}

/* samodel_error with R regions, S scenes and nb bottom types; parameters
 * [H_r | 100 B_{r,k} at R + r nb + k | q_{r,k} at R + R nb + r nb + k |
 *  100 P_s, 100 G_s, 100 X_s at R + 2 nb R + 3 s] (model/samodel.c:2463-2491). */
static double region_cost(const double *x, void *ctx) {
  po_rpixel *px = (po_rpixel *)ctx;
  const int R = px->R, S = px->S, nb = px->nb, qo = R + R * nb, off = R + 2 * nb * R;
  double err = 0.0, tot = 0.0, rrs_error, depth_mean, th, error_depth, n_out, bottom_mean,
         bottom_total, error_bottom, H, K_error, K_min = 1.0e4, model;
  int r, s, b, k, kb, nobs = 0;
  for (r = 0; r < R; r++) {
    for (s = 0; s < S; s++) {
      const po_scene *sc = px->sc[s];
      double Hr = fabs(x[r]), P = 0.01 * fabs(x[off + 3 * s]), G = 0.01 * fabs(x[off + 1 + 3 * s]),
             X = 0.01 * fabs(x[off + 2 + 3 * s]), B[PO_MAX_MIX], q[PO_MAX_MIX], q_sum = 0.0;
      for (k = 0; k < nb; k++) B[k] = 0.01 * fabs(x[R + r * nb + k]);
      for (k = 0; k < nb; k++) {
        q[k] = fabs(x[qo + r * nb + k]);
        q_sum += q[k];
      }
      for (k = 0; k < nb; k++) q[k] /= q_sum;
      for (b = 0; b < px->n_bands; b++) {
        double rho = 0.0, albedo = 0.0, Rm, d;
        for (k = 0; k < nb; k++) { /* model/samodel.c:2878-2883 */
          albedo += q[k] * B[k];
          rho += q[k] * B[k] * sc->refl[k][b];
        }
        px->bottom_albedo = albedo;
        Rm = hope_band(sc, b, P, G, X, rho, Hr, 0.0, px->r440[r][s], px->r490[r][s],
                       &px->K[s][b], &px->rrs_bot[r][s][b], &px->rrs_mod[r][s][b]);
        px->Rm[r][s][b] = Rm;
        d = Rm - px->rrs[r][s][b];
        err += pow(d, 2.0);
        tot += px->rrs[r][s][b];
        nobs++;
      }
    }
  }
  rrs_error = 100.0 * sqrt(err / (double)nobs) / (tot / (double)nobs);
  px->rrs_error = rrs_error;
  /* depth continuity, model/samodel.c:2594-2629 */
  depth_mean = 0.0;
  for (r = 0; r < R; r++) depth_mean += fabs(x[r]);
  depth_mean /= (double)R;
  if (depth_mean < 4.0) th = 0.4;
  else if (depth_mean < 8.0) th = 0.2;
  else if (depth_mean < 12.0) th = 0.1;
  else th = 0.05;
  error_depth = 0.0;
  n_out = 0.0;
  for (r = 0; r < R; r++)
    if (fabs(x[r]) < (1.0 - th) * depth_mean || fabs(x[r]) > (1.0 + th) * depth_mean) {
      error_depth += pow(fabs(x[r]) - depth_mean, 2.0);
      n_out += 1.0;
    }
  if (n_out > 0.5) error_depth = 100.0 * sqrt(error_depth / n_out) / depth_mean;
  /* bottom continuity, model/samodel.c:2633-2692: per bottom type the mean
   * over regions of |100 B| |q| / sum |q|, deviations beyond the threshold */
  if (depth_mean < 5.0) th = 0.25;
  else if (depth_mean < 10.0) th = 0.1;
  else if (depth_mean < 15.0) th = 0.05;
  else th = 0.01;
  error_bottom = 0.0;
  n_out = 0.0;
  bottom_total = 0.0;
  for (k = 0; k < nb; k++) {
    bottom_mean = 0.0;
    for (r = 0; r < R; r++) {
      double q_sum = 0.0;
      for (kb = 0; kb < nb; kb++) q_sum += fabs(x[qo + r * nb + kb]);
      bottom_mean += fabs(x[R + r * nb + k]) * fabs(x[qo + r * nb + k]) / q_sum;
    }
    bottom_mean /= (double)R;
    bottom_total += bottom_mean;
    for (r = 0; r < R; r++) {
      double q_sum = 0.0, bottom;
      for (kb = 0; kb < nb; kb++) q_sum += fabs(x[qo + r * nb + kb]);
      bottom = fabs(x[R + r * nb + k]) * fabs(x[qo + r * nb + k]) / q_sum;
      if (bottom < (1.0 - th) * bottom_mean || bottom > (1.0 + th) * bottom_mean) {
        error_bottom += pow(bottom - bottom_mean, 2.0);
        n_out += 1.0;
      }
    }
  }
  if (n_out > 0.5) {
    bottom_mean = bottom_total / ((double)nb);
    error_bottom = 100.0 * sqrt(error_bottom / n_out) / bottom_mean;
  }
  /* K penalties on the origin's depth and each scene's K (the last region's
   * bands); the very-high-K term on the last scene's, model/samodel.c:2696-2732 */
  H = fabs(x[px->origin]);
  K_error = 0.0;
  for (s = 0; s < S; s++) {
    K_min = 1.0e4;
    for (b = 0; b < px->n_bands; b++)
      if (!f_close((float)px->K[s][b], 0.0f, 1.0e-6f) && px->K[s][b] < K_min) K_min = px->K[s][b];
    K_error += k_penalty(H, K_min);
  }
  if (K_min > 0.7) K_error += 100.0 * pow(4.0 * (K_min - 0.7), 2);
  model = 80.0 * rrs_error + 15.0 * error_depth + 10.0 * error_bottom + 15.0 * K_error;
  model /= 80.0 + 15.0 + 10.0 + 15.0;
  px->model_error = model;
  return model;
}

/* Cold start (model/samodel.c:2249-2353). */
static void region_cold_start(const po_rpixel *px, double H0, double *start, double *step) {
  const int R = px->R, S = px->S, nb = px->nb, off = R + 2 * nb * R;
  double m490 = 0.0, m550, m640;
  int r, s, k;
  for (r = 0; r < R; r++) {
    start[r] = H0;
    step[r] = 1.25 * start[r];
  }
  for (r = 0; r < R; r++)
    for (s = 0; s < S; s++) m490 += px->r490[r][s];
  m490 /= (double)R * S;
  for (k = 0; k < nb; k++)
    for (r = 0; r < R; r++) {
      start[R + r * nb + k] = 100.0 * 4.0 * m490;
      step[R + r * nb + k] = 1.5 * start[R + r * nb + k];
    }
  for (k = 0; k < nb; k++)
    for (r = 0; r < R; r++) {
      start[R + nb * R + r * nb + k] = 1.0;
      step[R + nb * R + r * nb + k] = 0.5 * start[R + nb * R + r * nb + k];
    }
  for (s = 0; s < S; s++) {
    m490 = 0.0;
    m550 = 0.0;
    m640 = 0.0;
    for (r = 0; r < R; r++) {
      m490 += px->r490[r][s];
      m550 += px->r550[r][s];
      m640 += px->r640[r][s];
    }
    m490 /= (double)R;
    m550 /= (double)R;
    m640 /= (double)R;
    start[off + 3 * s] = 100.0 * 0.072 * pow(m490 / m550, -1.7);
    start[off + 1 + 3 * s] = 1.5 * start[off + 3 * s];
    start[off + 2 + 3 * s] = 100.0 * 30.0 * px->sc[s]->aw640 * m640;
    step[off + 3 * s] = 2.0 * start[off + 3 * s];
    step[off + 1 + 3 * s] = 2.0 * start[off + 1 + 3 * s];
    step[off + 2 + 3 * s] = 2.0 * start[off + 2 + 3 * s];
  }
}

static void region_reference_rrs(po_rpixel *px) {
  int r, s;
  for (r = 0; r < px->R; r++) /* model/samodel.c:1785-1799 */
    for (s = 0; s < px->S; s++) {
      const double *wl = px->sc[s]->wl;
      px->r440[r][s] = po_interp_1d(wl, px->rrs[r][s], px->n_bands, 440.0);
      px->r490[r][s] = po_interp_1d(wl, px->rrs[r][s], px->n_bands, 490.0);
      px->r550[r][s] = po_interp_1d(wl, px->rrs[r][s], px->n_bands, 550.0);
      px->r640[r][s] = po_interp_1d(wl, px->rrs[r][s], px->n_bands, 640.0);
      px->r750[r][s] = po_interp_1d(wl, px->rrs[r][s], px->n_bands, 750.0);
      if (px->r440[r][s] < 0.0) px->r440[r][s] = 0.0001;
    }
}

/* samodel_optimise for one pixel's regions (model/samodel.c:1768-2115):
 * depth starts, nelmin, early exit, the final re-evaluation and the post-fit
 * products.  h_emp: the single depth start (an empirical depth, or the
 * previous pixel's under a hot start), or NaN for the 8 cold starts.
 * hot_prev (3 per scene, or NULL): the hot start's P, G, X, each with twice
 * itself as step (model/samodel.c:2234-2241, 2288-2309).  best_out
 * (optional) receives the kept parameter vector. */
static void region_fit(po_rpixel *px, const po_fit *fit, double h_emp, const double *hot_prev,
                       double *o, double *best_out) {
  const int R = px->R, S = px->S, n = region_n_params(px), nb = px->nb, off = R + 2 * nb * R;
  double start[PO_MAX_PARAMS], step[PO_MAX_PARAMS], xm[PO_MAX_PARAMS], best[PO_MAX_PARAMS];
  double lowest = 1.0e4, y = 0.0;
  int icount = 0, numres = 0, ifault = 0, k, r, s, b, nst;
  long total = 0;
  int kept_evals = 0, kept_res = 0, kept_start = 0, kept_fault = 0, converged = 0;
  region_reference_rrs(px);
  memset(best, 0, sizeof best);
  nst = isnan(h_emp) ? fit->n_hstarts : 1;
  for (k = 0; k < nst; k++) {
    region_cold_start(px, isnan(h_emp) ? fit->hstarts[k] : h_emp, start, step);
    if (hot_prev)
      for (s = 0; s < 3 * S; s++) {
        start[off + s] = hot_prev[s];
        step[off + s] = 2.0 * start[off + s];
      }
    po_nelmin(region_cost, px, n, start, xm, &y, fit->reqmin, step, fit->konvge, fit->kcount,
              &icount, &numres, &ifault);
    total += icount;
    if (y < lowest) {
      lowest = y;
      memcpy(best, xm, n * sizeof(double));
      kept_evals = icount;
      kept_res = numres;
      kept_start = k;
      kept_fault = ifault;
      converged = (ifault == 0);
      if (lowest < 2.5 * ((float)S)) break; /* model/samodel.c:2404 */
    }
  }
  region_cost(best, px);
  if (best_out) memcpy(best_out, best, n * sizeof(double));
  {
    double K_min = 1.0e10, iod = 0.0, nobs = 0.0, depth = 0.0, ow = sqrt((double)R);
    double q_sum = 0.0, pct[PO_MAX_MIX], largest = 0.0, type = 0.0;
    int found = 0;
    for (s = 0; s < S; s++) /* array_min_double2 over md->K, model/samodel.c:1994 */
      for (b = 0; b < px->n_bands; b++)
        if (!f_close((float)px->K[s][b], (float)0.0, 1.0e-4f) && px->K[s][b] < K_min) {
          K_min = px->K[s][b];
          found = 1;
        }
    if (!found) K_min = 0.0;
    for (r = 0; r < R; r++) { /* origin-weighted depth, model/samodel.c:1999-2017 */
      double H = fabs(best[r]);
      if (r == px->origin) depth += ow * H;
      else depth += H;
    }
    depth /= ow + ((double)R) - 1.0;
    /* bottom shares of the origin region and the bottom type,
     * model/samodel.c:2021-2047 */
    for (k = 0; k < nb; k++) q_sum += fabs(best[R + R * nb + px->origin * nb + k]);
    for (k = 0; k < nb; k++) pct[k] = 100.0 * fabs(best[R + R * nb + px->origin * nb + k]) / q_sum;
    for (k = 0; k < nb; k++)
      if (pct[k] > largest) {
        largest = pct[k];
        type = 1.0 + k;
      }
    for (s = 0; s < S; s++) /* model/samodel.c:2051-2064 */
      for (r = 0; r < R; r++)
        for (b = 0; b < px->n_bands; b++) {
          iod += px->rrs_bot[r][s][b] / px->rrs_mod[r][s][b];
          nobs += 1.0;
        }
    iod = 100.0 * iod / nobs;
    o[0] = depth;
    o[1] = px->bottom_albedo;
    o[2] = px->model_error;
    o[3] = px->rrs_error;
    o[4] = K_min;
    o[5] = iod;
    for (k = 0; k < nb; k++) o[40 + k] = pct[k];
    o[43] = type;
  }
  o[6] = (double)kept_evals;
  o[7] = (double)total;
  o[8] = converged ? 1.0 : 0.0;
  o[9] = 0.0;
  o[10] = (double)S;
  for (s = 0; s < S; s++) {
    o[11 + s] = 0.01 * fabs(best[off + 3 * s]);
    o[19 + s] = 0.01 * fabs(best[off + 1 + 3 * s]);
    o[27 + s] = 0.01 * fabs(best[off + 2 + 3 * s]);
  }
  o[35] = (double)kept_res;
  o[36] = (double)kept_start;
  o[37] = (double)kept_fault;
  o[38] = (double)R;
  o[39] = (double)px->origin;
}

/* extract_Rrs_data (model/samodel.c:2957-3027) for pixel p of a
 * [n_scenes][nrows][ncols][n_bands] grid: the regions' spectra, their count
 * and the origin's slot. */
static void region_extract(const float *grid, int n_scenes, int nrows, int ncols, int n_bands,
                           float nodata, int n_spatial, int64_t p, po_rpixel *px) {
  const int64_t npix = (int64_t)nrows * ncols;
  const int i = (int)(p / ncols), j = (int)(p % ncols), w = n_spatial - 1;
  int ii, jj, sk, b;
  px->R = 0;
  px->origin = 0;
  for (ii = -w; ii <= w; ii++) {
    const int iii = i + ii < 0 ? 0 : (i + ii > nrows - 1 ? nrows - 1 : i + ii);
    for (jj = -w; jj <= w; jj++) {
      const int jjj = j + jj < 0 ? 0 : (j + jj > ncols - 1 ? ncols - 1 : j + jj);
      int nodata_region = 0;
      for (sk = 0; sk < n_scenes && !nodata_region; sk++) {
        const float *q = grid + ((int64_t)sk * npix + (int64_t)iii * ncols + jjj) * n_bands;
        for (b = 0; b < n_bands; b++) {
          if (!f_close(q[b], nodata, 1.0e-6f)) {
            px->rrs[px->R][sk][b] = q[b];
          } else {
            nodata_region = 1;
            break;
          }
        }
      }
      if (i == iii && j == jjj) px->origin = px->R;
      if (!nodata_region) px->R++;
    }
  }
}

/* grid: [n_scenes][nrows][ncols][n_bands]; theta_sun_deg: [n_scenes]. */
int po_region_fit_batch(int n_bands, const double *wl, const double *theta_sun_deg,
                        double theta_view_deg, double h_tide, const float *grid, int n_scenes,
                        int nrows, int ncols, float nodata, int n_spatial, int n_bottoms,
                        const double *h_empirical, double reqmin, int konvge, int kcount,
                        int nthreads, double *out) {
  po_scene sc[PO_MAX_SCENES];
  po_fit fit;
  int64_t p, npix = (int64_t)nrows * ncols;
  int s;
  if (n_bands < 2 || n_bands > PO_MAX_BANDS || n_spatial < 1 || n_spatial > 2 ||
      n_bottoms < 1 || n_bottoms > PO_MAX_MIX || n_scenes < 1 || n_scenes > PO_MAX_SCENES)
    return 1;
  for (s = 0; s < n_scenes; s++)
    scene_init(&sc[s], n_bands, wl, theta_sun_deg[s], theta_view_deg, h_tide);
  fit.seed_step_scale = 1.0;
  fit.reqmin = reqmin;
  fit.konvge = konvge;
  fit.kcount = kcount;
  fit.n_hstarts = 8;
  fit.hstarts = po_default_hstarts;
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (p = 0; p < npix; p++) {
    double *o = out + p * PO_NOUT;
    double h_emp = NAN;
    po_rpixel px;
    int sk, bad = 0;
    memset(o, 0, PO_NOUT * sizeof(double));
    for (sk = 0; sk < n_scenes && !bad; sk++) /* model/samodel.c:933-947 */
      bad = masked(grid + ((int64_t)sk * npix + p) * n_bands, n_bands, nodata);
    if (bad) {
      o[9] = 1.0;
      continue;
    }
    memset(&px, 0, sizeof px);
    px.n_bands = n_bands;
    px.nb = n_bottoms;
    px.S = n_scenes;
    for (sk = 0; sk < n_scenes; sk++) px.sc[sk] = &sc[sk];
    if (h_empirical && !isnan(h_empirical[p])) {
      h_emp = h_empirical[p];
      if (h_emp > 8.0) px.nb = 1; /* model/samodel.c:1781, 1826-1830 */
    }
    region_extract(grid, n_scenes, nrows, ncols, n_bands, nodata, n_spatial, p, &px);
    if (px.R == 0) continue;
    region_fit(&px, &fit, h_emp, NULL, o, NULL);
  }
  return 0;
}

int po_region_invert_batch(int n_bands, const double *wl, double theta_sun_deg,
                           double theta_view_deg, double h_tide, const float *grid, int nrows,
                           int ncols, float nodata, double reqmin, int konvge, int kcount,
                           int nthreads, double *out) {
  return po_region_fit_batch(n_bands, wl, &theta_sun_deg, theta_view_deg, h_tide, grid, 1, nrows,
                             ncols, nodata, 2, 1, NULL, reqmin, konvge, kcount, nthreads, out);
}

/* Cost, with its side outputs, of one explicit parameter vector for a pixel
 * given as its regions' spectra (rrs [R][S][n_bands], origin region, nb
 * bottom types, one sun zenith per scene): samodel_error
 * (model/samodel.c:2432-2759).  details[5] = Rrs error, model error, bottom
 * albedo, the last scene's K_min (the cost's test), 0; rm [R][S][n_bands]
 * (optional) the modelled Rrs. */
double po_region_cost(int n_bands, const double *wl, const double *theta_sun_deg,
                      double theta_view_deg, double h_tide, const double *rrs, int R, int S,
                      int origin, int n_bottoms, const double *params, double *details,
                      double *rm) {
  po_scene sc[PO_MAX_SCENES];
  po_rpixel px;
  int r, s, b;
  double c, K_min = 1.0e4;
  memset(&px, 0, sizeof px);
  for (s = 0; s < S; s++) {
    scene_init(&sc[s], n_bands, wl, theta_sun_deg[s], theta_view_deg, h_tide);
    px.sc[s] = &sc[s];
  }
  px.n_bands = n_bands;
  px.nb = n_bottoms;
  px.R = R;
  px.S = S;
  px.origin = origin;
  for (r = 0; r < R; r++)
    for (s = 0; s < S; s++)
      for (b = 0; b < n_bands; b++) px.rrs[r][s][b] = rrs[(r * S + s) * n_bands + b];
  region_reference_rrs(&px);
  c = region_cost(params, &px);
  for (b = 0; b < n_bands; b++)
    if (!f_close((float)px.K[S - 1][b], 0.0f, 1.0e-6f) && px.K[S - 1][b] < K_min)
      K_min = px.K[S - 1][b];
  if (details) {
    details[0] = px.rrs_error;
    details[1] = px.model_error;
    details[2] = px.bottom_albedo;
    details[3] = K_min;
    details[4] = 0.0;
  }
  if (rm)
    for (r = 0; r < R; r++)
      for (s = 0; s < S; s++)
        for (b = 0; b < n_bands; b++) {
          const double rr = px.rrs_mod[r][s][b];
          rm[(r * S + s) * n_bands + b] = 0.5 * rr / (1.0 - 1.5 * rr);
        }
  return c;
}


/* ------------------------------------------------------------------------
 * netCDF short packing of a float grid (model/nc.c:14-336).
 *
 * decompress_2d (model/nc.c:251-266): a packed value equal to the file's
 * missing_value becomes (float) spval, every other c becomes
 * (float) c * scale_factor + add_offset, a float product and a float sum.
 *
 * compress_2d (model/nc.c:271-320): the minimum and maximum are taken in
 * one pass with `if (g < grmin) ... else if (g > grmax)` from
 * grmin = FLT_MAX, grmax = FLT_MIN (model/nc.c:285-297), so a value that is
 * a new running minimum is never compared with the maximum, and grmax never
 * drops below FLT_MIN; cells equal to (float) spval are skipped.  Each cell
 * becomes (short) rint((g - grmin) / scale) with scale =
 * (grmax - grmin) / (float) SHRT_MAX in float arithmetic (model/nc.c:301-318).
 * The double -> short conversion of a value outside the range of int (or
 * NaN, e.g. 0/0 when every cell is equal) is undefined in C; it is pinned
 * here to the x86-64 result: the truncating conversion to a 32-bit int
 * (INT_MIN when out of range or NaN), then its low 16 bits.
 * ------------------------------------------------------------------------ */
static int16_t nc_to_short_x86(double v) {
  int32_t i;
  if (v >= -2147483648.0 && v < 2147483648.0) i = (int32_t)v;
  else i = INT32_MIN;
  return (int16_t)(uint16_t)((uint32_t)i & 0xFFFFu);
}

void po_nc_decompress(const int16_t *packed, int64_t n, float add_offset, float scale_factor,
                      int16_t missing_value, double spval, float *grid) {
  for (int64_t k = 0; k < n; k++) {
    if (packed[k] == missing_value) grid[k] = (float)spval;
    else grid[k] = ((float)packed[k]) * scale_factor + add_offset;
  }
}

void po_nc_compress(const float *grid, int64_t n, double spval, int16_t *packed,
                    float *add_offset, float *scale_factor, int16_t *missing_value) {
  const float fspv = (float)spval;
  float grmin = FLT_MAX, grmax = FLT_MIN, scale;
  *missing_value = SHRT_MIN;
  for (int64_t k = 0; k < n; k++) {
    const float g = grid[k];
    if (g == fspv) continue;
    if (g < grmin) grmin = g;
    else if (g > grmax) grmax = g;
  }
  *add_offset = grmin;
  scale = (grmax - grmin) / ((float)SHRT_MAX);
  *scale_factor = scale;
  for (int64_t k = 0; k < n; k++) {
    if (grid[k] == fspv) packed[k] = *missing_value;
    else packed[k] = nc_to_short_x86(rint((grid[k] - grmin) / scale));
  }
}

/* ------------------------------------------------------------------------
 * Spatially coherent synthetic scene: smooth parameter fields over the
 * grid (three seeded harmonics each), so that neighbouring pixels -- and
 * pixels far apart on the same depth contour and bottom class -- have
 * nearly equal spectra, as an image has.  This is the workload of the dynamic lookup table; the
 * per-pixel generator above draws independent pixels, which a table never
 * matches.  New: the reference has no generator.
 * ---------------------------------------------------------------------- */
static double field_value(uint64_t seed, uint32_t which, double u, double v) {
  double s = 0.0, norm = 0.0;
  int h;
  for (h = 0; h < 3; h++) {
    double w[4], amp = 1.0 / (double)(1 << h);
    draw4(seed, (uint64_t)(which * 4u + (uint32_t)h), 7u, 1u, w);
    {
      double fx = 1.0 + floor(4.0 * w[0]), fy = 1.0 + floor(4.0 * w[1]);
      double ph = 2.0 * PO_PI * w[2];
      s += amp * sin(2.0 * PO_PI * (fx * u + fy * v) + ph);
    }
    norm += amp;
  }
  return 0.5 + 0.5 * s / norm; /* in [0, 1] */
}

void po_field_truth(uint64_t seed, int64_t nrows, int64_t ncols, int64_t i, int64_t j,
                    double *t5) {
  /* one water mass over the scene (P, G, X within +/-10 % of values drawn
   * once), depth a smooth field over 0.5-25 m, and the bottom in three
   * albedo classes (dark, mixed, bright) with +/-5 % texture */
  const double u = ((double)i + 0.5) / (double)nrows, v = ((double)j + 0.5) / (double)ncols;
  static const double classes[3] = {0.08, 0.2, 0.4};
  double w[4], tH = field_value(seed, 0u, u, v), tB = field_value(seed, 4u, u, v);
  int cls = tB < 0.4 ? 0 : (tB < 0.6 ? 1 : 2);
  draw4(seed, 0u, 9u, 1u, w);
  t5[0] = 0.5 + 24.5 * tH * tH;
  t5[1] = log_uniform(w[0], 0.01, 0.05) * (0.9 + 0.2 * field_value(seed, 1u, u, v));
  t5[2] = log_uniform(w[1], 0.01, 0.08) * (0.9 + 0.2 * field_value(seed, 2u, u, v));
  t5[3] = log_uniform(w[2], 0.002, 0.02) * (0.9 + 0.2 * field_value(seed, 3u, u, v));
  t5[4] = classes[cls] * (0.95 + 0.1 * field_value(seed, 5u, u, v));
}

void po_generate_field(uint64_t seed, int64_t nrows, int64_t ncols, int64_t row0, int64_t n_rows,
                       int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                       double mask_frac, double noise_sigma, float nodata, float *rrs_out,
                       double *truth_out) {
  po_scene sc;
  int64_t k, n = n_rows * ncols;
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, 0.0);
#if _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (k = 0; k < n; k++) {
    const int64_t i = row0 + k / ncols, j = k % ncols;
    const uint64_t p = (uint64_t)(i * ncols + j);
    double t5[5], u1[4], r[PO_MAX_BANDS];
    int b;
    po_field_truth(seed, nrows, ncols, i, j, t5);
    synthesise(&sc, t5[0], t5[1], t5[2], t5[3], t5[4], r);
    add_noise(seed, p, 0u, n_bands, noise_sigma, r);
    for (b = 0; b < n_bands; b++) rrs_out[k * n_bands + b] = (float)r[b];
    draw4(seed, p, 1u, 0u, u1);
    apply_mask(u1[1], u1[2], mask_frac, n_bands, nodata, rrs_out + k * n_bands);
    if (truth_out) memcpy(truth_out + k * 5, t5, sizeof t5);
  }
}

/* ------------------------------------------------------------------------
 * samodel()'s pixel loop with its dynamic lookup table, one scene, one
 * region, one bottom type (model/samodel.c:649-660, 701-773, 901-1215).
 *
 *   order    every pixel sorted ascending by the spectral index
 *            |(Rrs_blue, Rrs_green, Rrs_red)| (bands 1, 2, 3), times the
 *            spectral angle to the noise spectrum when every band's noise
 *            is at least 1e-6 (:706-770), with glibc's merge sort (po_msort:
 *            ties keep the pixel order); the shallow pixels (no band nodata
 *            or negative, :933-947) in that order;
 *   chains   the sorted list cut into n_chains contiguous slices; each
 *            slice runs the reference's loop on its own, as one OpenMP
 *            thread of the reference runs it over the pixels it is given,
 *            with the slice's length as n_shallow (one chain is the
 *            reference run on one thread);
 *   lookup   over the table's slots in order, the entries whose depth and
 *            K_min are within 10 % of the previous pixel's (relative to it
 *            plus epsilon = 1e-4f, common.c:93), the smallest
 *            model_spectral_diff_mean (:2792-2842; strict <, first slot);
 *   serve    when that difference is at most the match threshold: the
 *            entry's outputs (partial_copy_md, :3031-3139), model error =
 *            the difference (:1066-1073);
 *   fit      otherwise samodel_optimise, hot-started from the previous
 *            pixel when the last two pixels were continuous (:2234-2309),
 *            then entered into the oldest slot when its model error is
 *            below the entry threshold and its depth below 32 m
 *            (:1035-1063);
 *   adapt    both thresholds every 0.1 % of the slice from the model
 *            errors and the served share since the previous update
 *            (:1182-1211; the sums restart at every update, :1326-1352).
 * ---------------------------------------------------------------------- */
typedef struct {
  double depth, kmin, rm[3], prev[3];
  int64_t src;
} po_lut_entry;

typedef struct {
  float value;
  int64_t idx;
} po_key;

/* sort_indexes_2d (model/common.c:180-209) sorts every pixel's index with
 * glibc's qsort, a top-down merge sort: halves of n / 2 and n - n / 2, the
 * merge taking the left element unless it compares greater.  The
 * comparator (cmp_floats, model/common.c:165-177) calls a NaN equal to
 * everything, so NaN indices -- pixels whose blue, green and red are all
 * nodata or zero, under the spectral-angle order -- stay where the merges
 * leave them; restating the same merge tree reproduces that order. */
static void po_msort(po_key *b, po_key *tmp, size_t n) {
  size_t n1, n2, i = 0, j, o = 0;
  if (n <= 1) return;
  n1 = n / 2;
  n2 = n - n1;
  po_msort(b, tmp, n1);
  po_msort(b + n1, tmp, n2);
  j = n1;
  while (i < n1 && j < n) {
    if (!(b[i].value > b[j].value))
      tmp[o++] = b[i++];
    else
      tmp[o++] = b[j++];
  }
  while (i < n1) tmp[o++] = b[i++];
  /* the right run's tail is already in place */
  memcpy(b, tmp, o * sizeof(po_key));
}

/* approx_equal of model/common.c:392-394: float arguments, double product */
static int ref_approx_eq(float a, float b, float eps) {
  return fabs(a - b) <= ((fabs(a) < fabs(b) ? fabs(b) : fabs(a)) * eps);
}

/* model_spectral_diff_mean (model/samodel.c:2792-2842) for one region and
 * one scene: bands 1..3 below n_bands. */
static float lut_spectral_diff(const double *meas, const double *lut_rm, int n_bands) {
  double error = 0.0;
  int k, n_total = 0;
  for (k = 1; k <= 3 && k < n_bands; k++) {
    double current = 0.0, previous = 0.0, nobs = 0.0;
    if (!ref_approx_eq((float)meas[k], 0.0f, 1.0e-6f) &&
        !ref_approx_eq((float)lut_rm[k - 1], 0.0f, 1.0e-6f)) {
      current += meas[k];
      previous += lut_rm[k - 1];
      nobs += 1.0;
    }
    if (nobs > 0.5) {
      current /= nobs;
      previous /= nobs;
    }
    error += pow((current - previous) / current, 2.0);
    n_total++;
  }
  error = 100.0 * sqrt(error / ((double)n_total));
  return (float)error;
}

/* The spectral index of one pixel (model/samodel.c:711-767), one scene. */
float po_lut_key(const float *r, int n_bands, float nodata, const double *noise) {
  float blue_sum = 0.0f, green_sum = 0.0f, red_sum = 0.0f, index;
  if (n_bands > 1 && !ref_approx_eq(r[1], nodata, 1.0e-6f)) blue_sum += r[1];
  if (n_bands > 2 && !ref_approx_eq(r[2], nodata, 1.0e-6f)) green_sum += r[2];
  if (n_bands > 3 && !ref_approx_eq(r[3], nodata, 1.0e-6f)) red_sum += r[3];
  index = (float)sqrt(pow(blue_sum, 2) + pow(green_sum, 2) + pow(red_sum, 2));
  if (noise) {
    double bn = 0.0, gn = 0.0, rn = 0.0, angle;
    bn += noise[1];
    gn += noise[2];
    rn += noise[3];
    angle = blue_sum * bn + green_sum * gn + red_sum * rn;
    angle /= index * sqrt(pow(bn, 2) + pow(gn, 2) + pow(rn, 2));
    angle = acos(angle);
    index *= angle;
  }
  return index;
}

static void lut_chain(const po_scene *sc, const po_fit *fit, const float *rrs, int nb,
                      const float *emp, float emp_nodata, const int64_t *order, int64_t n,
                      int n_lut, double *out, int64_t *source, double *stats) {
  const double eps = (double)1.0e-4f; /* the reference's global float epsilon */
  const double continuity = 0.1;
  const int64_t cap = n < (int64_t)n_lut ? n : (int64_t)n_lut;
  po_lut_entry *lut = (po_lut_entry *)calloc((size_t)(cap > 0 ? cap : 1), sizeof(po_lut_entry));
  int64_t total_lut = 0, k, n_complete = 0, err_count = 0, n_opt = 0;
  double md_depth = 0.0, md_kmin = 0.0, depth_prev = 0.0, kmin_prev = 0.0, prev[3] = {0, 0, 0};
  double match = 1.125 > 1.5 ? 1.125 : 1.5, entry; /* MAX(1.5, 1.125 n_scenes) */
  double n_modelled = 0.0, n_skipped = 0.0, total_model_error = 0.0, err_total = 0.0;
  int hot = 0, nprev = 0, nperc;
  entry = match;
  for (k = 0; k < n; k++) {
    const int64_t p = order[k];
    const float *r = rrs + p * nb;
    double meas[PO_MAX_BANDS], best = 1.0e4, model_error;
    int64_t pos = 0, j, in_use = total_lut < cap ? total_lut : cap;
    int b;
    for (b = 0; b < nb; b++) meas[b] = (double)r[b];
    for (j = 0; j < in_use; j++) {
      const po_lut_entry *e = lut + j;
      if (fabs(e->depth - md_depth) / (md_depth + eps) < continuity &&
          fabs(e->kmin - md_kmin) / (md_kmin + eps) < continuity) {
        double d = (double)lut_spectral_diff(meas, e->rm, nb);
        if (d < best) {
          best = d;
          pos = j;
        }
      }
    }
    if (best > match || in_use == 0) { /* see photic_lut.cu on an empty table */
      po_pixel px;
      double seed[6], bestv[PO_MAX_PARAMS], *o = out + p * PO_NOUT, h_emp = 0.0;
      int emp_present = 0, use_hot = hot;
      po_fit f1 = *fit;
      if (emp) { /* the pixel's empirical depth (:955-979) */
        if (!ref_approx_eq(emp[p], emp_nodata, 1.0e-6f)) {
          emp_present = 1;
          h_emp = emp[p] > -1.0 ? 1.0 : fabs(emp[p]);
        } else {
          use_hot = 0;
        }
      }
      memset(&px, 0, sizeof px);
      px.n_scenes = 1;
      px.n_bands = nb;
      px.n_bottoms = 1;
      px.layout = PO_LAYOUT_REFERENCE;
      px.sc[0] = sc;
      for (b = 0; b < nb; b++) px.rrs[0][b] = meas[b];
      pixel_reference_rrs(&px);
      if (use_hot) { /* :2234-2241: the empirical depth keeps its start */
        seed[0] = emp_present ? h_emp : depth_prev;
        seed[1] = 100.0 * 4.0 * (px.r490[0] / (double)1);
        seed[2] = 1.0;
        seed[3] = prev[0];
        seed[4] = prev[1];
        seed[5] = prev[2];
      } else if (emp_present) { /* one cold start at the empirical depth (:2221-2223) */
        f1.n_hstarts = 1;
        f1.hstarts = &h_emp;
      }
      fit_pixel_ex(&px, &f1, use_hot ? seed : NULL, o, bestv);
      source[p] = -1;
      md_depth = o[0];
      md_kmin = o[4];
      model_error = o[2];
      prev[0] = fabs(bestv[3]);
      prev[1] = fabs(bestv[4]);
      prev[2] = fabs(bestv[5]);
      n_opt++;
      if (!ref_approx_eq((float)model_error, 0.0f, 1.0e-4f)) { /* vec_mean2_double */
        err_total += model_error;
        err_count++;
      }
      if (model_error < entry && md_depth < 32.0) {
        po_lut_entry *e = lut + (total_lut % cap);
        e->depth = md_depth;
        e->kmin = md_kmin;
        for (b = 0; b < 3; b++) e->rm[b] = b + 1 < nb ? px.Rm[0][b + 1] : 0.0;
        memcpy(e->prev, prev, sizeof prev);
        e->src = p;
        total_lut++;
      }
      if (stats) stats[1] += 1.0;
    } else {
      const po_lut_entry *e = lut + pos;
      depth_prev = md_depth;
      kmin_prev = md_kmin;
      md_depth = e->depth;
      md_kmin = e->kmin;
      memcpy(prev, e->prev, sizeof prev);
      model_error = best;
      memcpy(out + p * PO_NOUT, out + e->src * PO_NOUT, PO_NOUT * sizeof(double));
      out[p * PO_NOUT + 2] = best;
      source[p] = e->src;
      n_skipped += 1.0;
      if (stats) stats[0] += 1.0;
    }
    hot = fabs(md_depth - depth_prev) / (eps + depth_prev) < continuity &&
          fabs(md_kmin - kmin_prev) / (eps + kmin_prev) < continuity;
    depth_prev = md_depth;
    kmin_prev = md_kmin;
    total_model_error += model_error;
    n_modelled += 1.0;
    nperc = (int)(1000 * ((double)++n_complete) / ((double)n));
    if (nperc > nprev) {
      if (n_opt > 0) {
        const double error_mean = (float)(err_count ? err_total / ((double)err_count) : 0.0);
        match += 0.75 * error_mean + 0.25 * total_model_error / n_modelled;
        match /= 2.0;
        entry = match;
      }
      if (n_skipped / n_modelled > 0.9925) {
        match *= 0.75;
        entry *= 0.75;
      }
      match = 1.5 > match ? 1.5 : match;
      entry = 1.5 > entry ? 1.5 : entry;
      nprev = nperc;
      /* the statistics restart with every display (:1326-1352) */
      total_model_error = 0.0;
      n_modelled = 0.0;
      n_skipped = 0.0;
      n_opt = 0;
      err_total = 0.0;
      err_count = 0;
    }
  }
  if (stats) {
    stats[2] = match;
    stats[3] = entry;
  }
  free(lut);
}

int po_lut_invert(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                  double h_tide, const float *rrs, int64_t npix, float nodata,
                  const double *rrs_noise, const float *emp, float emp_nodata, double reqmin,
                  int konvge, int kcount, int n_lut, int64_t n_chains, int nthreads,
                  int64_t *order_out, int64_t *n_shallow_out, double *out, int64_t *source,
                  double *chain_stats) {
  po_scene sc;
  po_fit fit;
  po_key *keys;
  int64_t p, S = 0, c;
  const double *noise = NULL;
  if (n_bands < 2 || n_bands > PO_MAX_BANDS || n_lut < 1 || n_chains < 1) return 1;
  if (rrs_noise) {
    int b, ok = 1;
    for (b = 0; b < n_bands; b++)
      if (rrs_noise[b] < 1.0e-6) ok = 0; /* model/samodel.c:590-600 */
    if (ok) noise = rrs_noise;
  }
  scene_init(&sc, n_bands, wl, theta_sun_deg, theta_view_deg, h_tide);
  fit.seed_step_scale = 1.0;
  fit.reqmin = reqmin;
  fit.konvge = konvge;
  fit.kcount = kcount;
  fit.n_hstarts = 8;
  fit.hstarts = po_default_hstarts;
  keys = (po_key *)malloc((size_t)(npix > 0 ? npix : 1) * sizeof(po_key));
  {
    po_key *tmp = (po_key *)malloc((size_t)(npix > 0 ? npix : 1) * sizeof(po_key));
    /* every pixel is keyed and sorted (:701-772); the masked ones are then
     * left out of the shallow list (:790-812) */
    for (p = 0; p < npix; p++) {
      /* the empirical depth itself when a grid of them is given (:708-710) */
      keys[p].value = emp ? emp[p] : po_lut_key(rrs + p * n_bands, n_bands, nodata, noise);
      keys[p].idx = p;
    }
    po_msort(keys, tmp, (size_t)npix);
    free(tmp);
  }
  for (p = 0; p < npix; p++) {
    const float *r = rrs + keys[p].idx * n_bands;
    memset(out + keys[p].idx * PO_NOUT, 0, PO_NOUT * sizeof(double));
    if (masked(r, n_bands, nodata)) {
      out[keys[p].idx * PO_NOUT + 9] = 1.0;
      source[keys[p].idx] = -2;
      continue;
    }
    order_out[S++] = keys[p].idx;
  }
  free(keys);
  *n_shallow_out = S;
  if (n_chains > S) n_chains = S > 0 ? S : 1;
  if (chain_stats) memset(chain_stats, 0, (size_t)n_chains * 4 * sizeof(double));
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (c = 0; c < n_chains; c++) {
    const int64_t a = c * S / n_chains, e = (c + 1) * S / n_chains;
    lut_chain(&sc, &fit, rrs, n_bands, emp, emp_nodata, order_out + a, e - a, n_lut, out,
              source, chain_stats ? chain_stats + 4 * c : NULL);
  }
  return 0;
}

/* ---- the pixel loop with its lookup table, general configuration -------
 * samodel() with LUT 1 (model/samodel.c:649-1352) for 3 x 3 regions, bottom
 * mixtures and stacks of scenes: the loop of lut_chain above with
 *   keys     blue, green and red summed over the scenes, each value that is
 *            not nodata, and the noise spectra summed over the scenes for
 *            the spectral angle (:711-767);
 *   shallow  every band of every scene neither nodata nor negative;
 *   lookup   entries with the pixel's region count (:985), the mean over
 *            scenes and regions of the measured and modelled Rrs of bands
 *            1..3 where both are non-zero (model_spectral_diff_mean,
 *            :2792-2842, scene-major sums);
 *   fit      samodel_optimise over the regions (region_fit), hot-started
 *            from the previous pixel when the last two were continuous: one
 *            depth start at the previous depth (or the empirical depth) for
 *            every region, cold albedos and mixing weights, each scene's
 *            P, G, X from the previous fit (:2234-2241, 2288-2309);
 *   entry    the fit's region count, depth, K_min, modelled Rrs of bands
 *            1..3 per region and scene, and P, G, X (partial_copy_md,
 *            :3031-3139).
 * h_empirical, which selects sand alone above 8 m (:1826), is set only by
 * a pixel with an empirical depth and kept by the pixels after it; before
 * the first such pixel the reference leaves it unset (md is allocated with
 * malloc, :375): it is taken as 0 here, i.e. every bottom type is fitted,
 * as in the reference runs the fixtures come from. */
typedef struct {
  int R;
  double depth, kmin;
  double rm[PO_MAX_REGIONS][PO_MAX_SCENES][3];
  double prev[3 * PO_MAX_SCENES];
  int64_t src;
} po_glut_entry;

static float glut_spectral_diff(const po_rpixel *px, const po_glut_entry *e) {
  double error = 0.0;
  int k, r, s, n_total = 0;
  for (k = 1; k <= 3 && k < px->n_bands; k++) {
    double current = 0.0, previous = 0.0, nobs = 0.0;
    for (s = 0; s < px->S; s++)
      for (r = 0; r < px->R; r++)
        if (!ref_approx_eq((float)px->rrs[r][s][k], 0.0f, 1.0e-6f) &&
            !ref_approx_eq((float)e->rm[r][s][k - 1], 0.0f, 1.0e-6f)) {
          current += px->rrs[r][s][k];
          previous += e->rm[r][s][k - 1];
          nobs += 1.0;
        }
    if (nobs > 0.5) {
      current /= nobs;
      previous /= nobs;
    }
    error += pow((current - previous) / current, 2.0);
    n_total++;
  }
  error = 100.0 * sqrt(error / ((double)n_total));
  return (float)error;
}

/* The spectral index of pixel p over n_scenes scenes (model/samodel.c:
 * 711-767); noise: [n_scenes][n_bands] or NULL. */
float po_glut_key(const float *grid, int n_scenes, int64_t npix, int64_t p, int n_bands,
                  float nodata, const double *noise) {
  float blue_sum = 0.0f, green_sum = 0.0f, red_sum = 0.0f, index;
  int s;
  for (s = 0; s < n_scenes; s++) {
    const float *r = grid + ((int64_t)s * npix + p) * n_bands;
    if (n_bands > 1 && !ref_approx_eq(r[1], nodata, 1.0e-6f)) blue_sum += r[1];
    if (n_bands > 2 && !ref_approx_eq(r[2], nodata, 1.0e-6f)) green_sum += r[2];
    if (n_bands > 3 && !ref_approx_eq(r[3], nodata, 1.0e-6f)) red_sum += r[3];
  }
  index = (float)sqrt(pow(blue_sum, 2) + pow(green_sum, 2) + pow(red_sum, 2));
  if (noise) {
    double bn = 0.0, gn = 0.0, rn = 0.0, angle;
    for (s = 0; s < n_scenes; s++) {
      bn += noise[s * n_bands + 1];
      gn += noise[s * n_bands + 2];
      rn += noise[s * n_bands + 3];
    }
    angle = blue_sum * bn + green_sum * gn + red_sum * rn;
    angle /= index * sqrt(pow(bn, 2) + pow(gn, 2) + pow(rn, 2));
    angle = acos(angle);
    index *= angle;
  }
  return index;
}

typedef struct {
  const po_scene *sc;
  const po_fit *fit;
  const float *grid;
  int S, nrows, ncols, nb, n_spatial, n_bottoms;
  float nodata;
  const float *emp;
  float emp_nodata;
  int n_lut;
} po_glut_ctx;

static void glut_chain(const po_glut_ctx *g, const int64_t *order, int64_t n, double *out,
                       int64_t *source, double *stats) {
  const double eps = (double)1.0e-4f;
  const double continuity = 0.1;
  const int S = g->S;
  const int64_t cap = n < (int64_t)g->n_lut ? n : (int64_t)g->n_lut;
  po_glut_entry *lut =
      (po_glut_entry *)calloc((size_t)(cap > 0 ? cap : 1), sizeof(po_glut_entry));
  int64_t total_lut = 0, k, n_complete = 0, err_count = 0, n_opt = 0;
  double md_depth = 0.0, md_kmin = 0.0, depth_prev = 0.0, kmin_prev = 0.0;
  double prev[3 * PO_MAX_SCENES], h_emp_state = 0.0;
  double match = 1.125 * (double)S > 1.5 ? 1.125 * (double)S : 1.5, entry;
  double n_modelled = 0.0, n_skipped = 0.0, total_model_error = 0.0, err_total = 0.0;
  int hot = 0, nprev = 0, nperc, i;
  memset(prev, 0, sizeof prev);
  entry = match;
  for (k = 0; k < n; k++) {
    const int64_t p = order[k];
    po_rpixel px;
    double best = 1.0e4, model_error, h_emp = NAN;
    int64_t pos = 0, j, in_use = total_lut < cap ? total_lut : cap;
    int emp_present = 0, s;
    memset(&px, 0, sizeof px);
    px.n_bands = g->nb;
    px.S = S;
    px.nb = g->n_bottoms;
    for (s = 0; s < S; s++) px.sc[s] = &g->sc[s];
    region_extract(g->grid, S, g->nrows, g->ncols, g->nb, g->nodata, g->n_spatial, p, &px);
    if (px.R == 0) continue; /* :951-953 (a shallow pixel keeps its own region) */
    if (g->emp) { /* :955-976 */
      if (!ref_approx_eq(g->emp[p], g->emp_nodata, 1.0e-6f)) {
        emp_present = 1;
        h_emp_state = g->emp[p] > -1.0 ? 1.0 : fabs(g->emp[p]);
        h_emp = h_emp_state;
      } else {
        hot = 0;
      }
    }
    for (j = 0; j < in_use; j++) {
      const po_glut_entry *e = lut + j;
      if (e->R == px.R && fabs(e->depth - md_depth) / (md_depth + eps) < continuity &&
          fabs(e->kmin - md_kmin) / (md_kmin + eps) < continuity) {
        double d = (double)glut_spectral_diff(&px, e);
        if (d < best) {
          best = d;
          pos = j;
        }
      }
    }
    if (best > match || in_use == 0) {
      double bestv[PO_MAX_PARAMS], *o = out + p * PO_NOUT, h0 = h_emp;
      int off;
      if (h_emp_state > 8.0) px.nb = 1; /* :1826-1830 */
      off = px.R + 2 * px.nb * px.R;
      if (hot && !emp_present) h0 = depth_prev;
      region_fit(&px, g->fit, h0, hot ? prev : NULL, o, bestv);
      source[p] = -1;
      md_depth = o[0];
      md_kmin = o[4];
      model_error = o[2];
      for (i = 0; i < 3 * S; i++) prev[i] = fabs(bestv[off + i]); /* :2086-2099 */
      n_opt++;
      if (!ref_approx_eq((float)model_error, 0.0f, 1.0e-4f)) {
        err_total += model_error;
        err_count++;
      }
      if (model_error < entry && md_depth < 32.0) {
        po_glut_entry *e = lut + (total_lut % cap);
        int r, b;
        e->R = px.R;
        e->depth = md_depth;
        e->kmin = md_kmin;
        for (r = 0; r < px.R; r++)
          for (s = 0; s < S; s++)
            for (b = 0; b < 3; b++) e->rm[r][s][b] = b + 1 < g->nb ? px.Rm[r][s][b + 1] : 0.0;
        memcpy(e->prev, prev, sizeof prev);
        e->src = p;
        total_lut++;
      }
      if (stats) stats[1] += 1.0;
    } else {
      const po_glut_entry *e = lut + pos;
      depth_prev = md_depth;
      kmin_prev = md_kmin;
      md_depth = e->depth;
      md_kmin = e->kmin;
      memcpy(prev, e->prev, sizeof prev);
      model_error = best;
      memcpy(out + p * PO_NOUT, out + e->src * PO_NOUT, PO_NOUT * sizeof(double));
      out[p * PO_NOUT + 2] = best;
      source[p] = e->src;
      n_skipped += 1.0;
      if (stats) stats[0] += 1.0;
    }
    hot = fabs(md_depth - depth_prev) / (eps + depth_prev) < continuity &&
          fabs(md_kmin - kmin_prev) / (eps + kmin_prev) < continuity;
    depth_prev = md_depth;
    kmin_prev = md_kmin;
    total_model_error += model_error;
    n_modelled += 1.0;
    nperc = (int)(1000 * ((double)++n_complete) / ((double)n));
    if (nperc > nprev) {
      if (n_opt > 0) {
        const double error_mean = (float)(err_count ? err_total / ((double)err_count) : 0.0);
        match += 0.75 * error_mean + 0.25 * total_model_error / n_modelled;
        match /= 2.0;
        entry = match;
      }
      if (n_skipped / n_modelled > 0.9925) {
        match *= 0.75;
        entry *= 0.75;
      }
      match = 1.5 > match ? 1.5 : match;
      entry = 1.5 > entry ? 1.5 : entry;
      nprev = nperc;
      total_model_error = 0.0;
      n_modelled = 0.0;
      n_skipped = 0.0;
      n_opt = 0;
      err_total = 0.0;
      err_count = 0;
    }
  }
  if (stats) {
    stats[2] = match;
    stats[3] = entry;
  }
  free(lut);
}

/* grid: [n_scenes][nrows][ncols][n_bands]; theta_sun_deg, rrs_noise:
 * per scene ([n_scenes], [n_scenes][n_bands]; the noise only when every
 * value is at least 1e-6, :590-600, and n_bands >= 4); emp: [nrows][ncols]
 * empirical depths or NULL.  Outputs as po_lut_invert. */
int po_glut_invert(int n_bands, const double *wl, const double *theta_sun_deg,
                   double theta_view_deg, double h_tide, const float *grid, int n_scenes,
                   int nrows, int ncols, float nodata, int n_spatial, int n_bottoms,
                   const double *rrs_noise, const float *emp, float emp_nodata, double reqmin,
                   int konvge, int kcount, int n_lut, int64_t n_chains, int nthreads,
                   int64_t *order_out, int64_t *n_shallow_out, double *out, int64_t *source,
                   double *chain_stats) {
  po_scene sc[PO_MAX_SCENES];
  po_fit fit;
  po_glut_ctx g;
  po_key *keys;
  const int64_t npix = (int64_t)nrows * ncols;
  int64_t p, S = 0, c;
  const double *noise = NULL;
  int s;
  if (n_bands < 2 || n_bands > PO_MAX_BANDS || n_lut < 1 || n_chains < 1 || n_scenes < 1 ||
      n_scenes > PO_MAX_SCENES || n_spatial < 1 || n_spatial > 2 || n_bottoms < 1 ||
      n_bottoms > PO_MAX_MIX)
    return 1;
  if (rrs_noise && n_bands >= 4) {
    int b, ok = 1;
    for (s = 0; s < n_scenes; s++)
      for (b = 0; b < n_bands; b++)
        if (rrs_noise[s * n_bands + b] < 1.0e-6) ok = 0;
    if (ok) noise = rrs_noise;
  }
  for (s = 0; s < n_scenes; s++)
    scene_init(&sc[s], n_bands, wl, theta_sun_deg[s], theta_view_deg, h_tide);
  fit.seed_step_scale = 1.0;
  fit.reqmin = reqmin;
  fit.konvge = konvge;
  fit.kcount = kcount;
  fit.n_hstarts = 8;
  fit.hstarts = po_default_hstarts;
  keys = (po_key *)malloc((size_t)(npix > 0 ? npix : 1) * sizeof(po_key));
  {
    po_key *tmp = (po_key *)malloc((size_t)(npix > 0 ? npix : 1) * sizeof(po_key));
    for (p = 0; p < npix; p++) {
      keys[p].value = emp ? emp[p] : po_glut_key(grid, n_scenes, npix, p, n_bands, nodata, noise);
      keys[p].idx = p;
    }
    po_msort(keys, tmp, (size_t)npix);
    free(tmp);
  }
  for (p = 0; p < npix; p++) {
    const int64_t q = keys[p].idx;
    int bad = 0;
    memset(out + q * PO_NOUT, 0, PO_NOUT * sizeof(double));
    for (s = 0; s < n_scenes && !bad; s++)
      bad = masked(grid + ((int64_t)s * npix + q) * n_bands, n_bands, nodata);
    if (bad) {
      out[q * PO_NOUT + 9] = 1.0;
      source[q] = -2;
      continue;
    }
    order_out[S++] = q;
  }
  free(keys);
  *n_shallow_out = S;
  if (n_chains > S) n_chains = S > 0 ? S : 1;
  if (chain_stats) memset(chain_stats, 0, (size_t)n_chains * 4 * sizeof(double));
  g.sc = sc;
  g.fit = &fit;
  g.grid = grid;
  g.S = n_scenes;
  g.nrows = nrows;
  g.ncols = ncols;
  g.nb = n_bands;
  g.n_spatial = n_spatial;
  g.n_bottoms = n_bottoms;
  g.nodata = nodata;
  g.emp = emp;
  g.emp_nodata = emp_nodata;
  g.n_lut = n_lut;
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (c = 0; c < n_chains; c++) {
    const int64_t a = c * S / n_chains, e = (c + 1) * S / n_chains;
    glut_chain(&g, order_out + a, e - a, out, source, chain_stats ? chain_stats + 4 * c : NULL);
  }
  return 0;
}

/* The depth uncertainty for the general fit (model/samodel.c:1368-1479
 * with regions, bottom mixtures or scene stacks): the samples of
 * po_depth_sigma, each sampled pixel's regions (extract_Rrs_data) with
 * every band of every scene moved by n r_sigma[scene][band] in double and
 * stored as float (as the GPU's region lists hold them), refitted cold by
 * the general fit with every bottom type (h_empirical 5 m, :1448).  grid:
 * [n_scenes][nrows][ncols][n_bands]; r_sigma: [n_scenes][n_bands]. */
int po_region_depth_sigma(int n_bands, const double *wl, const double *theta_sun_deg,
                          double theta_view_deg, const float *grid, int n_scenes, int nrows,
                          int ncols, float nodata, int n_spatial, int n_bottoms,
                          const float *depth, const double *r_sigma, int n_samples,
                          uint64_t seed, double reqmin, int konvge, int kcount, int nthreads,
                          const double *sample_depth_in, int32_t *sample_pixel,
                          double *sample_depth, double *table, float *depth_sigma) {
  const double interval = 0.25;
  const int64_t npix = (int64_t)nrows * ncols, ns = (int64_t)PO_DS_MAX * n_samples;
  const int n_int = ds_intervals_host(depth, npix, interval);
  po_scene sc[PO_MAX_SCENES];
  po_fit fit;
  int64_t g;
  int s;
  float *sn;
  if (n_bands < 2 || n_bands > PO_MAX_BANDS || n_scenes < 1 || n_scenes > PO_MAX_SCENES ||
      n_spatial < 1 || n_spatial > 2 || n_bottoms < 1 || n_bottoms > PO_MAX_MIX)
    return 1;
  sn = (float *)malloc((size_t)ns * sizeof(float));
  if (!sn) return 1;
  ds_select_host(depth, npix, n_samples, seed, n_int, interval, sample_pixel, sn);
  if (sample_depth_in) {
    memcpy(sample_depth, sample_depth_in, (size_t)ns * sizeof(double));
  } else {
    for (s = 0; s < n_scenes; s++)
      scene_init(&sc[s], n_bands, wl, theta_sun_deg[s], theta_view_deg, 0.0);
    fit.seed_step_scale = 1.0;
    fit.reqmin = reqmin;
    fit.konvge = konvge;
    fit.kcount = kcount;
    fit.n_hstarts = 8;
    fit.hstarts = po_default_hstarts;
#if _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (g = 0; g < ns; g++) {
      po_rpixel px;
      double o[PO_NOUT];
      int r, k, b;
      const int moved = !po_approx_f(sn[g], 0.0f, 1.0e-6f);
      sample_depth[g] = 0.0;
      if (sample_pixel[g] < 0) continue;
      memset(&px, 0, sizeof px);
      px.n_bands = n_bands;
      px.S = n_scenes;
      px.nb = n_bottoms;
      for (k = 0; k < n_scenes; k++) px.sc[k] = &sc[k];
      region_extract(grid, n_scenes, nrows, ncols, n_bands, nodata, n_spatial, sample_pixel[g],
                     &px);
      if (px.R == 0) continue;
      for (r = 0; r < px.R; r++)
        for (k = 0; k < n_scenes; k++)
          for (b = 0; b < n_bands; b++) {
            double v = px.rrs[r][k][b];
            if (moved) v += (double)sn[g] * r_sigma[k * n_bands + b];
            px.rrs[r][k][b] = (double)(float)v;
          }
      region_fit(&px, &fit, NAN, NULL, o, NULL);
      sample_depth[g] = o[0];
    }
  }
  free(sn);
  ds_finish_host(sample_depth, n_samples, n_int, interval, depth, npix, table, depth_sigma);
  return 0;
}
