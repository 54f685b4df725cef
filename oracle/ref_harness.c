/*
 * ref_harness.c -- batch driver around the REFERENCE's own inversion code.
 *
 * Test infrastructure only.  This file is compiled together with the
 * reference's unmodified model/samodel.c, model/asa047.c and model/common.c
 * (read in place, never copied) by oracle/Makefile into
 * oracle/_ref/libphotic_ref.so.  It exists to (1) pin the C restatement in
 * oracle/photic_oracle.c and (2) generate the golden fixtures under
 * tests/golden/.  Nothing in the product links or loads it.
 *
 * What it adds around the reference:
 *   - model_data set-up for one pixel, following samodel() in
 *     model/samodel.c:375-618 (table interpolation at band wavelengths,
 *     subsurface angles to secants, bottom table assembly :464-487);
 *   - the nodata/negative pixel mask of model/samodel.c:933-947;
 *   - a per-thread tolerance override.  The reference hard-codes
 *     reqmin/konvge/kcount as locals of
 *     samodel_optimise_one_bottom_combination (model/samodel.c:2142-2144);
 *     samodel.c is compiled with -Dnelmin=photic_ref_nelmin_shim so that its
 *     single nelmin call (model/samodel.c:2371) lands in the shim below,
 *     which swaps in the requested tolerances and forwards to the real
 *     nelmin from model/asa047.c.  Everything else -- start/step
 *     construction, the 8 depth starts, early exit, post-fit products -- is
 *     the reference's own code path.
 *   - an OpenMP parallel-for over pixels with one model_data per thread,
 *     mirroring the reference's schedule(dynamic) loop (model/samodel.c:901).
 */
#include "samodel.h"
#include <stdint.h>
#if _OPENMP
#include <omp.h>
#endif

/* Spectral tables defined at file scope in model/samodel.c:105-287. */
extern int n_ref_wlens;
extern double ref_wlens[], aw_Pope_Fry1997[], bbw_Morel_1974[], a0_Lee[], a1_Lee[];
extern double bottom_type_sand[], bottom_type_seagrass[], bottom_type_coral[],
    bottom_type_macrophytes[], bottom_type_dark_sediment[], bottom_type_coral_sand[],
    bottom_type_green_algae[], bottom_type_red_algae[];

#define REF_MAX_SCENES 8
#define REF_MAX_BANDS 8
#define REF_N_BOTTOM_TABLE 8
#define REF_NOUT 44

typedef struct {
  int active;
  double reqmin;
  int konvge;
  int kcount;
  long long evals;
} ref_tol_t;

static __thread ref_tol_t g_tol;

void photic_ref_nelmin_shim(double fn(double x[], model_data *md), model_data *md, int n,
                            double start[], double xmin[], double *ynewlo, double reqmin,
                            double step[], int konvge, int kcount, int *icount, int *numres,
                            int *ifault) {
  if (g_tol.active) {
    reqmin = g_tol.reqmin;
    konvge = g_tol.konvge;
    kcount = g_tol.kcount;
  }
  nelmin(fn, md, n, start, xmin, ynewlo, reqmin, step, konvge, kcount, icount, numres, ifault);
  g_tol.evals += *icount;
}

static double *bottom_table(int k) {
  /* Order of the HYDROLIGHT bottom table, model/samodel.c:464-475. */
  switch (k) {
    case 0: return bottom_type_sand;
    case 1: return bottom_type_seagrass;
    case 2: return bottom_type_coral;
    case 3: return bottom_type_macrophytes;
    case 4: return bottom_type_dark_sediment;
    case 5: return bottom_type_coral_sand;
    case 6: return bottom_type_green_algae;
    default: return bottom_type_red_algae;
  }
}

/* model_data for up to R spatial regions (R = 1: one pixel). */
static model_data *md_new_r(int R) {
  model_data *md = (model_data *)calloc(1, sizeof(model_data));
  int S = REF_MAX_SCENES, B = REF_MAX_BANDS;
  md->max_n_regions = R;
  md->n_bands = (int *)calloc(S, sizeof(int));
  md->n_raw_bands = (int *)calloc(S, sizeof(int));
  allocate_double_array_3d(&md->Rrs_measured, R, S, B);
  allocate_double_array_3d(&md->Rrs_modelled, R, S, B);
  allocate_double_array_3d(&md->rrs_modelled, R, S, B);
  allocate_double_array_3d(&md->rrs_bottom, R, S, B);
  allocate_double_array_3d(&md->rrs_dp, R, S, B);
  allocate_double_array_3d(&md->rho, R, S, B);
  allocate_double_array_2d(&md->wavelengths, S, B);
  allocate_double_array_2d(&md->raw_wavelengths, S, B);
  allocate_double_array_2d(&md->a_0, S, B);
  allocate_double_array_2d(&md->a_1, S, B);
  allocate_double_array_2d(&md->a_w, S, B);
  allocate_double_array_2d(&md->b_bw, S, B);
  allocate_double_array_2d(&md->K, S, B);
  allocate_double_array_2d(&md->rrs_noise, S, B);
  allocate_double_array_3d(&md->bottom_reflectance, REF_N_BOTTOM_TABLE, S, B);
  allocate_double_array_2d(&md->Rrs440, R, S);
  allocate_double_array_2d(&md->Rrs490, R, S);
  allocate_double_array_2d(&md->Rrs550, R, S);
  allocate_double_array_2d(&md->Rrs640, R, S);
  allocate_double_array_2d(&md->Rrs750, R, S);
  md->theta_view = (double *)calloc(S, sizeof(double));
  md->theta_sun = (double *)calloc(S, sizeof(double));
  md->sec_theta_view = (double *)calloc(S, sizeof(double));
  md->sec_theta_sun = (double *)calloc(S, sizeof(double));
  md->H_tide = (double *)calloc(S, sizeof(double));
  md->P = (double *)calloc(S, sizeof(double));
  md->G = (double *)calloc(S, sizeof(double));
  md->X = (double *)calloc(S, sizeof(double));
  md->D = (double *)calloc(S, sizeof(double));
  md->prev = (double *)calloc(4 * S, sizeof(double));
  md->a_w640 = interp_1d(ref_wlens, aw_Pope_Fry1997, n_ref_wlens, 640.0); /* samodel.c:505 */
  return md;
}

static model_data *md_new(void) { return md_new_r(1); }

static void md_free(model_data *md) {
  int S = REF_MAX_SCENES, R = md->max_n_regions;
  free_double_array_3d(md->Rrs_measured, R, S);
  free_double_array_3d(md->Rrs_modelled, R, S);
  free_double_array_3d(md->rrs_modelled, R, S);
  free_double_array_3d(md->rrs_bottom, R, S);
  free_double_array_3d(md->rrs_dp, R, S);
  free_double_array_3d(md->rho, R, S);
  free_double_array_2d(md->wavelengths, S);
  free_double_array_2d(md->raw_wavelengths, S);
  free_double_array_2d(md->a_0, S);
  free_double_array_2d(md->a_1, S);
  free_double_array_2d(md->a_w, S);
  free_double_array_2d(md->b_bw, S);
  free_double_array_2d(md->K, S);
  free_double_array_2d(md->rrs_noise, S);
  free_double_array_3d(md->bottom_reflectance, REF_N_BOTTOM_TABLE, S);
  free_double_array_2d(md->Rrs440, R);
  free_double_array_2d(md->Rrs490, R);
  free_double_array_2d(md->Rrs550, R);
  free_double_array_2d(md->Rrs640, R);
  free_double_array_2d(md->Rrs750, R);
  free(md->n_bands); free(md->n_raw_bands);
  free(md->theta_view); free(md->theta_sun); free(md->sec_theta_view); free(md->sec_theta_sun);
  free(md->H_tide); free(md->P); free(md->G); free(md->X); free(md->D); free(md->prev);
  free(md);
}

/* Per-scene constants, following samodel() model/samodel.c:521-618. */
static void md_set_scene(model_data *md, int k_scene, int n_bands, const double *wl,
                         double theta_sun_deg, double theta_view_deg, double h_tide) {
  int k_band, k_bottom;
  md->n_bands[k_scene] = n_bands;
  md->n_raw_bands[k_scene] = n_bands;
  md->H_tide[k_scene] = h_tide;
  md->theta_view[k_scene] = theta_view_deg;
  md->theta_view[k_scene] *= PI / 180.0;
  md->sec_theta_view[k_scene] = 1.0 / cos(md->theta_view[k_scene]);
  md->theta_sun[k_scene] = theta_sun_deg;
  md->theta_sun[k_scene] *= PI / 180.0;
  md->sec_theta_sun[k_scene] = 1.0 / cos(md->theta_sun[k_scene]);
  for (k_band = 0; k_band < n_bands; k_band++) {
    double l = wl[k_band];
    md->wavelengths[k_scene][k_band] = l;
    md->raw_wavelengths[k_scene][k_band] = l;
    md->a_0[k_scene][k_band] = interp_1d(ref_wlens, a0_Lee, n_ref_wlens, l);
    md->a_1[k_scene][k_band] = interp_1d(ref_wlens, a1_Lee, n_ref_wlens, l);
    md->b_bw[k_scene][k_band] = interp_1d(ref_wlens, bbw_Morel_1974, n_ref_wlens, l);
    md->a_w[k_scene][k_band] = interp_1d(ref_wlens, aw_Pope_Fry1997, n_ref_wlens, l);
    md->rrs_noise[k_scene][k_band] = 0.0;
    for (k_bottom = 0; k_bottom < REF_N_BOTTOM_TABLE; k_bottom++)
      md->bottom_reflectance[k_bottom][k_scene][k_band] =
          interp_1d(ref_wlens, bottom_table(k_bottom), n_ref_wlens, l);
  }
}

static void md_reset_pixel(model_data *md, int n_scenes, int n_bands) {
  int s, b;
  md->n_scenes = n_scenes;
  md->max_n_bands = n_bands;
  md->n_regions = 1;
  md->origin = 0;
  md->n_bottoms = 1;
  md->bottom_type_indexes[0] = 0;
  md->empirical_depth_present = false;
  md->start_at_previous = false;
  md->h_empirical = 0.0;
  md->depth_prev = 0.0;
  for (s = 0; s < n_scenes; s++)
    for (b = 0; b < n_bands; b++) {
      md->Rrs_measured[0][s][b] = 0.0;
      md->Rrs_modelled[0][s][b] = 0.0;
      md->rrs_modelled[0][s][b] = 0.0;
      md->rrs_bottom[0][s][b] = 0.0;
      md->rrs_dp[0][s][b] = 0.0;
      md->rho[0][s][b] = 0.0;
    }
}

/* Mask test of model/samodel.c:937-941. */
static int pixel_masked(const float *rrs, int n, float nodata) {
  int b;
  for (b = 0; b < n; b++) {
    float refl = rrs[b];
    if (approx_equal(refl, nodata, 1.0e-6) || refl < 0.0) return 1;
  }
  return 0;
}

static void store_result(model_data *md, double *o, long long evals) {
  int s;
  o[0] = md->depth;
  o[1] = md->bottom_albedo;
  o[2] = md->model_error;
  o[3] = md->Rrs_error;
  o[4] = md->K_min;
  o[5] = md->index_optical_depth;
  o[6] = (double)md->n_iterations;
  o[7] = (double)evals;
  o[8] = md->converged ? 1.0 : 0.0;
  o[9] = 0.0;
  o[10] = (double)md->n_scenes;
  for (s = 0; s < md->n_scenes && s < REF_MAX_SCENES; s++) {
    o[11 + s] = md->P[s];
    o[19 + s] = md->G[s];
    o[27 + s] = md->X[s];
  }
}

static void set_tol(int use_override, double reqmin, int konvge, int kcount) {
  g_tol.active = use_override;
  g_tol.reqmin = reqmin;
  g_tol.konvge = konvge;
  g_tol.kcount = kcount;
  g_tol.evals = 0;
}

int photic_ref_nout(void) { return REF_NOUT; }

/* Single-scene batch: rrs is [npix][n_bands] float (the reference reads
 * float grids, model/common.h:81).  out is [npix][REF_NOUT]. */
int photic_ref_invert_batch(int n_bands, const double *wl, double theta_sun_deg,
                            double theta_view_deg, double h_tide, const float *rrs,
                            long long npix, float nodata, int use_override, double reqmin,
                            int konvge, int kcount, int nthreads, double *out) {
  if (n_bands < 2 || n_bands > REF_MAX_BANDS) return 1;
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    model_data *md = md_new();
    long long p;
    md_set_scene(md, 0, n_bands, wl, theta_sun_deg, theta_view_deg, h_tide);
#if _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
    for (p = 0; p < npix; p++) {
      const float *r = rrs + p * n_bands;
      double *o = out + p * REF_NOUT;
      int b;
      memset(o, 0, REF_NOUT * sizeof(double));
      if (pixel_masked(r, n_bands, nodata)) {
        o[9] = 1.0;
        continue;
      }
      md_reset_pixel(md, 1, n_bands);
      for (b = 0; b < n_bands; b++) md->Rrs_measured[0][0][b] = r[b];
      set_tol(use_override, reqmin, konvge, kcount);
      samodel_optimise(md);
      store_result(md, o, g_tol.evals);
    }
    md_free(md);
  }
  return 0;
}

/* Temporal joint fit: pixel p owns observations scene_offsets[p] ..
 * scene_offsets[p+1]-1; each observation is one scene with its own
 * subsurface sun zenith.  rrs is [n_obs][n_bands]. */
int photic_ref_joint_invert_batch(int n_bands, const double *wl, double theta_view_deg,
                                  double h_tide, const int *scene_offsets,
                                  const double *theta_sun_deg, const float *rrs, long long npix,
                                  float nodata, int use_override, double reqmin, int konvge,
                                  int kcount, int nthreads, double *out) {
  if (n_bands < 2 || n_bands > REF_MAX_BANDS) return 1;
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    model_data *md = md_new();
    long long p;
#if _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (p = 0; p < npix; p++) {
      int o0 = scene_offsets[p], k = scene_offsets[p + 1] - scene_offsets[p];
      double *o = out + p * REF_NOUT;
      int s, b, masked = 0;
      memset(o, 0, REF_NOUT * sizeof(double));
      if (k < 1 || k > REF_MAX_SCENES) {
        o[9] = 2.0;
        continue;
      }
      for (s = 0; s < k; s++) masked |= pixel_masked(rrs + (size_t)(o0 + s) * n_bands, n_bands, nodata);
      if (masked) {
        o[9] = 1.0;
        continue;
      }
      md_reset_pixel(md, k, n_bands);
      for (s = 0; s < k; s++) {
        md_set_scene(md, s, n_bands, wl, theta_sun_deg[o0 + s], theta_view_deg, h_tide);
        for (b = 0; b < n_bands; b++)
          md->Rrs_measured[0][s][b] = rrs[(size_t)(o0 + s) * n_bands + b];
      }
      set_tol(use_override, reqmin, konvge, kcount);
      samodel_optimise(md);
      store_result(md, o, g_tol.evals);
    }
    md_free(md);
  }
  return 0;
}

/* The general fit of samodel()'s pixel loop through the reference's own
 * extract_Rrs_data and samodel_optimise: each pixel alone (n_spatial = 1)
 * or with its 3 x 3 neighbourhood (n_spatial = 2: edges clamped, neighbours
 * with nodata left out; model/samodel.c:2957-3027), over n_scenes scenes of
 * the same bands (sun zenith theta_sun_deg[s]), with n_bottoms bottom types
 * (the first entries of the bottom table, all at once as ALL_BOTTOMS
 * selects, model/samodel.c:1822-1858), smoothing radius 1.  grid is
 * [n_scenes][nrows][ncols][n_bands] float; h_empirical (NULL, or [npix]
 * with NaN for none) gives a pixel's empirical depth as samodel() sets it
 * (model/samodel.c:958-967).  out is [npix][REF_NOUT] with o[38] = regions,
 * o[39] = origin region, o[40..42] = B_type_percent of sand, seagrass and
 * coral, o[43] = bottom_type. */
int photic_ref_region_fit_batch(int n_bands, const double *wl, const double *theta_sun_deg,
                                double theta_view_deg, double h_tide, const float *grid,
                                int n_scenes, int nrows, int ncols, float nodata, int n_spatial,
                                int n_bottoms, const double *h_empirical, int use_override,
                                double reqmin, int konvge, int kcount, int nthreads,
                                double *out) {
  geogrid *gd;
  scene *sc;
  int b, s, R, scene_indexes[REF_MAX_SCENES];
  const long long npix = (long long)nrows * ncols;
  if (n_bands < 2 || n_bands > REF_MAX_BANDS || n_spatial < 1 || n_spatial > 2 ||
      n_bottoms < 1 || n_bottoms > 3 || n_scenes < 1 || n_scenes > REF_MAX_SCENES)
    return 1;
  R = (2 * n_spatial - 1) * (2 * n_spatial - 1);
  gd = (geogrid *)calloc((size_t)n_scenes * n_bands, sizeof(geogrid));
  sc = (scene *)calloc(n_scenes, sizeof(scene));
  for (s = 0; s < n_scenes; s++) {
    scene_indexes[s] = s;
    sc[s].n_bands = n_bands;
    sc[s].nrows = nrows;
    sc[s].ncols = ncols;
    for (b = 0; b < n_bands; b++) {
      geogrid *g = &gd[s * n_bands + b];
      int i, j;
      sc[s].band_indexes[b] = s * n_bands + b;
      g->nrows = nrows;
      g->ncols = ncols;
      g->nodata_value = nodata;
      allocate_float_array_2d(&g->array, nrows, ncols);
      for (i = 0; i < nrows; i++)
        for (j = 0; j < ncols; j++)
          g->array[i][j] = grid[(((size_t)s * nrows + i) * ncols + j) * n_bands + b];
    }
  }
#if _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    model_data *md = md_new_r(R);
    long long p;
    int ks;
    for (ks = 0; ks < n_scenes; ks++)
      md_set_scene(md, ks, n_bands, wl, theta_sun_deg[ks], theta_view_deg, h_tide);
#if _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (p = 0; p < npix; p++) {
      int i = (int)(p / ncols), j = (int)(p % ncols), r, ss, bb, bad = 0;
      double *o = out + p * REF_NOUT;
      memset(o, 0, REF_NOUT * sizeof(double));
      for (ss = 0; ss < n_scenes && !bad; ss++) /* model/samodel.c:933-947 */
        bad = pixel_masked(grid + ((size_t)ss * npix + p) * n_bands, n_bands, nodata);
      if (bad) {
        o[9] = 1.0;
        continue;
      }
      md_reset_pixel(md, n_scenes, n_bands);
      for (r = 0; r < R; r++) /* the loop's defaults, model/samodel.c:917-928 */
        for (ss = 0; ss < n_scenes; ss++)
          for (bb = 0; bb < n_bands; bb++) {
            md->Rrs_measured[r][ss][bb] = 0.0;
            md->Rrs_modelled[r][ss][bb] = 0.0;
            md->rrs_modelled[r][ss][bb] = 0.0;
            md->rrs_bottom[r][ss][bb] = 0.0;
            md->rrs_dp[r][ss][bb] = 0.0;
            md->rho[r][ss][bb] = 0.0;
          }
      md->n_bottoms = n_bottoms;
      if (h_empirical && !isnan(h_empirical[p])) {
        md->empirical_depth_present = true;
        md->h_empirical = h_empirical[p];
      }
      extract_Rrs_data(i, j, sc, gd, scene_indexes, n_scenes, n_spatial, 1, nrows, ncols, md,
                       0.0);
      if (md->n_regions == 0) continue;
      set_tol(use_override, reqmin, konvge, kcount);
      samodel_optimise(md);
      store_result(md, o, g_tol.evals);
      o[38] = (double)md->n_regions;
      o[39] = (double)md->origin;
      for (bb = 0; bb < 3; bb++) o[40 + bb] = md->B_type_percent[bb];
      o[43] = md->bottom_type;
    }
    md_free(md);
  }
  for (b = 0; b < n_scenes * n_bands; b++) free_float_array_2d(gd[b].array, nrows);
  free(gd);
  free(sc);
  return 0;
}

int photic_ref_region_invert_batch(int n_bands, const double *wl, double theta_sun_deg,
                                   double theta_view_deg, double h_tide, const float *grid,
                                   int nrows, int ncols, float nodata, int n_spatial,
                                   int use_override, double reqmin, int konvge, int kcount,
                                   int nthreads, double *out) {
  return photic_ref_region_fit_batch(n_bands, wl, &theta_sun_deg, theta_view_deg, h_tide, grid,
                                     1, nrows, ncols, nodata, n_spatial, 1, NULL, use_override,
                                     reqmin, konvge, kcount, nthreads, out);
}

/* Forward model + cost at given parameters, through samodel_error
 * (model/samodel.c:2432).  Rrs440/490/550/640/750 are interpolated from the
 * measured spectrum as samodel_optimise does (model/samodel.c:1785-1799).
 * Outputs: cost, Rrs_modelled[n_bands], K[n_bands]. */
double photic_ref_cost(int n_bands, const double *wl, double theta_sun_deg,
                       double theta_view_deg, double h_tide, const double *rrs_measured,
                       const double *params, int n_params, double *rrs_modelled, double *K_out) {
  model_data *md = md_new();
  double cost, prm[64];
  int b;
  (void)n_params;
  md_set_scene(md, 0, n_bands, wl, theta_sun_deg, theta_view_deg, h_tide);
  md_reset_pixel(md, 1, n_bands);
  for (b = 0; b < n_bands; b++) md->Rrs_measured[0][0][b] = rrs_measured[b];
  md->Rrs440[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 440.0);
  md->Rrs490[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 490.0);
  md->Rrs550[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 550.0);
  md->Rrs640[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 640.0);
  md->Rrs750[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 750.0);
  if (md->Rrs440[0][0] < 0.0) md->Rrs440[0][0] = 0.0001;
  md->n_params = 6;
  memcpy(prm, params, 6 * sizeof(double));
  cost = samodel_error(prm, md);
  for (b = 0; b < n_bands; b++) {
    rrs_modelled[b] = md->Rrs_modelled[0][0][b];
    K_out[b] = md->K[0][b];
  }
  md_free(md);
  return cost;
}

/* The reference's interp_1d (model/common.c:298), exported for the table
 * interpolation tests. */
double photic_ref_interp_1d(const double *X, const double *Y, int n, double x) {
  return interp_1d((double *)X, (double *)Y, n, x);
}

/* Band constants as samodel() computes them (model/samodel.c:521-618):
 * out[b*8 + 0..7] = a_0, a_1, a_w, b_bw, sand reflectance, sec_sun, sec_view, a_w640. */
void photic_ref_band_constants(int n_bands, const double *wl, double theta_sun_deg,
                               double theta_view_deg, double *out) {
  model_data *md = md_new();
  int b;
  md_set_scene(md, 0, n_bands, wl, theta_sun_deg, theta_view_deg, 0.0);
  for (b = 0; b < n_bands; b++) {
    out[b * 8 + 0] = md->a_0[0][b];
    out[b * 8 + 1] = md->a_1[0][b];
    out[b * 8 + 2] = md->a_w[0][b];
    out[b * 8 + 3] = md->b_bw[0][b];
    out[b * 8 + 4] = md->bottom_reflectance[0][0][b];
    out[b * 8 + 5] = md->sec_theta_sun[0];
    out[b * 8 + 6] = md->sec_theta_view[0];
    out[b * 8 + 7] = md->a_w640;
  }
  md_free(md);
}

/* Direct call of the reference nelmin (model/asa047.c:10) on samodel_error
 * with an explicit start/step and tolerances; for trajectory-level tests. */
void photic_ref_nelmin(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                       const double *rrs_measured, const double *start_in, const double *step_in,
                       double reqmin, int konvge, int kcount, double *xmin, double *ynewlo,
                       int *icount, int *numres, int *ifault) {
  model_data *md = md_new();
  double start[64], step[64];
  int b;
  md_set_scene(md, 0, n_bands, wl, theta_sun_deg, theta_view_deg, 0.0);
  md_reset_pixel(md, 1, n_bands);
  for (b = 0; b < n_bands; b++) md->Rrs_measured[0][0][b] = rrs_measured[b];
  md->Rrs440[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 440.0);
  md->Rrs490[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 490.0);
  md->Rrs750[0][0] = interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], n_bands, 750.0);
  if (md->Rrs440[0][0] < 0.0) md->Rrs440[0][0] = 0.0001;
  md->n_params = 6;
  memcpy(start, start_in, 6 * sizeof(double));
  memcpy(step, step_in, 6 * sizeof(double));
  nelmin(samodel_error, md, 6, start, xmin, ynewlo, reqmin, step, konvge, kcount, icount, numres,
         ifault);
  md_free(md);
}

/* The reference's own interval statistic of the depth uncertainty
 * (model/samodel.c:1459-1460): vec_mean2_double then vec_stddev_double
 * (model/common.c:877-940) with spval 0 over one interval's refitted sample
 * depths. */
double photic_ref_depth_sigma_stat(double *depths, int n) {
  double mean_trial_depths = vec_mean2_double(depths, n, 0.0);
  return vec_stddev_double(depths, n, 0.0, mean_trial_depths);
}

/* The reference's own product path: samodel() (model/samodel.c:289-1763)
 * over one scene's [nrows][ncols][n_bands] float grid with its compiled-in
 * dynamic LUT, spectral ordering and hot starts (LUT 1, model/samodel.c:97),
 * run on one thread so that its order-dependent results are reproducible,
 * at the reference's own tolerances.  r_sigma (n_bands values or NULL for
 * zeros) is the scene's noise spectrum, which orders the pixels when every
 * band's is at least 1e-6 (:590-600, :749-767); empirical (NULL or
 * [nrows][ncols] floats, empirical_nodata for none) is an empirical depth
 * grid, which then orders the pixels and starts their fits (:702-710,
 * 955-979).  grids_out receives the ten
 * result grids [10][nrows][ncols] exactly as samodel() leaves them: depth
 * (negative below the datum), depth sigma, model error, bottom albedo,
 * sand, seagrass, coral, K_min, bottom type, index of optical depth.  Its
 * depth-uncertainty pass and result files run as well (the netCDF stand-in
 * keeps the files in memory). */
/* samodel() over n_scenes co-registered scenes of the same bands:
 * grid [n_scenes][nrows][ncols][n_bands], theta_sun_deg and r_sigma per
 * scene ([n_scenes], [n_scenes][n_bands] or NULL); one thread. */
int photic_ref_samodel_stack(int n_bands, const double *wl, const double *theta_sun_deg,
                             double theta_view_deg, const float *grid, int n_scenes, int nrows,
                             int ncols, float nodata, const double *r_sigma,
                             const float *empirical, float empirical_nodata, int n_spatial,
                             int n_bottoms, float *grids_out) {
  scene *sc;
  geogrid *gd, none;
  float **out[10];
  int b, i, j, k, s, *idx;
  const size_t npix = (size_t)nrows * ncols;
  if (n_bands < 2 || n_bands > REF_MAX_BANDS || n_scenes < 1) return 1;
  sc = (scene *)calloc(n_scenes, sizeof(scene));
  idx = (int *)calloc(n_scenes, sizeof(int));
  memset(&none, 0, sizeof none);
  if (empirical) { /* an empirical depth grid (model/samodel.c:702-710, 955-979) */
    none.nrows = nrows;
    none.ncols = ncols;
    none.cellsize = 1.0f;
    none.nodata_value = empirical_nodata;
    allocate_float_array_2d(&none.array, nrows, ncols);
    for (i = 0; i < nrows; i++)
      for (j = 0; j < ncols; j++) none.array[i][j] = empirical[(size_t)i * ncols + j];
  }
  gd = (geogrid *)calloc((size_t)n_scenes * n_bands, sizeof(geogrid));
  for (s = 0; s < n_scenes; s++) {
    idx[s] = s;
    snprintf(sc[s].scene_name, sizeof sc[s].scene_name, "harness%d", s);
    sc[s].n_bands = n_bands;
    sc[s].nrows = nrows;
    sc[s].ncols = ncols;
    sc[s].theta_w = theta_sun_deg[s];
    sc[s].theta_v = theta_view_deg;
    for (b = 0; b < n_bands; b++) {
      geogrid *g = gd + s * n_bands + b;
      sc[s].band_indexes[b] = s * n_bands + b;
      sc[s].wavelengths[b] = (int)wl[b];
      sc[s].R_sigma[b] = r_sigma ? r_sigma[s * n_bands + b] : 0.0;
      g->nrows = nrows;
      g->ncols = ncols;
      g->cellsize = 1.0f;
      g->nodata_value = nodata;
      allocate_float_array_2d(&g->array, nrows, ncols);
      for (i = 0; i < nrows; i++)
        for (j = 0; j < ncols; j++)
          g->array[i][j] = grid[(s * npix + (size_t)i * ncols + j) * n_bands + b];
    }
  }
  for (k = 0; k < 10; k++) allocate_float_array_2d(&out[k], nrows, ncols);
  set_tol(0, 0.0, 0, 0);
#if _OPENMP
  omp_set_num_threads(1);
#endif
  samodel(sc, gd, idx, n_scenes, empirical != NULL, none, 1, n_spatial, n_bottoms, out[0],
          out[1], out[2], out[3], out[4], out[5], out[6], out[7], out[8], out[9], 10.0f, 0, 1);
  for (k = 0; k < 10; k++)
    for (i = 0; i < nrows; i++)
      for (j = 0; j < ncols; j++)
        grids_out[((size_t)k * nrows + i) * ncols + j] = out[k][i][j];
  if (empirical) free_float_array_2d(none.array, nrows);
  for (k = 0; k < 10; k++) free_float_array_2d(out[k], nrows);
  for (b = 0; b < n_scenes * n_bands; b++) free_float_array_2d(gd[b].array, nrows);
  free(gd);
  free(sc);
  free(idx);
  return 0;
}

/* samodel() over one scene (photic_ref_samodel_stack with n_scenes = 1). */
int photic_ref_samodel_grid(int n_bands, const double *wl, double theta_sun_deg,
                            double theta_view_deg, const float *grid, int nrows, int ncols,
                            float nodata, const double *r_sigma, const float *empirical,
                            float empirical_nodata, int n_spatial, int n_bottoms,
                            float *grids_out) {
  return photic_ref_samodel_stack(n_bands, wl, &theta_sun_deg, theta_view_deg, grid, 1, nrows,
                                  ncols, nodata, r_sigma, empirical, empirical_nodata, n_spatial,
                                  n_bottoms, grids_out);
}
