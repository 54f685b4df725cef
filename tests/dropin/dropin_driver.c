/* A C program written against the link-compatible samodel entry points of
 * include/photic_samodel.h, as a program of the reference would call them:
 * it fills a model_data the way the reference's samodel() prepares one
 * (model/samodel.c:402-618) and calls samodel_optimise / samodel_error /
 * samodel_Rrs per pixel, or samodel() over a gridded scene.  The GPU tests
 * compile it, run it and compare what it prints with the oracle.
 *
 * usage: dropin_driver MODE IN OUT
 *   IN  = int32 n_bands, int32 npix, int32 nrows, int32 ncols,
 *         double wavelengths[n_bands], theta_sun_deg, theta_view_deg,
 *         float rrs[npix][n_bands], double params[npix][6]
 *   MODE optimise : OUT = double [npix][18]: depth_prev and prev[0..2] as
 *                   they stood before the call, then depth, P, G, X, bottom
 *                   albedo, model error, Rrs error, K_min, IOD, n_iterations,
 *                   converged, Rrs440, B_type_percent[0], bottom_type
 *        prev     : as optimise, but each pixel after the first starts at
 *                   the previous pixel's optimum (start_at_previous)
 *        combo    : samodel_optimise_one_bottom_combination; OUT = double
 *                   [npix][8] (|best| H, 100 B, q, 100 P, 100 G, 100 X,
 *                   n_iterations, converged)
 *        error    : OUT = double [npix][1 + n_bands] (cost, Rrs_modelled)
 *        rrs      : OUT = double [npix][2 * n_bands] (Rrs_modelled, K) at
 *                   the model inputs samodel_error derives from params
 *        grid     : samodel() over an nrows x ncols grid (grid2: with
 *                   n_spatial = 2, 3 x 3 regions per pixel; grid3: 3 x 3
 *                   regions and n_bottoms = 3, the reference's default call;
 *                   grid13: pixels alone, n_bottoms = 3; gride: pixels
 *                   alone with the empirical depth grid taken from params[0]
 *                   as float, nodata -9999); OUT = float
 *                   [10][nrows][ncols] (depth, depth sigma, model error,
 *                   albedo, sand, seagrass, coral, K_min, type, IOD)
 *        optimise3: samodel_optimise with n_bottoms = 3 (sand, seagrass,
 *                   coral); OUT = double [npix][15]: depth, P, G, X, albedo,
 *                   model error, Rrs error, K_min, IOD, n_iterations,
 *                   converged, the three bottom shares, bottom type
 *        error3   : samodel_error with n_bottoms = 3 at the 10-vector
 *                   (H, 100B, 70B, 130B, q, q/2, q/4, 100P, 100G, 100X) made
 *                   from each 6-vector; OUT = double [npix][1 + n_bands] */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "photic_samodel.h"

static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n, s);
  if (!p) {
    fprintf(stderr, "out of memory\n");
    exit(2);
  }
  return p;
}

static double **mat2(int a, int b) {
  double **m = xcalloc((size_t)a, sizeof *m);
  for (int i = 0; i < a; i++) m[i] = xcalloc((size_t)b, sizeof **m);
  return m;
}

static double ***mat3(int a, int b, int c) {
  double ***m = xcalloc((size_t)a, sizeof *m);
  for (int i = 0; i < a; i++) m[i] = mat2(b, c);
  return m;
}

static float **fgrid(int r, int c) {
  float **g = xcalloc((size_t)r, sizeof *g);
  for (int i = 0; i < r; i++) g[i] = xcalloc((size_t)c, sizeof **g);
  return g;
}

/* One region, one scene, sand bottom: the model_data of a single-scene
 * pixel, band constants from photic_band_constants. */
static photic_model_data *md_new(int nb, const double *wl, double th_sun, double th_view) {
  photic_config cfg;
  photic_config_default(&cfg);
  cfg.n_bands = nb;
  for (int b = 0; b < nb; b++) cfg.wavelengths[b] = wl[b];
  cfg.theta_sun_deg = th_sun;
  cfg.theta_view_deg = th_view;
  double bc[PHOTIC_MAX_BANDS * 8];
  if (photic_band_constants(&cfg, bc)) {
    fprintf(stderr, "band constants: %s\n", photic_last_error());
    exit(3);
  }
  photic_model_data *md = xcalloc(1, sizeof *md);
  md->n_bottoms = 1;
  md->n_scenes = 1;
  md->n_regions = 1;
  double refl[3 * PHOTIC_MAX_BANDS];
  if (photic_bottom_reflectances(&cfg, 3, refl)) {
    fprintf(stderr, "bottom reflectances: %s\n", photic_last_error());
    exit(3);
  }
  md->max_n_bands = nb;
  md->max_n_regions = 1;
  md->n_bands = xcalloc(1, sizeof(int));
  md->n_bands[0] = nb;
  md->Rrs_measured = mat3(1, 1, nb);
  md->wavelengths = mat2(1, nb);
  md->bottom_reflectance = mat3(3, 1, nb);
  md->a_0 = mat2(1, nb);
  md->a_1 = mat2(1, nb);
  md->a_w = mat2(1, nb);
  md->b_bw = mat2(1, nb);
  for (int b = 0; b < nb; b++) {
    md->wavelengths[0][b] = wl[b];
    md->a_0[0][b] = bc[b * 8 + 0];
    md->a_1[0][b] = bc[b * 8 + 1];
    md->a_w[0][b] = bc[b * 8 + 2];
    md->b_bw[0][b] = bc[b * 8 + 3];
    for (int k = 0; k < 3; k++) md->bottom_reflectance[k][0][b] = refl[k * nb + b];
  }
  md->a_w640 = bc[7];
  md->H_tide = xcalloc(1, sizeof(double));
  md->theta_sun = xcalloc(1, sizeof(double));
  md->theta_view = xcalloc(1, sizeof(double));
  md->sec_theta_sun = xcalloc(1, sizeof(double));
  md->sec_theta_view = xcalloc(1, sizeof(double));
  md->theta_sun[0] = th_sun * (3.141592653589793 / 180.0);
  md->theta_view[0] = th_view * (3.141592653589793 / 180.0);
  md->sec_theta_sun[0] = bc[5];
  md->sec_theta_view[0] = bc[6];
  md->Rrs440 = mat2(1, 1);
  md->Rrs490 = mat2(1, 1);
  md->Rrs550 = mat2(1, 1);
  md->Rrs640 = mat2(1, 1);
  md->Rrs750 = mat2(1, 1);
  md->rrs_noise = mat2(1, nb);
  for (int k = 0; k < 3; k++) md->bottom_type_indexes[k] = k;
  strcpy(md->B_type_name[0], "sand");
  strcpy(md->B_type_name[1], "seagrass");
  strcpy(md->B_type_name[2], "coral");
  md->P = xcalloc(1, sizeof(double));
  md->G = xcalloc(1, sizeof(double));
  md->X = xcalloc(1, sizeof(double));
  md->B = xcalloc(1, sizeof(double));
  md->H = xcalloc(1, sizeof(double));
  md->D = xcalloc(1, sizeof(double));
  md->prev = xcalloc(4, sizeof(double));
  md->Rrs_modelled = mat3(1, 1, nb);
  md->rrs_modelled = mat3(1, 1, nb);
  md->rrs_bottom = mat3(1, 1, nb);
  md->rrs_dp = mat3(1, 1, nb);
  md->K = mat2(1, nb);
  md->rho = mat3(1, 1, nb);
  return md;
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s MODE IN OUT\n", argv[0]);
    return 1;
  }
  const char *mode = argv[1];
  FILE *f = fopen(argv[2], "rb");
  if (!f) return 1;
  int32_t hdr[4];
  if (fread(hdr, sizeof hdr, 1, f) != 1) return 1;
  const int nb = hdr[0], npix = hdr[1], nrows = hdr[2], ncols = hdr[3];
  double wl[PHOTIC_MAX_BANDS], th[2];
  if (nb < 2 || nb > PHOTIC_MAX_BANDS || npix < 1) return 1;
  if (fread(wl, sizeof(double), (size_t)nb, f) != (size_t)nb) return 1;
  if (fread(th, sizeof(double), 2, f) != 2) return 1;
  float *rrs = xcalloc((size_t)npix * nb, sizeof(float));
  double *params = xcalloc((size_t)npix * 6, sizeof(double));
  if (fread(rrs, sizeof(float), (size_t)npix * nb, f) != (size_t)npix * nb) return 1;
  if (fread(params, sizeof(double), (size_t)npix * 6, f) != (size_t)npix * 6) return 1;
  fclose(f);
  FILE *o = fopen(argv[3], "wb");
  if (!o) return 1;

  if (!strcmp(mode, "grid") || !strcmp(mode, "grid2") || !strcmp(mode, "grid3") ||
      !strcmp(mode, "grid13") || !strcmp(mode, "gride")) {
    const int n_spatial = (!strcmp(mode, "grid2") || !strcmp(mode, "grid3")) ? 2 : 0;
    const int n_bottoms = (!strcmp(mode, "grid3") || !strcmp(mode, "grid13")) ? 3 : 1;
    if (nrows * ncols != npix) return 1;
    photic_scene *sc = xcalloc(1, sizeof *sc);
    photic_geogrid *grids = xcalloc((size_t)nb, sizeof *grids);
    strcpy(sc->scene_name, "synthetic");
    sc->n_bands = nb;
    sc->nrows = nrows;
    sc->ncols = ncols;
    sc->theta_w = th[0];
    sc->theta_v = th[1];
    for (int b = 0; b < nb; b++) {
      sc->band_indexes[b] = b;
      sc->wavelengths[b] = (int)wl[b];
      grids[b].nrows = nrows;
      grids[b].ncols = ncols;
      grids[b].nodata_value = -9999.0f;
      grids[b].array = fgrid(nrows, ncols);
      for (int i = 0; i < nrows; i++)
        for (int j = 0; j < ncols; j++) grids[b].array[i][j] = rrs[((size_t)i * ncols + j) * nb + b];
    }
    photic_geogrid none;
    memset(&none, 0, sizeof none);
    const int emp = !strcmp(mode, "gride");
    if (emp) {
      none.nrows = nrows;
      none.ncols = ncols;
      none.nodata_value = -9999.0f;
      none.array = fgrid(nrows, ncols);
      for (int i = 0; i < nrows; i++)
        for (int j = 0; j < ncols; j++) none.array[i][j] = (float)params[((size_t)i * ncols + j) * 6];
    }
    float **g[10];
    for (int k = 0; k < 10; k++) g[k] = fgrid(nrows, ncols);
    int idx = 0;
    samodel(sc, grids, &idx, 1, emp, none, 1, n_spatial, n_bottoms, g[0], g[1], g[2], g[3], g[4],
            g[5], g[6], g[7], g[8], g[9], 0.0f, 0, 0);
    if (photic_last_error()[0]) {
      fprintf(stderr, "samodel: %s\n", photic_last_error());
      return 4;
    }
    for (int k = 0; k < 10; k++)
      for (int i = 0; i < nrows; i++) fwrite(g[k][i], sizeof(float), (size_t)ncols, o);
    fclose(o);
    return 0;
  }

  int xs = 0, xb = 0, xS = 0, xe = 0;
  if (sscanf(mode, "gridx:%d:%d:%d:%d", &xs, &xb, &xS, &xe) == 4) {
    /* a stack of xS scenes ([scene][row][col][band] in rrs), n_spatial xs,
     * n_bottoms xb; scene s's sun zenith in params[s * 6 + 1] and its R_sigma
     * in params[s * 6 + 2 ..] (four bands); with xe, the empirical depths in
     * params[p * 6] (nodata 9999) */
    const int np1 = nrows * ncols;
    if (xS < 1 || np1 * xS != npix || nb > 4) return 1;
    photic_scene *sc = xcalloc((size_t)xS, sizeof *sc);
    photic_geogrid *grids = xcalloc((size_t)xS * nb, sizeof *grids);
    int *idx = xcalloc((size_t)xS, sizeof(int));
    for (int k = 0; k < xS; k++) {
      idx[k] = k;
      snprintf(sc[k].scene_name, sizeof sc[k].scene_name, "synthetic%d", k);
      sc[k].n_bands = nb;
      sc[k].nrows = nrows;
      sc[k].ncols = ncols;
      sc[k].theta_w = params[k * 6 + 1];
      sc[k].theta_v = th[1];
      for (int b = 0; b < nb; b++) {
        photic_geogrid *gr = grids + k * nb + b;
        sc[k].band_indexes[b] = k * nb + b;
        sc[k].wavelengths[b] = (int)wl[b];
        sc[k].R_sigma[b] = params[k * 6 + 2 + b];
        gr->nrows = nrows;
        gr->ncols = ncols;
        gr->nodata_value = -9999.0f;
        gr->array = fgrid(nrows, ncols);
        for (int i = 0; i < nrows; i++)
          for (int j = 0; j < ncols; j++)
            gr->array[i][j] = rrs[(((size_t)k * nrows + i) * ncols + j) * nb + b];
      }
    }
    photic_geogrid none;
    memset(&none, 0, sizeof none);
    if (xe) {
      none.nrows = nrows;
      none.ncols = ncols;
      none.nodata_value = 9999.0f;
      none.array = fgrid(nrows, ncols);
      for (int i = 0; i < nrows; i++)
        for (int j = 0; j < ncols; j++) none.array[i][j] = (float)params[((size_t)i * ncols + j) * 6];
    }
    float **g[10];
    for (int k = 0; k < 10; k++) g[k] = fgrid(nrows, ncols);
    samodel(sc, grids, idx, xS, xe, none, 1, xs, xb, g[0], g[1], g[2], g[3], g[4], g[5], g[6],
            g[7], g[8], g[9], 0.0f, 0, 0);
    if (photic_last_error()[0]) {
      fprintf(stderr, "samodel: %s\n", photic_last_error());
      return 4;
    }
    for (int k = 0; k < 10; k++)
      for (int i = 0; i < nrows; i++) fwrite(g[k][i], sizeof(float), (size_t)ncols, o);
    fclose(o);
    return 0;
  }

  photic_model_data *md = md_new(nb, wl, th[0], th[1]);
  for (int p = 0; p < npix; p++) {
    for (int b = 0; b < nb; b++) md->Rrs_measured[0][0][b] = rrs[(size_t)p * nb + b];
    if (!strcmp(mode, "optimise") || !strcmp(mode, "prev")) {
      md->start_at_previous = !strcmp(mode, "prev") && p > 0;
      const double used[4] = {md->depth_prev, md->prev[0], md->prev[1], md->prev[2]};
      samodel_optimise(md);
      fwrite(used, sizeof used, 1, o);
      const double row[14] = {md->depth,       md->P[0],         md->G[0],
                              md->X[0],        md->bottom_albedo, md->model_error,
                              md->Rrs_error,   md->K_min,        md->index_optical_depth,
                              md->n_iterations, md->converged,   md->Rrs440[0][0],
                              md->B_type_percent[0], md->bottom_type};
      fwrite(row, sizeof row, 1, o);
      md->depth_prev = md->depth;
    } else if (!strcmp(mode, "optimise3")) {
      md->n_bottoms = 3;
      samodel_optimise(md);
      const double row[15] = {md->depth,         md->P[0],          md->G[0],
                              md->X[0],          md->bottom_albedo, md->model_error,
                              md->Rrs_error,     md->K_min,         md->index_optical_depth,
                              md->n_iterations,  md->converged,     md->B_type_percent[0],
                              md->B_type_percent[1], md->B_type_percent[2], md->bottom_type};
      fwrite(row, sizeof row, 1, o);
    } else if (!strcmp(mode, "error3")) {
      const double *x6 = params + (size_t)p * 6;
      double x[10] = {x6[0], x6[1], 0.7 * x6[1], 1.3 * x6[1], x6[2], 0.5 * x6[2],
                      0.25 * x6[2], x6[3], x6[4], x6[5]};
      md->n_bottoms = 3;
      double row[1 + PHOTIC_MAX_BANDS];
      row[0] = samodel_error(x, md);
      for (int b = 0; b < nb; b++) row[1 + b] = md->Rrs_modelled[0][0][b];
      fwrite(row, sizeof(double), (size_t)(1 + nb), o);
    } else if (!strcmp(mode, "combo")) {
      double x[8];
      samodel_optimise_one_bottom_combination(md, x);
      x[6] = md->n_iterations;
      x[7] = md->converged;
      fwrite(x, sizeof x, 1, o);
    } else if (!strcmp(mode, "error")) {
      double x[6];
      memcpy(x, params + (size_t)p * 6, sizeof x);
      double row[1 + PHOTIC_MAX_BANDS];
      row[0] = samodel_error(x, md);
      for (int b = 0; b < nb; b++) row[1 + b] = md->Rrs_modelled[0][0][b];
      fwrite(row, sizeof(double), (size_t)(1 + nb), o);
    } else if (!strcmp(mode, "rrs")) {
      /* the model inputs samodel_error derives from a parameter vector
       * (model/samodel.c:2470-2497) */
      const double *x = params + (size_t)p * 6;
      double B[1] = {0.01 * fabs(x[1])}, q[1] = {fabs(x[2])}, row[2 * PHOTIC_MAX_BANDS];
      q[0] /= q[0];
      /* samodel_Rrs reads the shape inputs the optimiser stores */
      md->Rrs440[0][0] = photic_interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], nb, 440.0);
      if (md->Rrs440[0][0] < 0.0) md->Rrs440[0][0] = 0.0001;
      md->Rrs490[0][0] = photic_interp_1d(md->wavelengths[0], md->Rrs_measured[0][0], nb, 490.0);
      for (int b = 0; b < nb; b++) {
        samodel_Rrs(0.01 * fabs(x[3]), 0.01 * fabs(x[4]), 0.01 * fabs(x[5]), B, q, fabs(x[0]),
                    0.0, md, 0, b, 0);
        row[b] = md->Rrs_modelled[0][0][b];
        row[nb + b] = md->K[0][b];
      }
      fwrite(row, sizeof(double), (size_t)(2 * nb), o);
    } else {
      return 1;
    }
    if (photic_last_error()[0]) {
      fprintf(stderr, "%s pixel %d: %s\n", mode, p, photic_last_error());
      return 4;
    }
  }
  fclose(o);
  return 0;
}
