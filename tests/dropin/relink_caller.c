/* The call photic's run_model_lee_semi_analytical makes (model/bam.c:
 * 3236-3241), compiled against the reference's own headers (model/common.h,
 * model/samodel.h) and linked with the reference's other objects and
 * libphotic_gb300 in place of model/samodel.c.  bam.c itself does not
 * compile as the reference ships it (EXIT is used at model/bam.c:287 and
 * declared nowhere), so this file stands in for its one call into the
 * inversion.  The link test only links it; run with an argument it inverts
 * a 4 x 4 grid of one synthetic spectrum. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "samodel.h"

static float **grid(int nrows, int ncols, float v) {
  float **g = malloc(sizeof *g * (size_t)nrows);
  for (int r = 0; r < nrows; r++) {
    g[r] = malloc(sizeof **g * (size_t)ncols);
    for (int c = 0; c < ncols; c++) g[r][c] = v;
  }
  return g;
}

int main(int argc, char **argv) {
  if (argc < 2) return 0; /* linked, not run, by the CPU test */
  const int nrows = 4, ncols = 4, nb = 4;
  const int wl[4] = {443, 482, 561, 655};
  const float rrs[4] = {0.0112f, 0.0125f, 0.0098f, 0.0021f};
  int ps_in[1] = {0};
  memset(&scene_data[0], 0, sizeof scene_data[0]);
  strcpy(scene_data[0].scene_name, "relink");
  scene_data[0].n_bands = nb;
  scene_data[0].nrows = nrows;
  scene_data[0].ncols = ncols;
  scene_data[0].theta_v = 0.0; /* subsurface view and sun zenith (deg) */
  scene_data[0].theta_w = 35.0;
  for (int b = 0; b < nb; b++) {
    scene_data[0].band_indexes[b] = b;
    scene_data[0].wavelengths[b] = wl[b];
    gridded_data[b].nrows = nrows;
    gridded_data[b].ncols = ncols;
    gridded_data[b].nodata_value = -9999.0f;
    gridded_data[b].array = grid(nrows, ncols, rrs[b]);
  }
  float **out[10];
  for (int k = 0; k < 10; k++) out[k] = grid(nrows, ncols, 0.0f);
  geogrid none;
  memset(&none, 0, sizeof none);
  samodel(scene_data, gridded_data, ps_in, 1, false, none, 1, 1, 1, out[0], out[1], out[2],
          out[3], out[4], out[5], out[6], out[7], out[8], out[9], 10.0f, 0, 1);
  printf("depth %g\n", (double)out[0][1][1]);
  return 0;
}
