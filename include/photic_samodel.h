/*
 * photic_samodel.h -- link-compatible drop-ins for photic's samodel entry
 * points, backed by the GB300 kernels of libphotic_gb300.
 *
 * The reference declares these in model/samodel.h:8-29 over the types of
 * model/common.h (geogrid :69-84, model_data :116-190, scene :194-216).  For
 * a program built against the reference headers to relink against this
 * library unchanged, the structs below repeat those layouts field for field
 * (same order, same types; the reference's bool is an int, MAX_STRING_LEN
 * 2048, MAX_GRIDS 265).  They carry photic_ names so this header never
 * clashes with the reference's own.
 *
 * Semantics kept: the per-pixel fit of samodel_optimise (cold multi-start,
 * the single empirical depth start when empirical_depth_present, or the hot
 * start from md->prev), the cost of samodel_error and the forward model of
 * samodel_Rrs, with one to three bottom types (sand, seagrass, coral) mixed
 * per region and one or a 3 x 3 neighbourhood of regions; samodel()'s pixel
 * loop, with its dynamic lookup table of earlier fits and hot starts
 * (model/samodel.c:649-1215) where the lookup-table kernel covers the
 * configuration (see samodel() below); outputs are written where the
 * reference writes them, and samodel() ends with the reference's netCDF
 * result files.  The functions return void like the reference; each clears
 * photic_last_error() on entry, and a failure leaves the outputs untouched
 * and its message there, so an empty message after the call means
 * success.
 *
 * Rrs_measured is read at float precision (samodel() fills it from float
 * grids).  samodel_optimise honours start_at_previous for one scene (one
 * start at depth_prev, or h_empirical, with P, G, X from md->prev); a joint
 * fit over n_scenes > 1 uses the cold multi-start and band constants from
 * the wavelengths' tables, with each scene's theta_sun from md.
 */
#ifndef PHOTIC_SAMODEL_H
#define PHOTIC_SAMODEL_H

#include "photic.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PHOTIC_REF_MAX_STRING_LEN 2048
#define PHOTIC_REF_MAX_GRIDS 265

typedef struct photic_geogrid {
  int nrows;
  int ncols;
  float cellsize;
  float wlon;
  float slat;
  float elon;
  float nlat;
  float nodata_value;
  float lambda;
  float theta_v;
  float theta_w;
  float **array;
} photic_geogrid;

typedef struct photic_model_data {
  int n_bottoms;
  int n_scenes;
  int n_regions;
  int max_n_bands;
  int max_n_regions;
  int *n_bands;
  int *n_raw_bands;
  int origin;
  int n_params;
  double ***Rrs_measured;
  double **wavelengths;
  double **raw_wavelengths;
  double ***bottom_reflectance;
  double **a_0;
  double **a_1;
  double **a_w;
  double **b_bw;
  double a_w640;
  double *H_tide;
  double *theta_sun;
  double *theta_view;
  double *sec_theta_sun;
  double *sec_theta_view;
  double **Rrs440;
  double **Rrs490;
  double **Rrs550;
  double **Rrs640;
  double **Rrs750;
  double **rrs_noise;
  double h_empirical;
  int bottom_type_indexes[12];
  char B_type_name[12][PHOTIC_REF_MAX_STRING_LEN];
  int empirical_depth_present;
  int i;
  int j;
  int prev_i;
  int prev_j;
  int start_at_previous;
  double *P;
  double *G;
  double *X;
  double *B;
  double *H;
  double *D;
  double *prev;
  double ***Rrs_modelled;
  double ***rrs_modelled;
  double ***rrs_bottom;
  double ***rrs_dp;
  double **K;
  double ***rho;
  double depth;
  double depth_prev;
  double depth_sigma;
  double Rrs_error;
  double SAM_error;
  double K_error;
  double depth_error;
  double bottom_error;
  double model_error;
  double K_min;
  double K_min_prev;
  double bottom_albedo;
  double B_type_percent[12];
  double index_optical_depth;
  int bottom_type;
  int converged;
  int n_iterations;
} photic_model_data;

typedef struct photic_scene {
  char scene_name[PHOTIC_REF_MAX_STRING_LEN];
  int n_bands;
  int nrows;
  int ncols;
  int band_indexes[PHOTIC_REF_MAX_GRIDS];
  int wavelengths[PHOTIC_REF_MAX_GRIDS];
  double theta_w;
  double theta_v;
  double H_tide;
  double R_inf[PHOTIC_REF_MAX_GRIDS];
  double R_sigma[PHOTIC_REF_MAX_GRIDS];
  double K[PHOTIC_REF_MAX_GRIDS];
  double K_sigma[PHOTIC_REF_MAX_GRIDS];
  double ratio_min;
  double ratio_max;
  double slope_min;
  double slope_max;
  int pgx_present;
  int ps_p;
  int ps_g;
  int ps_x;
} photic_scene;

/* The reference's SCENE command (model/bam.c:1300-1543), parsed from its
 * text into the scene record run_scene fills: name, band count, band
 * wavelengths (stored as int, as the record holds them), THETAVIEW and
 * THETASUN (subsurface, degrees), and the optional RINF, HTIDE, K, RSIGMA,
 * KSIGMA (an absent KSIGMA is K / 10) and P / G / X grid names.  The band
 * grid names are returned in band_names; band_indexes are 0..n_bands-1 and
 * a caller maps them onto its own grids.  Where the reference fills an
 * absent RINF, K or RSIGMA from deep-water estimates of other commands, the
 * record keeps zeros and `given` lacks that bit.  Host function;
 * PHOTIC_ERR_INVALID with the reference's usage text on a malformed line. */
#define PHOTIC_SCENE_MAX_BANDS 64
#define PHOTIC_SCENE_NAME_LEN 256
enum {
  PHOTIC_SCENE_RINF = 1,
  PHOTIC_SCENE_HTIDE = 2,
  PHOTIC_SCENE_K = 4,
  PHOTIC_SCENE_RSIGMA = 8,
  PHOTIC_SCENE_KSIGMA = 16
};
typedef struct photic_scene_spec {
  photic_scene scene;
  char band_names[PHOTIC_SCENE_MAX_BANDS][PHOTIC_SCENE_NAME_LEN];
  char pgx_names[3][PHOTIC_SCENE_NAME_LEN];
  int32_t given; /* PHOTIC_SCENE_* of the optional items present */
} photic_scene_spec;
int photic_parse_scene(const char *line, photic_scene_spec *out);

/* The inversion's configuration for a scene record: its bands and
 * wavelengths, THETASUN / THETAVIEW as the subsurface angles samodel() uses
 * (model/samodel.c:534-548) and HTIDE; everything else the defaults. */
int photic_config_from_scene(const photic_scene *scene, photic_config *cfg);

/* model/samodel.h:8-19.  Fits every pixel that has data in all bands of all
 * scenes (model/samodel.c:672-700), at the reference's tolerances
 * (reqmin 1e-2, konvge 100, kcount 5000), smoothing radius 1 (none) only,
 * through the reference's pixel loop with its dynamic lookup table: pixels
 * in spectral-index order (blue, green and red summed over the scenes; times
 * the spectral angle to the scenes' R_sigma when every band's is at least
 * 1e-6), or in the order of the empirical depths when given, served from
 * stored fits or fitted with hot starts (from the empirical depth where a
 * pixel has one); the order is cut into PHOTIC_LUT_CHAINS contiguous chains
 * (environment; 1 is the reference on one thread), else eight per lane or
 * warp the kernel keeps resident.  The fit is
 *   - one scene, n_bottoms == 1, n_spatial <= 1: the single-pixel fit
 *     (photic_lut_invert_batch, a lane per chain);
 *   - otherwise (n_bottoms 2..3, n_spatial == 2, stacks of scenes): the
 *     general fit of photic_region_fit_batch -- bottom mixtures, 3 x 3
 *     regions, each scene's P, G, X (photic_region_lut_invert_batch, a warp
 *     per chain).
 * depth_sigma is the reference's Monte Carlo estimate, computed by
 * photic_depth_sigma or photic_region_depth_sigma with the scenes' R_sigma,
 * 128 samples per 0.25 m interval and a fixed seed.  Depth is
 * written negative below the datum, as the reference does
 * (model/samodel.c:1486).  Like the reference, it ends by writing the result
 * grids as netCDF files in the working directory (model/samodel.c:1492-1690):
 * <scene>_K_coastal/_K_blue/_K_green/_K_red/_P/_G/_X.nc per scene and the ten
 * modelled_*.nc grids, packed as write_nc packs them (photic_nc.h). */
void samodel(photic_scene scene_data[], photic_geogrid gridded_data[], int *scene_indexes,
             int nscenes, int empirical_depth_present, photic_geogrid empirical_depths,
             int n_smoothing_radius, int n_spatial, int n_bottoms, float **depth,
             float **depth_sigma, float **model_error, float **bottom_albedo, float **bottom_sand,
             float **bottom_seagrass, float **bottom_coral, float **K_min, float **bottom_type,
             float **index_optical_depth, float pagesize, int background, int linewidth);

/* model/samodel.h:21.  Reads the measured spectra and band constants of md
 * (one region) and writes depth, P, G, X, bottom albedo, the errors, K_min,
 * index of optical depth, n_iterations, converged and Rrs_modelled. */
void samodel_optimise(photic_model_data *md);

/* model/samodel.h:23.  The fit of md's one scene, region and bottom type
 * (cold multi-start, empirical depth or start_at_previous, as
 * samodel_optimise): writes |best| into params[0..5] (H, 100 B, q, 100 P,
 * 100 G, 100 X), md->n_iterations, converged and what the final cost leaves
 * (Rrs_modelled, Rrs_error, model_error, bottom_albedo, depth). */
void samodel_optimise_one_bottom_combination(photic_model_data *md, double *params);

/* model/samodel.h:25.  Cost of params for md's first region; also writes
 * md->Rrs_modelled[0][s][b], Rrs_error and model_error. */
double samodel_error(double *params, photic_model_data *md);

/* model/samodel.h:27-29.  Forward model of one band at the given water
 * column, depth and bottom (q normalised, one bottom type); writes, as the
 * reference does, md->Rrs_modelled, rrs_modelled, rrs_bottom, rrs_dp and rho
 * at [k_region][k_scene][k_band] (each when allocated), md->K[k_scene][k_band],
 * md->depth and md->bottom_albedo. */
void samodel_Rrs(double P, double G, double X, double B[], double q[], double H, double Delta,
                 photic_model_data *md, int k_scene, int k_band, int k_region);

/* Forward model batch (samodel_Rrs over all bands of cfg): for n parameter
 * rows of 7 doubles -- P, G, X, B, q, H, Delta -- and the spectrum-shape
 * inputs Rrs(440) and Rrs(490) per row, writes Rrs [n * n_bands] and
 * K [n * n_bands] (doubles; K may be NULL).  Device pointers. */
int photic_forward_batch(const photic_config *cfg, const double *d_params,
                         const double *d_rrs440, const double *d_rrs490, int64_t n,
                         double *d_rrs, double *d_K, void *stream);

#ifdef __cplusplus
}
#endif
#endif
