/*
 * photic_oracle.h -- CPU restatement of photic's per-pixel inversion.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the tests, the smoke
 * check and bench.py's CPU baseline compare the GPU path against.  Nothing
 * in the product (photic_gb300/) includes, links or loads it.
 *
 * It restates, in plain C99 with double precision and the same order of
 * floating-point operations, the reference's
 *   samodel_Rrs        model/samodel.c:2846-2949   (HOPE forward model)
 *   samodel_error      model/samodel.c:2432-2759   (cost)
 *   nelmin             model/asa047.c:10-502       (modified AS 47)
 *   samodel_optimise   model/samodel.c:1768-2115   (per-pixel driver) with
 *   samodel_optimise_one_bottom_combination  model/samodel.c:2119-2427
 *   extract_Rrs_data   model/samodel.c:2957-3027   (3 x 3 regions)
 *   samodel()'s pixel loop with its lookup table, model/samodel.c:649-1352
 *   the depth uncertainty, model/samodel.c:1368-1479
 *   interp_1d          model/common.c:298-335
 *   the netCDF packing, model/nc.c:14-320
 * for one pixel or a 3 x 3 neighbourhood, one to three bottom types and
 * stacks of scenes.  It is pinned bit for bit against the reference
 * compiled from its own sources (oracle/_ref, built by oracle/Makefile) and
 * against the committed fixtures in tests/golden/.
 */
#ifndef PHOTIC_ORACLE_H
#define PHOTIC_ORACLE_H

#include <stdint.h>

#define PO_MAX_BANDS 8
#define PO_MAX_SCENES 8
#define PO_MAX_PARAMS 96
#define PO_N_BOTTOM_TYPES 8
#define PO_NOUT 44

/* Output record per pixel (doubles), shared with oracle/_ref and the GPU:
 *  0 depth H   1 bottom albedo   2 model error (cost)   3 Rrs error (%)
 *  4 K_min     5 index of optical depth   6 evaluations of the kept start
 *  7 evaluations over all starts          8 converged (ifault == 0)
 *  9 status (0 fitted, 1 masked, 2 invalid)   10 scene count
 * 11..18 P per scene   19..26 G per scene   27..34 X per scene
 * 35 restarts of the kept start   36 index of the kept start   37 ifault
 * 38 regions  39 origin region (region fits)
 * 40..42 bottom shares (%) of sand, seagrass, coral in the origin region
 * 43 bottom type (1 + index of the largest share; region fits) */

#ifdef __cplusplus
extern "C" {
#endif

int po_nout(void);
double po_interp_1d(const double *X, const double *Y, int n, double x);
void po_band_constants(int n_bands, const double *wl, double theta_sun_deg,
                       double theta_view_deg, double *out);
double po_cost(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
               double h_tide, const double *rrs_measured, const double *params,
               double *rrs_modelled, double *K_out);
void po_nelmin_fn(double (*fn)(const double *x, void *ctx), void *ctx, int n,
                  const double *start_in, const double *step, double reqmin, int konvge,
                  int kcount, double *xmin, double *ynewlo, int *icount, int *numres,
                  int *ifault);
void po_nelmin_pixel(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                     const double *rrs_measured, const double *start, const double *step,
                     double reqmin, int konvge, int kcount, double *xmin, double *ynewlo,
                     int *icount, int *numres, int *ifault);
int po_invert_batch(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                    double h_tide, const float *rrs, int64_t npix, float nodata, double reqmin,
                    int konvge, int kcount, int n_hstarts, const double *hstarts,
                    const double *seeds, double seed_step_scale, int nthreads, double *out);
int po_joint_invert_batch(int n_bands, const double *wl, double theta_view_deg, double h_tide,
                          const int32_t *scene_offsets, const double *theta_sun_deg,
                          const float *rrs, int64_t npix, float nodata, int layout,
                          double reqmin, int konvge, int kcount, int n_hstarts,
                          const double *hstarts, int nthreads, double *out);
void po_generate_single(uint64_t seed, int64_t pix0, int64_t npix, int n_bands, const double *wl,
                        double theta_sun_deg, double theta_view_deg, double mask_frac,
                        double noise_sigma, float nodata, float *rrs_out, double *truth_out);
void po_joint_counts(uint64_t seed, int64_t npix, int kmin, int kmax, int32_t *counts);
void po_generate_joint(uint64_t seed, int64_t npix, int n_bands, const double *wl,
                       double theta_view_deg, double theta_sun_min, double theta_sun_max,
                       double mask_frac, double noise_sigma, float nodata,
                       const int32_t *scene_offsets, double *theta_sun_out, float *rrs_out,
                       double *truth_out);
void po_philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                   uint32_t *out4);
int po_region_invert_batch(int n_bands, const double *wl, double theta_sun_deg,
                           double theta_view_deg, double h_tide, const float *grid, int nrows,
                           int ncols, float nodata, double reqmin, int konvge, int kcount,
                           int nthreads, double *out);
int po_region_fit_batch(int n_bands, const double *wl, const double *theta_sun_deg,
                        double theta_view_deg, double h_tide, const float *grid, int n_scenes,
                        int nrows, int ncols, float nodata, int n_spatial, int n_bottoms,
                        const double *h_empirical, double reqmin, int konvge, int kcount,
                        int nthreads, double *out);
double po_region_cost(int n_bands, const double *wl, const double *theta_sun_deg,
                      double theta_view_deg, double h_tide, const double *rrs, int R, int S,
                      int origin, int n_bottoms, const double *params, double *details,
                      double *rm);
int po_depth_sigma(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                   const float *rrs, int64_t npix, const float *depth, const double *r_sigma,
                   int n_samples, uint64_t seed, double reqmin, int konvge, int kcount,
                   int nthreads, const double *sample_depth_in, int32_t *sample_pixel,
                   double *sample_depth, double *table, float *depth_sigma);

/* netCDF short packing (model/nc.c:251-320): see photic_oracle.c. */
void po_nc_decompress(const int16_t *packed, int64_t n, float add_offset, float scale_factor,
                      int16_t missing_value, double spval, float *grid);
/* Spatially coherent synthetic scene (smooth parameter fields) and the
 * pixel loop with the dynamic lookup table (model/samodel.c:649-1215). */
void po_field_truth(uint64_t seed, int64_t nrows, int64_t ncols, int64_t i, int64_t j,
                    double *t5);
void po_generate_field(uint64_t seed, int64_t nrows, int64_t ncols, int64_t row0, int64_t n_rows,
                       int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                       double mask_frac, double noise_sigma, float nodata, float *rrs_out,
                       double *truth_out);
float po_lut_key(const float *r, int n_bands, float nodata, const double *noise);
int po_region_depth_sigma(int n_bands, const double *wl, const double *theta_sun_deg,
                          double theta_view_deg, const float *grid, int n_scenes, int nrows,
                          int ncols, float nodata, int n_spatial, int n_bottoms,
                          const float *depth, const double *r_sigma, int n_samples,
                          uint64_t seed, double reqmin, int konvge, int kcount, int nthreads,
                          const double *sample_depth_in, int32_t *sample_pixel,
                          double *sample_depth, double *table, float *depth_sigma);
float po_glut_key(const float *grid, int n_scenes, int64_t npix, int64_t p, int n_bands,
                  float nodata, const double *noise);
int po_glut_invert(int n_bands, const double *wl, const double *theta_sun_deg,
                   double theta_view_deg, double h_tide, const float *grid, int n_scenes,
                   int nrows, int ncols, float nodata, int n_spatial, int n_bottoms,
                   const double *rrs_noise, const float *emp, float emp_nodata, double reqmin,
                   int konvge, int kcount, int n_lut, int64_t n_chains, int nthreads,
                   int64_t *order_out, int64_t *n_shallow_out, double *out, int64_t *source,
                   double *chain_stats);
int po_lut_invert(int n_bands, const double *wl, double theta_sun_deg, double theta_view_deg,
                  double h_tide, const float *rrs, int64_t npix, float nodata,
                  const double *rrs_noise, const float *emp, float emp_nodata, double reqmin,
                  int konvge, int kcount, int n_lut, int64_t n_chains, int nthreads,
                  int64_t *order_out, int64_t *n_shallow_out, double *out, int64_t *source,
                  double *chain_stats);
void po_nc_compress(const float *grid, int64_t n, double spval, int16_t *packed,
                    float *add_offset, float *scale_factor, int16_t *missing_value);

#ifdef __cplusplus
}
#endif
#endif
